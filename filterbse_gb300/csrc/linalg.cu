// Orthogonalisation, subspace diagonalisation and sigma_E.
#include "fbse_internal.cuh"

namespace fbse {

int ortho_diag_sigma(fbse_ctx *c, double *psitot, long n, long *n_kept, double *eval, double *sigma)
{
  (void)psitot; (void)n; (void)n_kept; (void)eval; (void)sigma;
  return set_err(c, FBSE_ERR_UNSUPPORTED, "ortho/diag/sigma not built yet");
}

}  // namespace fbse
