// Host side of H psi with the projectors fused into the plane passes
// (hpsi_fused.cuh): eligibility, scratch and the four launches on the
// context's stream.
#include "fft_common.cuh"
#include "fft_fast.cuh"
#include "hpsi_fused.cuh"

namespace fbse {

bool hpsi_fused_ok(fbse_ctx *c)
{
  if (c->tune.hpsi_fused != 1 || c->tune.fft_kernels != 0 || c->tune.fft_plane_cluster != 0) return false;
  if (c->nx != fused::N || c->ny != fused::N) return false;
  return (c->so || c->nl) && c->proj.nat > 0 && c->proj.fz_ok;
}

template <int CH>
static int launch_fused(fbse_ctx *c, const fused::FusedArgs &A, long nstates)
{
  constexpr size_t sf = fused::plane_proj_smem<CH>(false), si = fused::plane_proj_smem<CH>(true);
  const unsigned planes = (unsigned)(A.nblk * c->nz);
  FBSE_CUDA(c, cudaFuncSetAttribute(fused::k_plane_proj_fwd<CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sf));
  FBSE_CUDA(c, cudaFuncSetAttribute(fused::k_plane_proj_inv<CH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)si));
  fused::k_plane_proj_fwd<CH><<<planes, fused::THREADS, sf, c->stream>>>(A);
  FBSE_CHECK_LAUNCH(c);
  fused::k_proj_red<CH><<<dim3((unsigned)((c->proj.nat + 31) / 32), (unsigned)nstates), fused::THREADS, 0, c->stream>>>(A);
  FBSE_CHECK_LAUNCH(c);
  int rc = zpass_kinetic(c, A.wk, A.nblk);
  if (rc) return rc;
  fused::k_plane_proj_inv<CH><<<planes, fused::THREADS, si, c->stream>>>(A);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

int hpsi_fused_apply(fbse_ctx *c, const float2 *in, float2 *out, long nstates, double a, double b)
{
  const ProjDev &p = c->proj;
  const long nblk = nstates * c->nspin;
  const int ch = (c->so ? 1 : 0) | (c->nl ? 2 : 0);
  const int nch = (ch & 1) + ((ch >> 1) & 1);
  if (nblk * c->nz > 2147483647L || nstates > 65535)
    return set_err(c, FBSE_ERR_UNSUPPORTED, "fused H psi: batch too large");
  int rc;
  // scratch: the FFT blocks, the coefficients, the segment partials
  if ((rc = ensure(c, &c->wk, &c->wk_bytes, (size_t)nblk * c->ngrid * sizeof(float2)))) return rc;
  if ((rc = ensure(c, &c->coef, &c->coef_bytes, (size_t)nstates * p.nat * 2 * 30 * sizeof(float2)))) return rc;
  void *part = nullptr;
  if ((rc = cached(c, kSlotProj, (size_t)nblk * p.fz_nseg * 30 * nch * sizeof(float), &part))) return rc;
  fused::FusedArgs A{};
  A.in = in;
  A.out = out;
  A.wk = reinterpret_cast<float2 *>(c->wk);
  A.coef = reinterpret_cast<float2 *>(c->coef);
  A.part = reinterpret_cast<float *>(part);
  A.pot = c->pot32;
  A.rx = c->ax[0].tw32;
  A.tb = fused::ProjTable{p.fz_ent, p.fz_y, p.fz_so, p.fz_nl, p.fz_lay, p.fz_atoms, p.fz_natoms, p.fz_seg_beg,
                          p.fz_plane_seg, p.fz_aseg_beg, p.fz_aseg, p.LS, p.sgn, p.fz_nent, p.fz_nseg, p.nat, p.nproj};
  A.ngrid = c->ngrid;
  A.nblk = (int)nblk;
  A.nspin = c->nspin;
  A.ca = (float)a;
  A.cb = (float)b;
  A.dv = (float)c->dv;
  switch (ch) {
    case 1: return launch_fused<1>(c, A, nstates);
    case 2: return launch_fused<2>(c, A, nstates);
    default: return launch_fused<3>(c, A, nstates);
  }
}

}  // namespace fbse
