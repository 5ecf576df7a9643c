// Host-buffer entry point for the whole filter stage: random starts in host
// memory in, eigenvalues / sigma_E / eigenvectors in host memory out.  This is
// the call a drop-in Filter executable makes after the setup: it covers
// run_filter_cycles + mod_ortho + mod_diag + mod_sigma + the state selection
// of mod_output (filter_mpi/filter.c:5-183, mod_ortho.c:3-94,
// mod_diag.c:324-449, mod_sigma.c:6-63, mod_output.c:5-162).
#include <cmath>
#include <cstdint>
#include <vector>

#include "fbse_internal.cuh"

namespace fbse {
int newton_filter(fbse_ctx *c, const double *zn, const double *an, long ncheby, long m, double vmin, double de,
                  const double *psi0, long nstart, double *filtered);
int ortho_diag_sigma(fbse_ctx *c, double *psitot, long n, long *n_kept, double *eval, double *sigma);
}  // namespace fbse

using namespace fbse;

// selected states straight into mapped pinned host memory: dst[w] = src[sel[w]],
// 16-byte stores (stlen is even)
__global__ void k_gather_states(const double2 *__restrict__ src, const int *__restrict__ sel, long nsel, long n2,
                                double2 *__restrict__ dst)
{
  const long total = nsel * n2;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long w = e / n2, k = e - w * n2;
    dst[e] = src[(long)sel[w] * n2 + k];
  }
}

extern "C" int fbse_filter_job(fbse_ctx *c, const double *zn, const double *an, long ncheby, long m, double vmin,
                               double de, const double *psi0_host, long nstart, double sigma_cut, long *n_out,
                               double *eval_host, double *sigma_host, double *psi_host)
{
  if (!c || !zn || !an || !psi0_host || nstart < 1 || m < 1 || !n_out || !eval_host || !sigma_host)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_filter_job: bad arguments") : FBSE_ERR_ARG;
  const long stlen = (long)(c->is_complex + 1) * c->nspin * c->ngrid;
  const long n = nstart * m;
  double *d0 = nullptr, *df = nullptr;
  int rc = FBSE_OK;
  {
    void *a = nullptr, *b = nullptr;
    if (cached(c, kSlotJobStarts, (size_t)nstart * stlen * sizeof(double), &a) ||
        cached(c, kSlotJobStates, (size_t)n * stlen * sizeof(double), &b))
      return set_err(c, FBSE_ERR_OOM, "fbse_filter_job: state buffers");
    d0 = (double *)a;
    df = (double *)b;
  }
  std::vector<double> ev(n), sg(n);
  long nk = 0;
  do {
    if (cudaMemcpyAsync(d0, psi0_host, (size_t)nstart * stlen * sizeof(double), cudaMemcpyHostToDevice, c->stream) !=
        cudaSuccess) { rc = set_err(c, FBSE_ERR_CUDA, "fbse_filter_job: upload"); break; }
    if ((rc = newton_filter(c, zn, an, ncheby, m, vmin, de, d0, nstart, df))) break;
    if ((rc = ortho_diag_sigma(c, df, n, &nk, ev.data(), sg.data()))) break;
    // mod_output: all states (sigma_cut <= 0, getAllStates = 1) or those with sigma <= cut
    std::vector<int> sel;
    for (long i = 0; i < nk; i++) {
      if (sigma_cut > 0 && !(sg[i] <= sigma_cut)) continue;
      eval_host[sel.size()] = ev[i];
      sigma_host[sel.size()] = sg[i];
      sel.push_back((int)i);
    }
    const long w = (long)sel.size();
    *n_out = w;
    if (psi_host && w > 0) {
      // pinned host memory the device can address: one gather kernel writes the
      // states into it (C2C stores); anything else: one copy per state
      void *hdev = nullptr;
      const bool mapped = (reinterpret_cast<uintptr_t>(psi_host) % 16 == 0) && stlen % 2 == 0 &&
                          cudaHostGetDevicePointer(&hdev, psi_host, 0) == cudaSuccess && hdev;
      if (!mapped) cudaGetLastError();
      int *dsel = nullptr;
      if (mapped && cudaMalloc(&dsel, w * sizeof(int)) == cudaSuccess &&
          cudaMemcpyAsync(dsel, sel.data(), w * sizeof(int), cudaMemcpyHostToDevice, c->stream) == cudaSuccess) {
        k_gather_states<<<4096, 256, 0, c->stream>>>(reinterpret_cast<const double2 *>(df), dsel, w, stlen / 2,
                                                     reinterpret_cast<double2 *>(hdev));
        FBSE_COUNT(1);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
          rc = set_err(c, FBSE_ERR_CUDA, "fbse_filter_job: download");
        cudaFree(dsel);
      } else {
        cudaGetLastError();
        if (dsel) cudaFree(dsel);
        for (long q = 0; q < w && !rc; q++)
          if (cudaMemcpyAsync(psi_host + q * stlen, df + (long)sel[q] * stlen, stlen * sizeof(double),
                              cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
            rc = set_err(c, FBSE_ERR_CUDA, "fbse_filter_job: download");
      }
      if (rc) break;
    }
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "fbse_filter_job");
  } while (0);
  cudaStreamSynchronize(c->stream);
  return rc;
}
