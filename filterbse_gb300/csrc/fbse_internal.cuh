// Internal declarations shared by the CUDA translation units of libfbse_gpu.
//
// Layout in HBM (all device buffers are owned by an fbse_ctx):
//   * a "state" is nspin blocks of ngrid complex values (spin-up block first),
//     grid index jxyz = nx*(ny*jz + jy) + jx, interleaved (re, im) -- the same
//     layout as the reference's zomplex arrays (filter_mpi/fd.h:333-337);
//   * working states are complex in the context's precision (float2 for the
//     mixed path, double2 for the plain FP64 path); real-valued jobs pack two
//     real states into one complex state (re = state 2i, im = state 2i+1),
//     which is exact because every operator on the filter path is real for
//     real jobs (kinetic, local potential and the l = 1 nonlocal projector);
//   * filtered-state accumulators and everything handed back to the caller
//     use the reference's psi_rank / psitot layout in FP64: stlen doubles per
//     state, 1 double per point for real jobs, (re, im) pairs otherwise.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/fbse.h"

namespace fbse {

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
template <typename T> struct cplx_t;
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<double> { using type = double2; };
template <typename T> using C = typename cplx_t<T>::type;

template <typename T> __host__ __device__ __forceinline__ C<T> mk(T re, T im) { C<T> r; r.x = re; r.y = im; return r; }
template <typename T> __host__ __device__ __forceinline__ C<T> cadd(C<T> a, C<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __host__ __device__ __forceinline__ C<T> csub(C<T> a, C<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __host__ __device__ __forceinline__ C<T> cmul(C<T> a, C<T> b)
{
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b) when conjb, else a * b
template <typename T> __host__ __device__ __forceinline__ C<T> cmulc(C<T> a, C<T> b, bool conjb)
{
  T by = conjb ? -b.y : b.y;
  return mk<T>(a.x * b.x - a.y * by, a.x * by + a.y * b.x);
}
template <typename T> __host__ __device__ __forceinline__ C<T> cscale(C<T> a, T s) { return mk<T>(a.x * s, a.y * s); }

// ---------------------------------------------------------------------------
// FFT plan for one axis: mixed-radix Stockham stages + root table
// ---------------------------------------------------------------------------
constexpr int kMaxStages = 16;
struct AxisPlan {
  int n = 0;
  int nst = 0;
  int radix[kMaxStages] = {0};
  double2 *tw64 = nullptr;  // device, n roots e^{-2 pi i t / n}
  float2 *tw32 = nullptr;   // device, same roots rounded to FP32
};

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct ProjDev {
  long nat = 0, npts = 0;
  int nproj = 0;
  int so = 0, nl = 0;
  int *nl_cnt = nullptr;      // [nat]
  int *jxyz = nullptr;        // [nat*npts]
  double *y1 = nullptr;       // [3][nat*npts] complex Y_1m (structure of arrays)
  double *sop = nullptr;      // [nproj][nat*npts]
  double *nlp = nullptr;      // [nproj][nat*npts]
  int *sgn = nullptr;         // [nat*nproj]
  double2 *LS = nullptr;      // [36]
  float *y1f = nullptr, *sopf = nullptr, *nlpf = nullptr;  // FP32 copies for the mixed path
  // point-major copy of the table for the scatter: the ncov grid points that
  // lie in at least one sphere in increasing grid index (cov_j), each with its
  // entries cov_beg[k] .. cov_beg[k+1]-1 in increasing atom order; per entry
  // the atom (pe_atom), Y_1m and the radial values in the same structure-of-
  // arrays form as above.  One thread owns each covered point, so the scatter
  // adds in a fixed order and needs no atomics.
  long ncov = 0, nent = 0;
  int *cov_j = nullptr, *cov_beg = nullptr, *pe_atom = nullptr;
  // the covered points in chunks (consecutive points, at most
  // kScatterChunkPoints of them and kScatterChunkAtoms distinct atoms): chunk
  // c holds points chunk_beg[c] .. chunk_beg[c+1]-1, its atoms
  // chunk_atoms[c * kScatterChunkAtoms + s] (-1 unused), and pe_slot[e] is the
  // slot of entry e's atom in its chunk
  long nchunk = 0;
  int *chunk_beg = nullptr, *chunk_atoms = nullptr;
  unsigned char *pe_slot = nullptr;
  double *pe_y1 = nullptr, *pe_sop = nullptr, *pe_nlp = nullptr;
  float *pe_y1f = nullptr, *pe_sopf = nullptr, *pe_nlpf = nullptr;
  // plane-major copy for the projector-fused plane passes (hpsi_fused.cuh;
  // FP32 contexts on 128 x 128 x nz grids whose Y_1m have the form (y0, y1),
  // (y2, 0), (-y0, y1)): fz_ok when built
  int fz_ok = 0;
  long fz_nent = 0, fz_nseg = 0;
  unsigned *fz_ent = nullptr;
  float *fz_y = nullptr, *fz_so = nullptr, *fz_nl = nullptr;
  int *fz_lay = nullptr, *fz_atoms = nullptr, *fz_natoms = nullptr, *fz_seg_beg = nullptr, *fz_plane_seg = nullptr;
  int *fz_aseg_beg = nullptr, *fz_aseg = nullptr;
};

constexpr int kScatterChunkPoints = 128, kScatterChunkAtoms = 32;
// projector-fused plane passes (hpsi_fused.cuh): plane edge, atoms whose
// spheres meet one plane, entries of one grid point, table entries per gather
// segment
constexpr int kPipeN = 128, kPipePlaneAtoms = 192, kPipeMaxLayers = 8, kPipeSegMax = 128;

// one decision of the autotuner: candidate values with their times (us)
struct TuneRecord {
  std::string kernel, problem;
  std::vector<std::pair<long, double>> cand;
  long choice = 0;
};

}  // namespace fbse

struct fbse_ctx {
  int precision = FBSE_FP64;
  long nx = 0, ny = 0, nz = 0, ngrid = 0;
  int nspin = 1, is_complex = 0, so = 0, nl = 0;
  double dx = 0, dy = 0, dz = 0, dv = 0, ke_max = 0;
  double kemax_scaled = 0;                 // KE_max / N (init.c:338)
  double dk[3] = {0, 0, 0};                // reciprocal spacings dkx, dky, dkz (init.c:65-80)
  fbse::AxisPlan ax[3];                    // x, y, z
  double *k2x = nullptr, *k2y = nullptr, *k2z = nullptr;  // per-axis 0.5 k^2 / N (device)
  float *k2xf = nullptr, *k2yf = nullptr, *k2zf = nullptr;  // the same rounded to FP32 (mixed path)
  double *pot64 = nullptr;                 // [ngrid]
  float *pot32 = nullptr;
  double vpot_min = 0, vpot_max = 0;
  fbse::ProjDev proj;
  cudaStream_t stream = nullptr;
  static constexpr int kSide = 3;
  cudaStream_t side[kSide] = {};           // further streams: parts of an H psi batch beside the first
  cudaEvent_t ev_fork = nullptr, ev_join[kSide] = {};
  // scratch (grown on demand)
  void *wk = nullptr; size_t wk_bytes = 0;       // FFT work states
  void *coef = nullptr; size_t coef_bytes = 0;   // projector coefficients
  void *tmp = nullptr; size_t tmp_bytes = 0;     // general
  double *red = nullptr; size_t red_bytes = 0;   // reduction partials
  int *dstatus = nullptr;                        // device error flags of kernels with bounded waits
  int tc_poisoned = 0;  // a tensor-core wait timed out: MMAs may still be in flight, the path is refused
  int nsm = 0;          // multiprocessors of the device (queried on first use)
  // large buffers kept between calls (grown on demand, freed by fbse_destroy):
  // the Newton ring, the Rayleigh-Ritz H psi and rotated states, the
  // filter job's device copies of the starts and filtered states
  void *cache[8] = {};
  size_t cache_bytes[8] = {};
  fbse_tuning tune{};                      // fixed choices (nonzero fields) of the caller
  std::vector<fbse::TuneRecord> tuned;     // the autotuner's decisions
  std::string err;
};

namespace fbse {

// error plumbing ------------------------------------------------------------
int set_err(fbse_ctx *c, int code, const std::string &msg);
#define FBSE_CUDA(ctx, call)                                                                  \
  do {                                                                                        \
    cudaError_t e__ = (call);                                                                 \
    if (e__ != cudaSuccess)                                                                   \
      return ::fbse::set_err((ctx), FBSE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e__)); \
  } while (0)
// every kernel launch of the library is counted (fbse_launch_count)
extern std::atomic<long> g_launches;
#define FBSE_COUNT(k) (::fbse::g_launches += (k))
#define FBSE_CHECK_LAUNCH(ctx)              \
  do {                                      \
    FBSE_COUNT(1);                          \
    FBSE_CUDA(ctx, cudaGetLastError());     \
  } while (0)
// the same inside a do { } while (0) block whose exit frees the caller's
// scratch: records the error in rc and leaves the block with break
#define FBSE_LAUNCH_OR_BREAK(ctx, rc)                                                                      \
  if (FBSE_COUNT(1), (rc = ::fbse::launch_status(ctx)) != FBSE_OK) break

int ensure(fbse_ctx *c, void **p, size_t *have, size_t need);
// FBSE_OK, or the last launch's error recorded in the context
inline int launch_status(fbse_ctx *c)
{
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? FBSE_OK : set_err(c, FBSE_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
}
enum CacheSlot { kSlotRing = 0, kSlotHpsi, kSlotRot, kSlotJobStarts, kSlotJobStates, kSlotJacobi, kSlotTc, kSlotProj };
inline int cached(fbse_ctx *c, int slot, size_t need, void **out)
{
  const int rc = ensure(c, &c->cache[slot], &c->cache_bytes[slot], need);
  *out = c->cache[slot];
  return rc;
}
// reads (and clears) the device error flags of the kernels with bounded waits
int check_dev_status(fbse_ctx *c);

// autotuner: the recorded choice for (kernel, problem), or -- on the first
// call -- times launch(v) for each candidate v on the context's stream (one
// untimed and two timed runs each, CUDA events) and records the fastest.
// launch(v) must enqueue work whose result does not depend on v, or write
// only scratch.  Returns FBSE_OK with *choice set.
template <typename F>
int autotune(fbse_ctx *c, const char *kernel, const std::string &problem, const std::vector<long> &cands, F launch,
             long *choice)
{
  for (const TuneRecord &r : c->tuned)
    if (r.kernel == kernel && r.problem == problem) {
      *choice = r.choice;
      return FBSE_OK;
    }
  TuneRecord rec;
  rec.kernel = kernel;
  rec.problem = problem;
  cudaEvent_t e0, e1;
  FBSE_CUDA(c, cudaEventCreate(&e0));
  FBSE_CUDA(c, cudaEventCreate(&e1));
  int rc = FBSE_OK;
  double best = 1e300;
  for (long v : cands) {
    if ((rc = launch(v))) break;
    FBSE_CUDA(c, cudaEventRecord(e0, c->stream));
    for (int k = 0; k < 2 && !rc; k++) rc = launch(v);
    if (rc) break;
    FBSE_CUDA(c, cudaEventRecord(e1, c->stream));
    FBSE_CUDA(c, cudaEventSynchronize(e1));
    float ms = 0;
    FBSE_CUDA(c, cudaEventElapsedTime(&ms, e0, e1));
    const double us = 500.0 * ms;
    rec.cand.push_back({v, us});
    if (us < best) {
      best = us;
      rec.choice = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  c->tuned.push_back(rec);
  *choice = rec.choice;
  return FBSE_OK;
}

// host copies ordered on the context's (non-blocking) stream; d2h returns
// after the data has arrived
inline cudaError_t h2d(cudaStream_t s, void *dst, const void *src, size_t bytes)
{
  return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
}
inline cudaError_t d2h(cudaStream_t s, void *dst, const void *src, size_t bytes)
{
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
  return e != cudaSuccess ? e : cudaStreamSynchronize(s);
}

// FFT (fft.cu) ----------------------------------------------------------------
int plan_axis(fbse_ctx *c, AxisPlan &p, int n);
void free_axis(AxisPlan &p);
// kinetic part of H: out = a * (T in + V in) + b * in  (V from the context),
// for nblk 3D blocks (states x spins).  work is a scratch of nblk*ngrid complex.
template <typename T>
int kinetic_apply(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *work, long nblk, double a, double b, int with_v);

// out = F^-1 (kq . F in) per 3D block (the hartree convolution); kq holds the
// k-space multiplier including 1/N
template <typename T>
int conv_apply(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *work, long nblk, const double2 *kq);

// psitot rows (FP64) <-> working states in precision T (filter.cu)
template <typename T> int pack(fbse_ctx *c, const double *src, C<T> *dst, long nsrc);
template <typename T> int unpack(fbse_ctx *c, const C<T> *src, double *dst, long ndst);

// projectors (hpsi.cu) --------------------------------------------------------
template <typename T>
int proj_apply(fbse_ctx *c, const C<T> *in, C<T> *out, long nstates, double scale, C<T> *scratch = nullptr);
template <typename T>
int hpsi_apply(fbse_ctx *c, const C<T> *in, C<T> *out, long nstates, double a, double b);
// H psi with the projectors fused into the plane passes (hpsi_fused.cu):
// whether it applies to this context, and out = a H in + b in
bool hpsi_fused_ok(fbse_ctx *c);
int hpsi_fused_apply(fbse_ctx *c, const float2 *in, float2 *out, long nstates, double a, double b);
// the z pass of the kinetic operator (forward, min(k^2/2, KE_max)/N,
// inverse) in place on nblk FP32 blocks (fft.cu)
int zpass_kinetic(fbse_ctx *c, float2 *data, long nblk);

// tensor-core complex products (tcgemm.cu):
//   out[i][j] = scale * sum_r f(A[i][r]) B[j][r], f = conj when conj_a
template <typename S>
int tc_complex_nt(fbse_ctx *c, const S *A, int ma, const S *B, int nb, long L, bool conj_a, double scale,
                  double2 *out);

// reductions / vector ops (filter.cu) ------------------------------------------
template <typename T>
int state_dots(fbse_ctx *c, const C<T> *x, const C<T> *y, long nstates, long len, double *out_host, int mode);

}  // namespace fbse
