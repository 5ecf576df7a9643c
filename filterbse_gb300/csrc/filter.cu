// Newton filter, normalisation, energies and the spectrum range on the GPU
// (Newton recursion, accumulation, normalisation, energies, spectrum range).
//
// Newton filter (replaces filter_cycle, filter_mpi/filter.c:187-371): all
// random starts advance in lockstep as one batch.  The Newton vectors
// phi_j = prod_{i<j}(H_s - z_i) psi_0 live in a ring of K slots: p_hnorm reads
// slot (j-1) % K and writes slot j % K (no copies), and every K terms one
// accumulation kernel forms F_t += sum_q a_{t,j0+q} phi_{j0+q} for all m
// targets, so the m accumulators are read and written once per K terms
// instead of once per term (filter.c:329-359 touches all m every term).
// Accumulators are FP64 in the reference's psi_rank layout.
#include <cmath>

#include "fbse_internal.cuh"

namespace fbse {

constexpr int kMaxTargets = 32;

// ---------------------------------------------------------------------------
// psitot (FP64, stlen per state) <-> working complex states
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_pack(const double *__restrict__ src, C<T> *__restrict__ dst, long nsrc, long len, int cplx)
{
  // len = nspin*ngrid complex elements per working state
  const long nw = cplx ? nsrc : (nsrc + 1) / 2;
  const long total = nw * len;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long w = i / len, k = i - w * len;
    if (cplx) {
      const double *s = src + w * 2 * len;
      dst[i] = mk<T>((T)s[2 * k], (T)s[2 * k + 1]);
    } else {
      const double re = src[(2 * w) * len + k];
      const double im = (2 * w + 1 < nsrc) ? src[(2 * w + 1) * len + k] : 0.0;
      dst[i] = mk<T>((T)re, (T)im);
    }
  }
}

template <typename T>
__global__ void k_unpack(const C<T> *__restrict__ src, double *__restrict__ dst, long ndst, long len, int cplx)
{
  const long nw = cplx ? ndst : (ndst + 1) / 2;
  const long total = nw * len;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long w = i / len, k = i - w * len;
    const C<T> v = src[i];
    if (cplx) {
      dst[w * 2 * len + 2 * k] = (double)v.x;
      dst[w * 2 * len + 2 * k + 1] = (double)v.y;
    } else {
      dst[(2 * w) * len + k] = (double)v.x;
      if (2 * w + 1 < ndst) dst[(2 * w + 1) * len + k] = (double)v.y;
    }
  }
}

static unsigned grid_for(long n, int threads = 256)
{
  long g = (n + threads - 1) / threads;
  if (g > 152L * 32) g = 152L * 32;  // a few waves over the 152 SMs, grid-stride beyond
  if (g < 1) g = 1;
  return (unsigned)g;
}

template <typename T>
int pack(fbse_ctx *c, const double *src, C<T> *dst, long nsrc)
{
  const long len = (long)c->nspin * c->ngrid;
  const long nw = c->is_complex ? nsrc : (nsrc + 1) / 2;
  k_pack<T><<<grid_for(nw * len), 256, 0, c->stream>>>(src, dst, nsrc, len, c->is_complex);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <typename T>
int unpack(fbse_ctx *c, const C<T> *src, double *dst, long ndst)
{
  const long len = (long)c->nspin * c->ngrid;
  const long nw = c->is_complex ? ndst : (ndst + 1) / 2;
  k_unpack<T><<<grid_for(nw * len), 256, 0, c->stream>>>(src, dst, ndst, len, c->is_complex);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template int pack<float>(fbse_ctx *, const double *, C<float> *, long);
template int pack<double>(fbse_ctx *, const double *, C<double> *, long);
template int unpack<float>(fbse_ctx *, const C<float> *, double *, long);
template int unpack<double>(fbse_ctx *, const C<double> *, double *, long);

int pack_states(fbse_ctx *c, const double *src, void *dst, long nsrc)
{
  return c->precision == FBSE_MIXED ? pack<float>(c, src, (float2 *)dst, nsrc) : pack<double>(c, src, (double2 *)dst, nsrc);
}

int unpack_states(fbse_ctx *c, const void *src, double *dst, long ndst)
{
  return c->precision == FBSE_MIXED ? unpack<float>(c, (const float2 *)src, dst, ndst)
                                    : unpack<double>(c, (const double2 *)src, dst, ndst);
}

// ---------------------------------------------------------------------------
// K-blocked Newton accumulation into the psi_rank layout
// F[start][t] (+)= sum_q a[t][j0+q] * ring[(j0+q) % K][w]
// M: the number of targets rounded up to 4, 8, 16 or 32 (compile time).
// The in-block sums run in the working precision T (FP32 on the mixed path)
// and each block's sum is added to the FP64 accumulator, so a larger ring (K
// up to 128 slots) means fewer FP64 read-modify-write passes over F.
// ---------------------------------------------------------------------------
constexpr int kMaxRing = 128;

// ring slots unrolled by 16: more slot loads in flight per thread (2.98 ->
// 2.94 s for the 16 x 16 x 2048 spinor filter at 128^3 against 4)
template <typename T, int M, int U = 16>
__global__ void __launch_bounds__(256) k_newton_acc(const C<T> *__restrict__ ring, long j0, int nk,
                                                   const double *__restrict__ a, long ncheby, int m,
                                                   double *__restrict__ F, long nstart, long nw, long len, int cplx,
                                                   int init)
{
  __shared__ T as[kMaxRing * M];  // as[q * M + t]
  for (int i = threadIdx.x; i < nk * M; i += blockDim.x) {
    const int q = i / M, t = i % M;
    as[i] = t < m ? (T)a[t * ncheby + j0 + q] : T(0);
  }
  __syncthreads();
  const long slot_stride = nw * len;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < slot_stride; i += (long)gridDim.x * blockDim.x) {
    T ar[M], ai[M];
#pragma unroll
    for (int t = 0; t < M; t++) { ar[t] = T(0); ai[t] = T(0); }
    // j0 is a multiple of the ring length: term j0 + q sits in slot q
#pragma unroll U
    for (int q = 0; q < nk; q++) {
      const C<T> v = ring[(long)q * slot_stride + i];
      const T *cq = as + q * M;
#pragma unroll
      for (int t = 0; t < M; t++) {
        ar[t] += cq[t] * v.x;
        ai[t] += cq[t] * v.y;
      }
    }
    const long w = i / len, k = i - w * len;
    // psi_rank layout: ns_block = jns*m*stlen, jstate = ns_block + t*stlen
#pragma unroll
    for (int t = 0; t < M; t++) {
      if (t >= m) break;
      if (cplx) {
        double2 *d = reinterpret_cast<double2 *>(F) + (w * m + t) * len + k;
        double2 o = init ? make_double2(0.0, 0.0) : *d;
        o.x += (double)ar[t];
        o.y += (double)ai[t];
        *d = o;
      } else {
        double *d0 = F + ((2 * w) * m + t) * len + k;
        *d0 = (init ? 0.0 : *d0) + (double)ar[t];
        if (2 * w + 1 < nstart) {
          double *d1 = F + ((2 * w + 1) * m + t) * len + k;
          *d1 = (init ? 0.0 : *d1) + (double)ai[t];
        }
      }
    }
  }
}

template <typename T>
static int launch_newton_acc(fbse_ctx *c, const C<T> *ring, long j0, int nk, const double *a, long ncheby, int m,
                             double *F, long nstart, long nw, long len)
{
  const unsigned g = grid_for(nw * len);
  const int cp = c->is_complex, init = j0 == 0;
  if (m <= 4) k_newton_acc<T, 4><<<g, 256, 0, c->stream>>>(ring, j0, nk, a, ncheby, m, F, nstart, nw, len, cp, init);
  else if (m <= 8) k_newton_acc<T, 8><<<g, 256, 0, c->stream>>>(ring, j0, nk, a, ncheby, m, F, nstart, nw, len, cp, init);
  else if (m <= 16) k_newton_acc<T, 16><<<g, 256, 0, c->stream>>>(ring, j0, nk, a, ncheby, m, F, nstart, nw, len, cp, init);
  else k_newton_acc<T, 32><<<g, 256, 0, c->stream>>>(ring, j0, nk, a, ncheby, m, F, nstart, nw, len, cp, init);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

// ring length: fbse_tuning.newton_ring slots (128 by default), halved while
// the ring would take more than 40% of the free device memory (the ring the
// context already holds counts as free), at most ncheby.  The FP32 block sums
// of the accumulation depend on it.
static long ring_slots(fbse_ctx *c, long ncheby, size_t slot_bytes)
{
  long K = c->tune.newton_ring > 0 ? std::min<long>(c->tune.newton_ring, kMaxRing) : kMaxRing;
  size_t free_b = 0, tot_b = 0;
  if (cudaMemGetInfo(&free_b, &tot_b) != cudaSuccess) {
    cudaGetLastError();
    free_b = 0;
  }
  free_b += c->cache_bytes[kSlotRing];
  while (K > 8 && (double)K * slot_bytes > 0.4 * (double)free_b) K /= 2;
  return ncheby < K ? ncheby : K;
}

// the real parts of the Newton coefficients (gen_newton_coeff's are real)
static int real_coeffs(fbse_ctx *c, const double *an, long ncheby, long m, std::vector<double> &are)
{
  are.assign((size_t)m * ncheby, 0.0);
  for (long t = 0; t < m; t++)
    for (long j = 0; j < ncheby; j++) {
      if (an[2 * (t * ncheby + j) + 1] != 0.0)
        return set_err(c, FBSE_ERR_UNSUPPORTED, "complex Newton coefficients are not supported");
      are[t * ncheby + j] = an[2 * (t * ncheby + j)];
    }
  return FBSE_OK;
}

// the kernel sequence of filter_cycle for every start on the context's
// stream: no allocation and no host synchronisation, so it can be captured
// into a CUDA graph.  ring: K slots of the working states; a_dev: the real
// coefficients [m][ncheby] on the device.
template <typename T>
static int newton_enqueue_t(fbse_ctx *c, const double *zn, long ncheby, long m, double vmin, double de,
                            const double *psi0, long nstart, double *filtered, C<T> *ring, long K,
                            const double *a_dev)
{
  const long len = (long)c->nspin * c->ngrid;
  const long nw = c->is_complex ? nstart : (nstart + 1) / 2;
  const double de_1 = 4.0 / de;
  int rc;
  if ((rc = pack<T>(c, psi0, ring, nstart))) return rc;
  const long slot_stride = nw * len;
  for (long jc = 0; jc < ncheby; jc++) {
    if (jc > 0) {
      const C<T> *src = ring + ((jc - 1) % K) * slot_stride;
      C<T> *dst = ring + (jc % K) * slot_stride;
      // p_hnorm: dE_1 * H psi - (2 + zn + Vmin * dE_1) psi   (filter.c:401-407)
      if ((rc = hpsi_apply<T>(c, src, dst, nw, de_1, -(2.0 + zn[jc - 1] + vmin * de_1)))) return rc;
    }
    if ((jc % K) == K - 1 || jc == ncheby - 1) {
      const long j0 = jc - (jc % K);
      const int nk = (int)(jc - j0 + 1);
      if ((rc = launch_newton_acc<T>(c, ring, j0, nk, a_dev, ncheby, (int)m, filtered, nstart, nw, len))) return rc;
    }
  }
  return FBSE_OK;
}

// ring slots and the ring buffer (kept in the context) for nstart starts
template <typename T>
static int newton_ring_t(fbse_ctx *c, long ncheby, long nstart, long *K_out, void **ring)
{
  const long len = (long)c->nspin * c->ngrid;
  const long nw = c->is_complex ? nstart : (nstart + 1) / 2;
  const long K = ring_slots(c, ncheby, (size_t)nw * len * sizeof(C<T>));
  if (cached(c, kSlotRing, (size_t)K * nw * len * sizeof(C<T>), ring)) return set_err(c, FBSE_ERR_OOM, "newton ring");
  *K_out = K;
  return FBSE_OK;
}

template <typename T>
static int newton_filter_t(fbse_ctx *c, const double *zn, const double *an, long ncheby, long m, double vmin,
                           double de, const double *psi0, long nstart, double *filtered)
{
  std::vector<double> are;
  int rc = real_coeffs(c, an, ncheby, m, are);
  if (rc) return rc;
  long K = 0;
  void *ring = nullptr;
  if ((rc = newton_ring_t<T>(c, ncheby, nstart, &K, &ring))) return rc;
  double *a_dev = nullptr;
  if (cudaMalloc(&a_dev, are.size() * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_OOM, "newton coefficients");
  }
  do {
    if (cudaMemcpyAsync(a_dev, are.data(), are.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream) !=
        cudaSuccess) { rc = set_err(c, FBSE_ERR_CUDA, "coefficient upload"); break; }
    if ((rc = newton_enqueue_t<T>(c, zn, ncheby, m, vmin, de, psi0, nstart, filtered, static_cast<C<T> *>(ring), K,
                                  a_dev)))
      break;
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "newton filter");
    if (!rc) rc = check_dev_status(c);
  } while (0);
  cudaStreamSynchronize(c->stream);
  cudaFree(a_dev);
  return rc;
}

static int newton_args(fbse_ctx *c, long ncheby, long m, long nstart, double de)
{
  if (m < 1 || m > kMaxTargets) return set_err(c, FBSE_ERR_UNSUPPORTED, "mStatesPerFilter must be 1..32");
  if (ncheby < 1 || nstart < 1) return set_err(c, FBSE_ERR_ARG, "ncheby and nstart must be positive");
  if (!(de > 0)) return set_err(c, FBSE_ERR_ARG, "dE must be positive");
  return FBSE_OK;
}

int newton_filter(fbse_ctx *c, const double *zn, const double *an, long ncheby, long m, double vmin, double de,
                  const double *psi0, long nstart, double *filtered)
{
  int rc = newton_args(c, ncheby, m, nstart, de);
  if (rc) return rc;
  if (c->precision == FBSE_MIXED)
    return newton_filter_t<float>(c, zn, an, ncheby, m, vmin, de, psi0, nstart, filtered);
  return newton_filter_t<double>(c, zn, an, ncheby, m, vmin, de, psi0, nstart, filtered);
}

// for the multi-dot batch: validate and upload the coefficients into a_dev
// (m * ncheby doubles, owned by the caller) and size the ring; then
// newton_filter_enqueue only enqueues kernels (capturable)
int newton_filter_prepare(fbse_ctx *c, const double *an, long ncheby, long m, long nstart, double de,
                          double *a_dev, long *K)
{
  int rc = newton_args(c, ncheby, m, nstart, de);
  if (rc) return rc;
  std::vector<double> are;
  if ((rc = real_coeffs(c, an, ncheby, m, are))) return rc;
  if (h2d(c->stream, a_dev, are.data(), are.size() * sizeof(double)) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return set_err(c, FBSE_ERR_CUDA, "coefficient upload");
  void *ring = nullptr;
  return c->precision == FBSE_MIXED ? newton_ring_t<float>(c, ncheby, nstart, K, &ring)
                                    : newton_ring_t<double>(c, ncheby, nstart, K, &ring);
}

int newton_filter_enqueue(fbse_ctx *c, const double *zn, long ncheby, long m, double vmin, double de,
                          const double *psi0, long nstart, double *filtered, const double *a_dev, long K)
{
  void *ring = c->cache[kSlotRing];
  if (!ring) return set_err(c, FBSE_ERR_STATE, "newton ring not prepared");
  if (c->precision == FBSE_MIXED)
    return newton_enqueue_t<float>(c, zn, ncheby, m, vmin, de, psi0, nstart, filtered, static_cast<float2 *>(ring), K,
                                   a_dev);
  return newton_enqueue_t<double>(c, zn, ncheby, m, vmin, de, psi0, nstart, filtered, static_cast<double2 *>(ring), K,
                                  a_dev);
}

// ---------------------------------------------------------------------------
// per-state reductions, FP64 accumulation, deterministic two-stage
//   mode 0: sum |x|^2            (one output per state)
//   mode 1: sum Re(conj(x) y)    (one output per state)
//   mode 2: sum x.re*y.re and sum x.im*y.im   (two outputs per state:
//           the two packed real states of a working state)
// ---------------------------------------------------------------------------
constexpr int kRedBlocks = 64;

template <typename T>
__global__ void __launch_bounds__(256) k_dots(const C<T> *__restrict__ x, const C<T> *__restrict__ y, long len,
                                              int mode, double *__restrict__ part)
{
  const long st = blockIdx.y;
  const C<T> *xs = x + st * len;
  const C<T> *ys = y ? y + st * len : nullptr;
  double s0 = 0.0, s1 = 0.0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < len; k += (long)gridDim.x * blockDim.x) {
    const C<T> a = xs[k];
    if (mode == 0) {
      s0 += (double)a.x * a.x + (double)a.y * a.y;
    } else {
      const C<T> b = ys[k];
      if (mode == 1) s0 += (double)a.x * b.x + (double)a.y * b.y;
      else { s0 += (double)a.x * b.x; s1 += (double)a.y * b.y; }
    }
  }
  __shared__ double r0[8], r1[8];
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
  }
  if ((threadIdx.x & 31) == 0) { r0[threadIdx.x >> 5] = s0; r1[threadIdx.x >> 5] = s1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = 0, a1 = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) { a0 += r0[w]; a1 += r1[w]; }
    part[(st * gridDim.x + blockIdx.x) * 2] = a0;
    part[(st * gridDim.x + blockIdx.x) * 2 + 1] = a1;
  }
}

__global__ void k_dots_final(const double *__restrict__ part, int nb, long nstates, double *__restrict__ out)
{
  for (long st = blockIdx.x * (long)blockDim.x + threadIdx.x; st < nstates; st += (long)gridDim.x * blockDim.x) {
    double a0 = 0, a1 = 0;
    for (int b = 0; b < nb; b++) { a0 += part[(st * nb + b) * 2]; a1 += part[(st * nb + b) * 2 + 1]; }
    out[2 * st] = a0;
    out[2 * st + 1] = a1;
  }
}

// out_dev: 2 doubles per state (second used by mode 2)
template <typename T>
int state_dots_dev(fbse_ctx *c, const C<T> *x, const C<T> *y, long nstates, long len, int mode, double *out_dev)
{
  const size_t need = (size_t)nstates * kRedBlocks * 2 * sizeof(double);
  int rc = ensure(c, (void **)&c->red, &c->red_bytes, need);
  if (rc) return rc;
  if (nstates > 65535) return set_err(c, FBSE_ERR_UNSUPPORTED, "too many states for one reduction");
  dim3 g(kRedBlocks, (unsigned)nstates);
  k_dots<T><<<g, 256, 0, c->stream>>>(x, y, len, mode, c->red);
  FBSE_CHECK_LAUNCH(c);
  k_dots_final<<<(unsigned)((nstates + 127) / 128), 128, 0, c->stream>>>(c->red, kRedBlocks, nstates, out_dev);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <typename T>
int state_dots(fbse_ctx *c, const C<T> *x, const C<T> *y, long nstates, long len, double *out_host, int mode)
{
  double *d = nullptr;
  if (cudaMalloc(&d, nstates * 2 * sizeof(double)) != cudaSuccess) return set_err(c, FBSE_ERR_OOM, "dots");
  int rc = state_dots_dev<T>(c, x, y, nstates, len, mode, d);
  if (!rc && cudaMemcpyAsync(out_host, d, nstates * 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
    rc = set_err(c, FBSE_ERR_CUDA, "dots download");
  if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "dots sync");
  cudaFree(d);
  return rc;
}
template int state_dots<float>(fbse_ctx *, const C<float> *, const C<float> *, long, long, double *, int);
template int state_dots<double>(fbse_ctx *, const C<double> *, const C<double> *, long, long, double *, int);

// ---------------------------------------------------------------------------
// psitot-level normalisation / energies
// ---------------------------------------------------------------------------
__global__ void k_sumsq(const double *__restrict__ x, long len, double *__restrict__ part)
{
  const long st = blockIdx.y;
  const double *xs = x + st * len;
  double s = 0.0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < len; k += (long)gridDim.x * blockDim.x)
    s += xs[k] * xs[k];
  __shared__ double r[8];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) r[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) a += r[w];
    part[(st * gridDim.x + blockIdx.x) * 2] = a;
    part[(st * gridDim.x + blockIdx.x) * 2 + 1] = 0.0;
  }
}

__global__ void k_scale_states(double *__restrict__ x, long len, long n, const double *__restrict__ f)
{
  const long total = n * len;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
    x[i] *= f[i / len];
}

int normalize_all(fbse_ctx *c, double *psitot, long n, double *norms)
{
  const long stlen = (long)(c->is_complex + 1) * c->nspin * c->ngrid;
  if (n < 1) return FBSE_OK;
  if (n > 65535) return set_err(c, FBSE_ERR_UNSUPPORTED, "too many states for one reduction");
  int rc = ensure(c, (void **)&c->red, &c->red_bytes, (size_t)n * kRedBlocks * 2 * sizeof(double));
  if (rc) return rc;
  double *d = nullptr;
  if (cudaMalloc(&d, n * 2 * sizeof(double)) != cudaSuccess) return set_err(c, FBSE_ERR_OOM, "norms");
  std::vector<double> h(2 * n), f(n);
  do {
    FBSE_COUNT(2); k_sumsq<<<dim3(kRedBlocks, (unsigned)n), 256, 0, c->stream>>>(psitot, stlen, c->red);
    k_dots_final<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(c->red, kRedBlocks, n, d);
    if (cudaMemcpyAsync(h.data(), d, n * 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) { rc = set_err(c, FBSE_ERR_CUDA, "norm reduction"); break; }
    for (long i = 0; i < n; i++) {
      const double nr = h[2 * i] * c->dv;  // norm.c:138-140
      if (norms) norms[i] = nr;
      if (nr == 0.0) { rc = set_err(c, FBSE_ERR_NAN, "Norm is 0! exiting!"); break; }
      if (std::isnan(nr)) { rc = set_err(c, FBSE_ERR_NAN, "Norm is NAN! exiting!"); break; }
      f[i] = 1.0 / std::sqrt(nr);
    }
    if (rc) break;
    if (cudaMemcpyAsync(d, f.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "norm upload");
      break;
    }
    FBSE_COUNT(1); k_scale_states<<<grid_for(n * stlen), 256, 0, c->stream>>>(psitot, stlen, n, d);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "normalize");
  } while (0);
  cudaFree(d);
  return rc;
}

template <typename T>
static int energy_all_t(fbse_ctx *c, const double *psitot, long n, double *ene, double *sigma)
{
  const long len = (long)c->nspin * c->ngrid;
  const long nw = c->is_complex ? n : (n + 1) / 2;
  // process in chunks of working states to bound scratch
  const long chunk = nw < 16 ? nw : 16;
  C<T> *buf = nullptr;
  if (cudaMalloc(&buf, 2 * chunk * len * sizeof(C<T>)) != cudaSuccess) return set_err(c, FBSE_ERR_OOM, "energy_all");
  std::vector<double> h(2 * chunk), h2(2 * chunk);
  int rc = FBSE_OK;
  const long stlen = (long)(c->is_complex + 1) * len;
  // sigma_E = sqrt|<H^2> - <H>^2| with <H^2> = dv <H psi|H psi> (calc_sigma_E,
  // energy.c:383-539, applies H twice and takes <psi|H H psi>; the same for
  // Hermitian H)
  auto sig = [&](double e2, double e) { return std::sqrt(std::fabs(e2 * c->dv - e * e)); };
  for (long w0 = 0; w0 < nw && !rc; w0 += chunk) {
    const long cw = (nw - w0 < chunk) ? nw - w0 : chunk;
    const long s0 = c->is_complex ? w0 : 2 * w0;
    const long ns = c->is_complex ? cw : ((n - s0) < 2 * cw ? n - s0 : 2 * cw);
    C<T> *hb = buf + chunk * len;
    if ((rc = pack<T>(c, psitot + s0 * stlen, buf, ns))) break;
    if ((rc = hpsi_apply<T>(c, buf, hb, cw, 1.0, 0.0))) break;
    if ((rc = state_dots<T>(c, buf, hb, cw, len, h.data(), c->is_complex ? 1 : 2))) break;
    if (sigma && (rc = state_dots<T>(c, hb, hb, cw, len, h2.data(), c->is_complex ? 0 : 2))) break;
    for (long w = 0; w < cw; w++) {
      if (c->is_complex) {
        ene[s0 + w] = h[2 * w] * c->dv;
        if (sigma) sigma[s0 + w] = sig(h2[2 * w], ene[s0 + w]);
      } else {
        ene[s0 + 2 * w] = h[2 * w] * c->dv;
        if (sigma) sigma[s0 + 2 * w] = sig(h2[2 * w], ene[s0 + 2 * w]);
        if (s0 + 2 * w + 1 < n) {
          ene[s0 + 2 * w + 1] = h[2 * w + 1] * c->dv;
          if (sigma) sigma[s0 + 2 * w + 1] = sig(h2[2 * w + 1], ene[s0 + 2 * w + 1]);
        }
      }
    }
  }
  cudaFree(buf);
  return rc;
}

int energy_all(fbse_ctx *c, const double *psitot, long n, double *ene, double *sigma)
{
  if (n < 1) return FBSE_OK;
  return c->precision == FBSE_MIXED ? energy_all_t<float>(c, psitot, n, ene, sigma)
                                    : energy_all_t<double>(c, psitot, n, ene, sigma);
}

// ---------------------------------------------------------------------------
// spectrum range (energy.c:169-379, iterative branch)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_axpby(C<T> *__restrict__ y, const C<T> *__restrict__ x, long len, double a, double b)
{  // y = a*y + b*x
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < len; i += (long)gridDim.x * blockDim.x) {
    C<T> v = y[i], u = x[i];
    y[i] = mk<T>((T)(a * v.x + b * u.x), (T)(a * v.y + b * u.y));
  }
}

template <typename T>
__global__ void k_cast_in(const double *__restrict__ s, C<T> *__restrict__ d, long len)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < len; i += (long)gridDim.x * blockDim.x)
    d[i] = mk<T>((T)s[2 * i], (T)s[2 * i + 1]);
}

extern "C" long fbse_host_init_psi(double *psi, long seed, long ngrid, int is_complex, double dv);

template <typename T>
static int energy_range_t(fbse_ctx *c, long seed, long max_iter, double *emin_out, double *emax_out, long *iters)
{
  const long len = (long)c->nspin * c->ngrid;
  C<T> *buf = nullptr;  // phi, h
  double *hd = nullptr;
  if (cudaMalloc(&buf, 2 * len * sizeof(C<T>)) != cudaSuccess) return set_err(c, FBSE_ERR_OOM, "energy range");
  if (cudaMalloc(&hd, len * 2 * sizeof(double)) != cudaSuccess) { cudaFree(buf); return set_err(c, FBSE_ERR_OOM, "energy range"); }
  C<T> *phi = buf, *h = buf + len;
  std::vector<double> host(2 * len);
  double dd[2];
  int rc = FBSE_OK;
  long it_total = 0;
  auto draw = [&](void) -> int {
    for (int s = 0; s < c->nspin; s++) seed = fbse_host_init_psi(host.data() + 2 * s * c->ngrid, seed, c->ngrid, c->is_complex, c->dv);
    if (cudaMemcpyAsync(hd, host.data(), len * 2 * sizeof(double), cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
      return set_err(c, FBSE_ERR_CUDA, "energy range upload");
    k_cast_in<T><<<grid_for(len), 256, 0, c->stream>>>(hd, phi, len);
    FBSE_CHECK_LAUNCH(c);
    return FBSE_OK;
  };
  do {
    // ---- E_min: phi <- normalize(phi - tau H phi)   (energy.c:221-271)
    if ((rc = draw())) break;
    double tau = 0.05, emin = 10.0, old = 0.0;
    if ((rc = hpsi_apply<T>(c, phi, h, 1, 1.0, 0.0))) break;
    for (long i = 0; std::fabs((emin - old) / emin) > 1.0e-6 && i < max_iter; i++) {
      // h holds H phi_i
      FBSE_COUNT(1); k_axpby<T><<<grid_for(len), 256, 0, c->stream>>>(phi, h, len, 1.0, -tau);
      if ((rc = state_dots<T>(c, phi, nullptr, 1, len, dd, 0))) break;
      const double nrm = std::sqrt(dd[0] * c->dv);
      FBSE_COUNT(1); k_axpby<T><<<grid_for(len), 256, 0, c->stream>>>(phi, phi, len, 1.0 / nrm, 0.0);
      if ((rc = hpsi_apply<T>(c, phi, h, 1, 1.0, 0.0))) break;
      if ((rc = state_dots<T>(c, phi, h, 1, len, dd, 1))) break;
      old = emin;
      emin = dd[0] * c->dv;
      if (i > 5 && (emin - old) > 0) tau -= 0.025;  // energy.c:262-269
      it_total++;
    }
    if (rc) break;
    // ---- E_max: power iteration psi <- normalize(H psi)   (energy.c:281-303)
    if ((rc = draw())) break;
    double emax = 0.1;
    old = 0.0;
    if ((rc = hpsi_apply<T>(c, phi, h, 1, 1.0, 0.0))) break;
    for (long i = 0; std::fabs((emax - old) / emax) > 1.0e-6 && i < max_iter; i++) {
      if ((rc = state_dots<T>(c, h, nullptr, 1, len, dd, 0))) break;
      const double nrm = std::sqrt(dd[0] * c->dv);
      FBSE_COUNT(1); k_axpby<T><<<grid_for(len), 256, 0, c->stream>>>(phi, h, len, 0.0, 1.0 / nrm);
      if ((rc = hpsi_apply<T>(c, phi, h, 1, 1.0, 0.0))) break;
      if ((rc = state_dots<T>(c, phi, h, 1, len, dd, 1))) break;
      old = emax;
      emax = dd[0] * c->dv;
      it_total++;
    }
    if (rc) break;
    *emin_out = emin;
    *emax_out = emax;
    if (iters) *iters = it_total;
  } while (0);
  cudaStreamSynchronize(c->stream);
  cudaFree(buf);
  cudaFree(hd);
  return rc;
}

int energy_range(fbse_ctx *c, long seed, long max_iter, double *emin, double *emax, long *iters)
{
  return c->precision == FBSE_MIXED ? energy_range_t<float>(c, seed, max_iter, emin, emax, iters)
                                    : energy_range_t<double>(c, seed, max_iter, emin, emax, iters);
}

}  // namespace fbse

// ---------------------------------------------------------------------------
// normalize_all without any allocation: the partial sums, norms, scale
// factors and the error key live in one file-scope device array.  Its device
// address is looked up (cudaGetSymbolAddress, with the caller's device
// current) on the first call in each CUDA context -- the device's primary
// context for runtime-API callers -- and kept per context id, so a device
// reset or another context gets its own lookup.  Only the error key must start
// at a known value; it is set on the stream at the start of every call.  The
// array is shared by every fbse context on the device, so overlapping calls
// race.
// ---------------------------------------------------------------------------

#include <cuda.h>  // CUcontext / CUresult types only; the driver is reached through the runtime

#include <mutex>

namespace fbse {

constexpr long kNoAllocMaxStates = 1024;
constexpr long kNoAllocPart = kNoAllocMaxStates * kRedBlocks * 2;  // doubles of partial sums
constexpr long kNoAllocDoubles = kNoAllocPart + 2 * kNoAllocMaxStates + 32;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

namespace {
std::mutex g_noalloc_mu;
struct NoAllocEntry {
  unsigned long long ctx_id;
  double *ptr;
};
std::vector<NoAllocEntry> g_noalloc_cache;
typedef CUresult (*PfnCtxGetCurrent)(CUcontext *);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long *);
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;
}  // namespace

// norms, factors and the first failing state: key = 2 * index + (NaN ? 1 : 0)
__global__ void k_norm_factors(const double *__restrict__ part, int nb, long n, double dv, double *__restrict__ norms,
                               double *__restrict__ f, int *__restrict__ key)
{
  for (long st = blockIdx.x * (long)blockDim.x + threadIdx.x; st < n; st += (long)gridDim.x * blockDim.x) {
    double a = 0;
    for (int b = 0; b < nb; b++) a += part[(st * nb + b) * 2];
    const double nr = a * dv;  // norm.c:138-140
    norms[st] = nr;
    if (nr == 0.0) atomicMin(key, (int)(2 * st));
    else if (isnan(nr)) atomicMin(key, (int)(2 * st + 1));
    f[st] = 1.0 / sqrt(nr);
  }
}

__global__ void k_scale_states_if_ok(double *__restrict__ x, long len, long n, const double *__restrict__ f,
                                     const int *__restrict__ key)
{
  if (*key != 0x7f7f7f7f) return;  // a zero or NaN norm: leave the states as they were
  const long total = n * len;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
    x[i] *= f[i / len];
}

// id of the caller's current CUDA context (after the runtime has made the
// device's primary context current), through driver entry points obtained
// from the runtime, so the library does not link the driver library itself
static int current_ctx_id(fbse_ctx *c, unsigned long long *id)
{
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2) {
      cudaGetLastError();
      return set_err(c, FBSE_ERR_CUDA, "fbse_normalize_all_noalloc: driver entry points unavailable");
    }
    g_ctx_get_current = (PfnCtxGetCurrent)f1;
    g_ctx_get_id = (PfnCtxGetId)f2;
  }
  if (cudaFree(nullptr) != cudaSuccess) {  // makes the device's primary context current
    cudaGetLastError();
    return set_err(c, FBSE_ERR_CUDA, "fbse_normalize_all_noalloc: no usable device");
  }
  CUcontext cu = nullptr;
  if (g_ctx_get_current(&cu) != CUDA_SUCCESS || !cu || g_ctx_get_id(cu, id) != CUDA_SUCCESS)
    return set_err(c, FBSE_ERR_CUDA, "fbse_normalize_all_noalloc: no current context");
  return FBSE_OK;
}

static int noalloc_scratch(fbse_ctx *c, double **out)
{
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  unsigned long long id = 0;
  int rc = current_ctx_id(c, &id);
  if (rc) return rc;
  for (const NoAllocEntry &e : g_noalloc_cache)
    if (e.ctx_id == id) {
      *out = e.ptr;
      return FBSE_OK;
    }
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_CUDA,
                   std::string("fbse_normalize_all_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  }
  g_noalloc_cache.push_back({id, (double *)p});
  *out = (double *)p;
  return FBSE_OK;
}

int normalize_all_noalloc(fbse_ctx *c, double *psitot, long n, double *norms)
{
  if (n < 1) return FBSE_OK;
  if (n > kNoAllocMaxStates)
    return set_err(c, FBSE_ERR_ARG, "fbse_normalize_all_noalloc: " + std::to_string(n) + " states exceed the " +
                                        std::to_string(kNoAllocMaxStates) + "-state scratch");
  double *s = nullptr;
  int rc = noalloc_scratch(c, &s);
  if (rc) return rc;
  double *part = s, *nrm = s + kNoAllocPart, *f = nrm + kNoAllocMaxStates;
  int *key = (int *)(f + kNoAllocMaxStates);
  const long stlen = (long)(c->is_complex + 1) * c->nspin * c->ngrid;
  int hkey = 0;
  if (cudaMemsetAsync(key, 0x7f, sizeof(int), c->stream) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_CUDA, "fbse_normalize_all_noalloc: key reset");
  }
  k_sumsq<<<dim3(kRedBlocks, (unsigned)n), 256, 0, c->stream>>>(psitot, stlen, part);
  FBSE_CHECK_LAUNCH(c);
  k_norm_factors<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(part, kRedBlocks, n, c->dv, nrm, f, key);
  FBSE_CHECK_LAUNCH(c);
  k_scale_states_if_ok<<<grid_for(n * stlen), 256, 0, c->stream>>>(psitot, stlen, n, f, key);
  FBSE_CHECK_LAUNCH(c);
  // norms as fbse_normalize_all leaves them: up to and including the first
  // state with a zero or NaN norm when there is one, all n otherwise
  if (d2h(c->stream, &hkey, key, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_CUDA, "fbse_normalize_all_noalloc: download");
  }
  const long nout = hkey != 0x7f7f7f7f ? std::min<long>(n, hkey / 2 + 1) : n;
  if (norms && d2h(c->stream, norms, nrm, nout * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_CUDA, "fbse_normalize_all_noalloc: download");
  }
  if (hkey != 0x7f7f7f7f) return set_err(c, FBSE_ERR_NAN, (hkey & 1) ? "Norm is NAN! exiting!" : "Norm is 0! exiting!");
  return FBSE_OK;
}

}  // namespace fbse

extern "C" int fbse_normalize_all_noalloc(fbse_ctx *c, double *psitot, long n, double *norms)
{
  if (!c || !psitot) return c ? fbse::set_err(c, FBSE_ERR_ARG, "fbse_normalize_all_noalloc: null") : FBSE_ERR_ARG;
  return fbse::normalize_all_noalloc(c, psitot, n, norms);
}
