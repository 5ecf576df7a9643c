// Batched mixed-radix 3D FFT for the kinetic term of H.
//
// Replaces kinetic() (filter_mpi/hamiltonian.c:62-99), i.e. FFTW's
// fftw_plan_dft_3d(nz, ny, nx) forward transform, the ksqr multiply and the
// unnormalised backward transform (plans made in filter_mpi/aux.c:259-270).
//
// Design: every axis is transformed by a self-sorting Stockham FFT held in
// shared memory.  The grid sizes the reference's auto-grid produces are
// arbitrary (e.g. 57 x 52 x 45 = 3*19 x 4*13 x 9*5), so each axis is factored
// into radix-4/2/3 stages with hand-written butterflies plus generic odd-prime
// stages; twiddles and butterfly roots come from one table of n roots
// e^{-2 pi i t/n} per axis, computed on the host in extended precision.
//   pass 1  x lines (contiguous): forward
//   pass 2  y lines, tiles of TX consecutive x columns: forward
//   pass 3  z lines, tiles of TX consecutive x columns: forward, multiply by
//           min(kx^2 + ky^2 + kz^2 terms, KE_max)/N computed from the indices
//           exactly as filter_mpi/init.c:318-351 builds ksqr, inverse
//   pass 4  y lines: inverse
//   pass 5  x lines: inverse, fused epilogue out = a (T psi + V psi) + b psi
// so the k^2 table costs no HBM traffic and the local potential and the
// Newton scale-and-shift ride on the last pass.
#include <cmath>

#include "fbse_internal.cuh"

namespace fbse {

struct Stages {
  int n;
  int nst;
  int radix[kMaxStages];
};

static std::vector<int> factorize(int n)
{
  std::vector<int> r;
  while (n % 4 == 0) { r.push_back(4); n /= 4; }
  while (n % 2 == 0) { r.push_back(2); n /= 2; }
  while (n % 3 == 0) { r.push_back(3); n /= 3; }
  for (int p = 5; (long)p * p <= n; p += 2)
    while (n % p == 0) { r.push_back(p); n /= p; }
  if (n > 1) r.push_back(n);
  return r;
}

int plan_axis(fbse_ctx *c, AxisPlan &p, int n)
{
  if (n < 1) return set_err(c, FBSE_ERR_ARG, "grid axis must have at least one point");
  std::vector<int> f = factorize(n);
  if ((int)f.size() > kMaxStages) return set_err(c, FBSE_ERR_UNSUPPORTED, "axis length has too many factors");
  p.n = n;
  p.nst = (int)f.size();
  for (int i = 0; i < p.nst; i++) p.radix[i] = f[i];
  std::vector<double2> h64(n);
  std::vector<float2> h32(n);
  for (int t = 0; t < n; t++) {
    // e^{-2 pi i t / n} in extended precision, then rounded
    long double a = 2.0L * 3.14159265358979323846264338327950288L * (long double)t / (long double)n;
    double cr = (double)cosl(a), ci = -(double)sinl(a);
    h64[t] = make_double2(cr, ci);
    h32[t] = make_float2((float)cr, (float)ci);
  }
  FBSE_CUDA(c, cudaMalloc(&p.tw64, n * sizeof(double2)));
  FBSE_CUDA(c, cudaMalloc(&p.tw32, n * sizeof(float2)));
  FBSE_CUDA(c, cudaMemcpy(p.tw64, h64.data(), n * sizeof(double2), cudaMemcpyHostToDevice));
  FBSE_CUDA(c, cudaMemcpy(p.tw32, h32.data(), n * sizeof(float2), cudaMemcpyHostToDevice));
  return FBSE_OK;
}

void free_axis(AxisPlan &p)
{
  if (p.tw64) cudaFree(p.tw64);
  if (p.tw32) cudaFree(p.tw32);
  p.tw64 = nullptr;
  p.tw32 = nullptr;
}

static Stages stages_of(const AxisPlan &p)
{
  Stages s;
  s.n = p.n;
  s.nst = p.nst;
  for (int i = 0; i < kMaxStages; i++) s.radix[i] = p.radix[i];
  return s;
}

template <typename T> static const C<T> *roots(const AxisPlan &p);
template <> const C<float> *roots<float>(const AxisPlan &p) { return p.tw32; }
template <> const C<double> *roots<double>(const AxisPlan &p) { return p.tw64; }

// ---------------------------------------------------------------------------
// one Stockham stage in shared memory
//   COLS = false: lines are contiguous (element stride 1, line stride n) and
//                 consecutive threads walk along a line;
//   COLS = true : element i of line c sits at i*L + c, consecutive threads
//                 walk across lines (conflict-free for column tiles).
// ---------------------------------------------------------------------------
template <typename T, bool COLS>
__device__ __forceinline__ void stage(C<T> *__restrict__ src, C<T> *__restrict__ dst, const C<T> *__restrict__ tw,
                                      int n, int L, int p, int Ns, bool inv)
{
  const int nb = n / p;
  const int total = nb * L;
  const int twstep = n / (Ns * p);
  const int rstep = nb;  // root index of e^{-2 pi i / p}
  const T sg = inv ? T(1) : T(-1);
  for (int w = threadIdx.x; w < total; w += blockDim.x) {
    int c, j;
    if (COLS) { c = w % L; j = w / L; }
    else { c = w / nb; j = w - c * nb; }
    const int k = j % Ns;
    const int obase = (j / Ns) * Ns * p + k;
    auto IN = [&](int i) -> C<T> & { return COLS ? src[i * L + c] : src[c * n + i]; };
    auto OUT = [&](int i) -> C<T> & { return COLS ? dst[i * L + c] : dst[c * n + i]; };
    auto W = [&](int t) -> C<T> { C<T> r = tw[t]; if (inv) r.y = -r.y; return r; };
    if (p == 2) {
      C<T> v0 = IN(j), v1 = cmul<T>(IN(j + nb), W(k * twstep));
      OUT(obase) = cadd<T>(v0, v1);
      OUT(obase + Ns) = csub<T>(v0, v1);
    } else if (p == 4) {
      C<T> v0 = IN(j);
      C<T> v1 = cmul<T>(IN(j + nb), W(k * twstep));
      C<T> v2 = cmul<T>(IN(j + 2 * nb), W(2 * k * twstep));
      C<T> v3 = cmul<T>(IN(j + 3 * nb), W(3 * k * twstep));
      C<T> a = cadd<T>(v0, v2), b = csub<T>(v0, v2), cc = cadd<T>(v1, v3), d = csub<T>(v1, v3);
      // s*i*d with s = -1 forward, +1 inverse
      C<T> id = mk<T>(-sg * d.y, sg * d.x);
      OUT(obase) = cadd<T>(a, cc);
      OUT(obase + Ns) = cadd<T>(b, id);
      OUT(obase + 2 * Ns) = csub<T>(a, cc);
      OUT(obase + 3 * Ns) = csub<T>(b, id);
    } else if (p == 3) {
      C<T> v0 = IN(j);
      C<T> v1 = cmul<T>(IN(j + nb), W(k * twstep));
      C<T> v2 = cmul<T>(IN(j + 2 * nb), W(2 * k * twstep));
      const T h = T(0.86602540378443864676372317075293618);
      C<T> s12 = cadd<T>(v1, v2), d12 = csub<T>(v1, v2);
      C<T> t = mk<T>(v0.x - T(0.5) * s12.x, v0.y - T(0.5) * s12.y);
      // u = s*(sqrt(3)/2)*(v1 - v2); i*u
      C<T> iu = mk<T>(-sg * h * d12.y, sg * h * d12.x);
      OUT(obase) = cadd<T>(v0, s12);
      OUT(obase + Ns) = cadd<T>(t, iu);
      OUT(obase + 2 * Ns) = csub<T>(t, iu);
    } else {
      // generic radix: twiddle this butterfly's inputs in place (each input
      // element of a stage is read by exactly one butterfly), then a direct
      // length-p DFT with roots from the table.
      for (int r = 1; r < p; r++) IN(j + r * nb) = cmul<T>(IN(j + r * nb), W(r * k * twstep));
      for (int q = 0; q < p; q++) {
        C<T> acc = IN(j);
        int e = 0;
        for (int r = 1; r < p; r++) {
          e += q;
          if (e >= p) e -= p;
          acc = cadd<T>(acc, cmul<T>(IN(j + r * nb), W(e * rstep)));
        }
        OUT(obase + q * Ns) = acc;
      }
    }
  }
}

// full transform of L lines held in a; returns the buffer holding the result
template <typename T, bool COLS>
__device__ C<T> *fft_lines(C<T> *a, C<T> *b, const C<T> *tw, const Stages &st, int L, bool inv)
{
  int Ns = 1;
  for (int s = 0; s < st.nst; s++) {
    stage<T, COLS>(a, b, tw, st.n, L, st.radix[s], Ns, inv);
    __syncthreads();
    Ns *= st.radix[s];
    C<T> *t = a;
    a = b;
    b = t;
  }
  return a;
}

// ---------------------------------------------------------------------------
// x pass: L contiguous lines per CTA.  EPI = 0: store; EPI = 1: fused
// out = a (kin + V phi) + b phi with V indexed by the spatial point.
// ---------------------------------------------------------------------------
template <typename T, int EPI>
__global__ void __launch_bounds__(256) k_fft_x(const C<T> *__restrict__ in, C<T> *__restrict__ out, Stages st,
                                               const C<T> *__restrict__ twg, long nlines, int L, bool inv,
                                               const C<T> *__restrict__ phi, const T *__restrict__ pot, long ngrid,
                                               T ca, T cb)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = st.n;
  C<T> *tw = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *A = tw + n;
  C<T> *B = A + (long)L * n;
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];
  const long line0 = (long)blockIdx.x * L;
  const int nl = (int)min((long)L, nlines - line0);
  const long off = line0 * n;
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) A[t] = in[off + t];
  __syncthreads();
  C<T> *r = fft_lines<T, false>(A, B, tw, st, nl, inv);
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    C<T> v = r[t];
    if (EPI == 1) {
      const long g = off + t;
      const C<T> ph = phi[g];
      if (pot) {
        const T V = pot[g % ngrid];
        v.x += V * ph.x;
        v.y += V * ph.y;
      }
      v.x = ca * v.x + cb * ph.x;
      v.y = ca * v.y + cb * ph.y;
    }
    out[off + t] = v;
  }
}

// ---------------------------------------------------------------------------
// column pass (y or z lines): a tile of TX consecutive x columns of one
// (block, plane) with element stride es.  Tile o addresses
// base = (o / cnt) * s1 + (o % cnt) * s2 + xt * TX.
// KMUL: forward, multiply by the kinetic factor, inverse (z pass only).
// ---------------------------------------------------------------------------
struct KinArgs {
  const double *k2x, *k2y, *k2z;
  double kemax;
  int nx, ny;
};

template <typename T, bool KMUL>
__global__ void __launch_bounds__(256) k_fft_cols(C<T> *__restrict__ data, Stages st, const C<T> *__restrict__ twg,
                                                  long es, int nxc, int TX, int nxt, long cnt, long s1, long s2,
                                                  bool inv, KinArgs ka)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = st.n;
  C<T> *tw = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *A = tw + n;
  C<T> *B = A + (long)TX * n;
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];
  const long o = blockIdx.x / nxt;
  const int xt = blockIdx.x % nxt;
  const int x0 = xt * TX;
  const int L = min(TX, nxc - x0);
  const long base = (o / cnt) * s1 + (o % cnt) * s2 + x0;
  for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
    const int cc = t % L, i = t / L;
    A[i * L + cc] = data[base + (long)i * es + cc];
  }
  __syncthreads();
  C<T> *r = fft_lines<T, true>(A, B, tw, st, L, KMUL ? false : inv);
  if (KMUL) {
    const int jy = (int)(o % cnt);
    const double ky = ka.k2y[jy];
    for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
      const int cc = t % L, i = t / L;
      double kk = ka.k2x[x0 + cc] + ky + ka.k2z[i];
      if (kk > ka.kemax) kk = ka.kemax;
      r[t] = cscale<T>(r[t], (T)kk);
    }
    __syncthreads();
    C<T> *other = (r == A) ? B : A;
    r = fft_lines<T, true>(r, other, tw, st, L, true);
  }
  for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
    const int cc = t % L, i = t / L;
    data[base + (long)i * es + cc] = r[i * L + cc];
  }
}

template <typename T> static const T *pot_of(fbse_ctx *c);
template <> const float *pot_of<float>(fbse_ctx *c) { return c->pot32; }
template <> const double *pot_of<double>(fbse_ctx *c) { return c->pot64; }

static int cols_tile(int nx) { return nx < 16 ? nx : 16; }

template <typename T>
static int launch_x(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, bool inv, int epi, const C<T> *phi,
                    const T *pot, T ca, T cb)
{
  const AxisPlan &p = c->ax[0];
  const int n = p.n;
  const long nlines = nblk * c->ny * c->nz;
  int L = 2048 / n;
  if (L < 1) L = 1;
  if (L > 64) L = 64;
  const size_t smem = (size_t)(n + 2L * L * n) * sizeof(C<T>);
  const long grid = (nlines + L - 1) / L;
  Stages st = stages_of(p);
  if (epi) {
    FBSE_CUDA(c, cudaFuncSetAttribute(k_fft_x<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_x<T, 1><<<grid, 256, smem, c->stream>>>(in, out, st, roots<T>(p), nlines, L, inv, phi, pot, c->ngrid, ca, cb);
  } else {
    FBSE_CUDA(c, cudaFuncSetAttribute(k_fft_x<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_x<T, 0><<<grid, 256, smem, c->stream>>>(in, out, st, roots<T>(p), nlines, L, inv, nullptr, nullptr,
                                                   c->ngrid, T(1), T(0));
  }
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <typename T>
static int launch_cols(fbse_ctx *c, C<T> *data, long nblk, int axis, bool inv, bool kmul)
{
  const AxisPlan &p = c->ax[axis];
  const int n = p.n;
  const int TX = cols_tile((int)c->nx);
  const int nxt = (int)((c->nx + TX - 1) / TX);
  long es, cnt, s1, s2, nouter;
  if (axis == 1) {  // y lines: outer = block*nz + z
    es = c->nx;
    cnt = 1;
    s1 = c->nx * c->ny;
    s2 = 0;
    nouter = nblk * c->nz;
  } else {  // z lines: outer = block*ny + y
    es = c->nx * c->ny;
    cnt = c->ny;
    s1 = c->ngrid;
    s2 = c->nx;
    nouter = nblk * c->ny;
  }
  const size_t smem = (size_t)(n + 2L * TX * n) * sizeof(C<T>);
  const long grid = nouter * nxt;
  KinArgs ka{c->k2x, c->k2y, c->k2z, c->kemax_scaled, (int)c->nx, (int)c->ny};
  Stages st = stages_of(p);
  if (kmul) {
    FBSE_CUDA(c, cudaFuncSetAttribute(k_fft_cols<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_cols<T, true><<<grid, 256, smem, c->stream>>>(data, st, roots<T>(p), es, (int)c->nx, TX, nxt, cnt, s1, s2,
                                                         inv, ka);
  } else {
    FBSE_CUDA(c, cudaFuncSetAttribute(k_fft_cols<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_cols<T, false><<<grid, 256, smem, c->stream>>>(data, st, roots<T>(p), es, (int)c->nx, TX, nxt, cnt, s1,
                                                          s2, inv, ka);
  }
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <typename T>
int kinetic_apply(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *work, long nblk, double a, double b, int with_v)
{
  int rc;
  if ((rc = launch_x<T>(c, in, work, nblk, false, 0, nullptr, nullptr, T(1), T(0)))) return rc;
  if ((rc = launch_cols<T>(c, work, nblk, 1, false, false))) return rc;
  if ((rc = launch_cols<T>(c, work, nblk, 2, false, true))) return rc;
  if ((rc = launch_cols<T>(c, work, nblk, 1, true, false))) return rc;
  return launch_x<T>(c, work, out, nblk, true, 1, in, with_v ? pot_of<T>(c) : nullptr, (T)a, (T)b);
}

template int kinetic_apply<float>(fbse_ctx *, const C<float> *, C<float> *, C<float> *, long, double, double, int);
template int kinetic_apply<double>(fbse_ctx *, const C<double> *, C<double> *, C<double> *, long, double, double, int);

}  // namespace fbse
