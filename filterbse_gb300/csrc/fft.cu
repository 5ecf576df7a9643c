// Batched mixed-radix 3D FFT for the kinetic term of H.
//
// Replaces kinetic() (filter_mpi/hamiltonian.c:62-99), i.e. FFTW's
// fftw_plan_dft_3d(nz, ny, nx) forward transform, the ksqr multiply and the
// unnormalised backward transform (plans made in filter_mpi/aux.c:259-270).
//
// Each axis is a self-sorting mixed-radix Stockham FFT on lines held in shared
// memory.  The grid sizes the reference's auto-grid produces are arbitrary
// (e.g. 57 x 52 x 45 = 3*19 x 4*13 x 9*5), so an axis is factored into
// register radices: powers of two grouped into radix-16 / 8 / 4 / 2 passes
// (in-register DIF butterflies with compile-time roots) and the odd primes
// 3, 5, 7 (in-register direct DFTs with roots from the axis table); a larger
// prime takes a shared-memory pass with a scratch line.  Each pass is in place:
// every thread reads its butterflies' inputs into registers, the block
// synchronises, then the outputs are written -- so a pass costs one read and
// one write of shared memory and two barriers, and the butterfly radices keep
// the number of passes at 2-3 for typical axes (128 = 16 x 8).  Lanes of a
// warp always take consecutive lines at the same butterfly index, so index
// arithmetic and twiddles are warp-uniform; row-major lines use an odd row
// stride so the accesses are free of bank conflicts.  Twiddles come from one
// table of n roots e^{-2 pi i t/n} per axis, computed on the host in extended
// precision.
//
// Plane path (an xy plane fits in shared memory, the usual case in FP32):
//   pass 1  per (block, z): load the plane, x then y forward, store
//   pass 2  z lines in tiles of x-columns: forward, multiply by
//           min(kx^2 + ky^2 + kz^2 terms, KE_max)/N computed from the indices
//           exactly as filter_mpi/init.c:318-351 builds ksqr, inverse
//   pass 3  per (block, z): y then x inverse, fused epilogue
//           out = a (T psi + V psi) + b psi
// Line path (larger planes, FP64): x, y, z-fused, y, x passes.
// Blocks are processed in chunks sized so that a chunk's scratch stays in L2
// between the passes.
#include <cmath>

#include "fbse_internal.cuh"
#include "fft_common.cuh"

namespace fbse {

struct Stages {
  int n;
  int nst;
  int radix[kMaxStages];
  int big;  // 1 when a radix exceeds the register limit (needs a scratch line)
};

constexpr int kRegMax = 8;  // odd radices above this take the scratch pass

static std::vector<int> factorize(int n)
{
  std::vector<int> r;
  int a = 0;
  while (n % 2 == 0) { a++; n /= 2; }
  while (a > 4) { r.push_back(16); a -= 4; }
  if (a > 0) r.push_back(1 << a);
  for (int p = 3; (long)p * p <= n; p += 2)
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
  s.big = 0;
  for (int i = 0; i < kMaxStages; i++) {
    s.radix[i] = p.radix[i];
    if (i < p.nst && p.radix[i] > kRegMax && p.radix[i] != 16) s.big = 1;
  }
  return s;
}

template <typename T> static const C<T> *roots(const AxisPlan &p);
template <> const C<float> *roots<float>(const AxisPlan &p) { return p.tw32; }
template <> const C<double> *roots<double>(const AxisPlan &p) { return p.tw64; }

// direct DFT for an odd radix with roots w[e] = e^{sg 2 pi i e / R}
template <typename T, int R>
__device__ __forceinline__ void dft_odd(C<T> *v, const C<T> *w)
{
  C<T> o[R];
#pragma unroll
  for (int q = 0; q < R; q++) {
    C<T> acc = v[0];
#pragma unroll
    for (int r = 1; r < R; r++) acc = cadd<T>(acc, cmul<T>(v[r], w[(q * r) % R]));
    o[q] = acc;
  }
#pragma unroll
  for (int q = 0; q < R; q++) v[q] = o[q];
}

template <typename T>
__device__ __forceinline__ void dft3(C<T> *v, T sg)
{
  const T h = T(0.86602540378443864676372317075293618);
  const C<T> s12 = cadd<T>(v[1], v[2]), d12 = csub<T>(v[1], v[2]);
  const C<T> t = mk<T>(v[0].x - T(0.5) * s12.x, v[0].y - T(0.5) * s12.y);
  const C<T> iu = mk<T>(-sg * h * d12.y, sg * h * d12.x);
  v[0] = cadd<T>(v[0], s12);
  v[1] = cadd<T>(t, iu);
  v[2] = csub<T>(t, iu);
}

template <typename T, int R> struct IsPow2 { static constexpr bool value = (R & (R - 1)) == 0; };

// ---------------------------------------------------------------------------
// one in-place Stockham pass of radix R over L lines (element i of line c at
// buf[c * ls + i * es]); lanes take consecutive lines at one butterfly index
// ---------------------------------------------------------------------------
template <typename T, int R>
__device__ __forceinline__ void pass_reg(C<T> *buf, int es, int ls, int n, int L, int Ns, const C<T> *__restrict__ tw,
                                      bool inv)
{
  constexpr int kMaxE = R;                              // one butterfly per thread per round
  constexpr int BMAX = (kMaxE / R) > 0 ? kMaxE / R : 1;
  const int nb = n / R;
  const int twstep = n / (Ns * R);
  const T sg = inv ? T(1) : T(-1);
  C<T> w[IsPow2<T, R>::value ? 1 : R];
  if (!IsPow2<T, R>::value && R != 3) {
#pragma unroll
    for (int e = 0; e < (IsPow2<T, R>::value ? 1 : R); e++) {
      C<T> r = tw[e * nb];
      if (inv) r.y = -r.y;
      w[e] = r;
    }
  }
  const int lines_per_round = max(1, (int)(blockDim.x * BMAX) / nb);
  for (int l0 = 0; l0 < L; l0 += lines_per_round) {
    const int lr = min(lines_per_round, L - l0);
    const int tb = nb * lr;
    C<T> v[BMAX][R];
#pragma unroll
    for (int b = 0; b < BMAX; b++) {
      const int wi = threadIdx.x + b * blockDim.x;
      if (wi < tb) {
        const int c = l0 + wi % lr, j = wi / lr;
        const int k = j % Ns;
        const C<T> *x = buf + c * ls;
        v[b][0] = x[j * es];
#pragma unroll
        for (int q = 1; q < R; q++) {
          C<T> t = tw[q * k * twstep];
          if (inv) t.y = -t.y;
          v[b][q] = cmul<T>(x[(j + q * nb) * es], t);
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < BMAX; b++) {
      const int wi = threadIdx.x + b * blockDim.x;
      if (wi < tb) {
        const int c = l0 + wi % lr, j = wi / lr;
        const int k = j % Ns;
        const int ob = (j / Ns) * Ns * R + k;
        C<T> *x = buf + c * ls;
        if (IsPow2<T, R>::value) {
          dif_pow2<T, R>(v[b], sg);
#pragma unroll
          for (int q = 0; q < R; q++) x[(ob + q * Ns) * es] = v[b][bitrev(q, ilog2(R))];
        } else {
          if (R == 3) dft3<T>(v[b], sg);
          else dft_odd<T, R>(v[b], w);
#pragma unroll
          for (int q = 0; q < R; q++) x[(ob + q * Ns) * es] = v[b][q];
        }
      }
    }
    __syncthreads();
  }
}

// a pass with a radix above the register limit: direct DFT from buf into a
// scratch of L lines (element i of line c at scr[i * L + c]), then copy back
template <typename T>
__device__ __noinline__ void pass_big(C<T> *buf, int es, int ls, int n, int L, int R, int Ns, const C<T> *__restrict__ tw,
                         bool inv, C<T> *scr)
{
  const int nb = n / R;
  const int twstep = n / (Ns * R);
  const int total = n * L;  // one output element per work item
  for (int wi = threadIdx.x; wi < total; wi += blockDim.x) {
    const int c = wi % L, rest = wi / L;
    const int j = rest % nb, q = rest / nb;
    const int k = j % Ns;
    const int ob = (j / Ns) * Ns * R + k;
    const C<T> *x = buf + c * ls;
    C<T> acc = x[j * es];
    int e = 0;
    for (int r = 1; r < R; r++) {
      e += q;
      if (e >= R) e -= R;
      C<T> t1 = tw[r * k * twstep], t2 = tw[e * nb];
      if (inv) { t1.y = -t1.y; t2.y = -t2.y; }
      acc = cadd<T>(acc, cmul<T>(cmul<T>(x[(j + r * nb) * es], t1), t2));
    }
    scr[(ob + q * Ns) * L + c] = acc;
  }
  __syncthreads();
  for (int wi = threadIdx.x; wi < total; wi += blockDim.x) {
    const int c = wi % L, i = wi / L;
    buf[c * ls + i * es] = scr[i * L + c];
  }
  __syncthreads();
}

template <typename T>
__device__ void fft_lines(C<T> *buf, int es, int ls, int L, const Stages &st, const C<T> *tw, bool inv, C<T> *scr)
{
  int Ns = 1;
  for (int s = 0; s < st.nst; s++) {
    const int R = st.radix[s];
    switch (R) {
      case 2: pass_reg<T, 2>(buf, es, ls, st.n, L, Ns, tw, inv); break;
      case 3: pass_reg<T, 3>(buf, es, ls, st.n, L, Ns, tw, inv); break;
      case 4: pass_reg<T, 4>(buf, es, ls, st.n, L, Ns, tw, inv); break;
      case 5: pass_reg<T, 5>(buf, es, ls, st.n, L, Ns, tw, inv); break;
      case 7: pass_reg<T, 7>(buf, es, ls, st.n, L, Ns, tw, inv); break;
      case 8: pass_reg<T, 8>(buf, es, ls, st.n, L, Ns, tw, inv); break;
      case 16: pass_reg<T, 16>(buf, es, ls, st.n, L, Ns, tw, inv); break;
      default: pass_big<T>(buf, es, ls, st.n, L, R, Ns, tw, inv, scr); break;
    }
    Ns *= R;
  }
}

// ---------------------------------------------------------------------------
// plane pass: one (block, z) plane of ny x nx in shared memory, rows stored
// with an odd stride nxp.
//   MODE 0: forward x then y, store to out
//   MODE 1: inverse y then x, epilogue out = a (kin + V phi) + b phi
// ---------------------------------------------------------------------------
template <typename T, int MODE>
__global__ void __launch_bounds__(1024, 1) k_fft_plane(const C<T> *__restrict__ in, C<T> *__restrict__ out, Stages sx,
                                                   Stages sy, const C<T> *__restrict__ twxg,
                                                   const C<T> *__restrict__ twyg, const C<T> *__restrict__ phi,
                                                   const T *__restrict__ pot, long ngrid, T ca, T cb)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nx = sx.n, ny = sy.n;
  const int nxp = nx | 1;
  const int npl = nx * ny;
  C<T> *twx = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *twy = twx + nx;
  C<T> *P = twy + ny;
  for (int t = threadIdx.x; t < nx; t += blockDim.x) twx[t] = twxg[t];
  for (int t = threadIdx.x; t < ny; t += blockDim.x) twy[t] = twyg[t];
  const long base = (long)blockIdx.x * npl;
#pragma unroll 8
  for (int t = threadIdx.x; t < npl; t += blockDim.x) P[(t / nx) * nxp + t % nx] = in[base + t];
  __syncthreads();
  if (MODE == 0) {
    fft_lines<T>(P, 1, nxp, ny, sx, twx, false, nullptr);  // rows
    fft_lines<T>(P, nxp, 1, nx, sy, twy, false, nullptr);  // columns
#pragma unroll 8
    for (int t = threadIdx.x; t < npl; t += blockDim.x) out[base + t] = P[(t / nx) * nxp + t % nx];
  } else {
    fft_lines<T>(P, nxp, 1, nx, sy, twy, true, nullptr);
    fft_lines<T>(P, 1, nxp, ny, sx, twx, true, nullptr);
#pragma unroll 8
    for (int t = threadIdx.x; t < npl; t += blockDim.x) {
      const long g = base + t;
      C<T> v = P[(t / nx) * nxp + t % nx];
      const C<T> ph = phi[g];
      if (pot) {
        const T V = pot[g % ngrid];
        v.x += V * ph.x;
        v.y += V * ph.y;
      }
      v.x = ca * v.x + cb * ph.x;
      v.y = ca * v.y + cb * ph.y;
      out[g] = v;
    }
  }
}

// ---------------------------------------------------------------------------
// x line pass (line path): L contiguous lines per CTA, line stride n|1.
// EPI = 1: fused out = a (kin + V phi) + b phi.
// ---------------------------------------------------------------------------
template <typename T, int EPI>
__global__ void __launch_bounds__(256, 4) k_fft_x(const C<T> *__restrict__ in, C<T> *__restrict__ out, Stages st,
                                               const C<T> *__restrict__ twg, long nlines, int L, bool inv,
                                               const C<T> *__restrict__ phi, const T *__restrict__ pot, long ngrid,
                                               T ca, T cb)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = st.n, np = n | 1;
  C<T> *tw = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *A = tw + n;
  C<T> *S = A + (long)L * np;  // scratch for a radix above the register limit
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];
  const long line0 = (long)blockIdx.x * L;
  const int nl = (int)min((long)L, nlines - line0);
  const long off = line0 * n;
#pragma unroll 8
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) A[(t / n) * np + t % n] = in[off + t];
  __syncthreads();
  fft_lines<T>(A, 1, np, nl, st, tw, inv, st.big ? S : nullptr);
#pragma unroll 8
  for (int t = threadIdx.x; t < nl * n; t += blockDim.x) {
    C<T> v = A[(t / n) * np + t % n];
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
template <typename T, bool KMUL>
__global__ void __launch_bounds__(256, 4) k_fft_cols(C<T> *__restrict__ data, Stages st, const C<T> *__restrict__ twg,
                                                  long es, int nxc, int TX, int nxt, long cnt, long s1, long s2,
                                                  bool inv, KinArgs ka)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = st.n;
  C<T> *tw = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *A = tw + n;
  C<T> *S = A + (long)TX * n;  // scratch for a radix above the register limit
  for (int t = threadIdx.x; t < n; t += blockDim.x) tw[t] = twg[t];
  const long o = blockIdx.x / nxt;
  const int xt = blockIdx.x % nxt;
  const int x0 = xt * TX;
  const int L = min(TX, nxc - x0);
  const long base = (o / cnt) * s1 + (o % cnt) * s2 + x0;
#pragma unroll 8
  for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
    const int cc = t % L, i = t / L;
    A[i * L + cc] = data[base + (long)i * es + cc];
  }
  __syncthreads();
  fft_lines<T>(A, L, 1, L, st, tw, KMUL ? false : inv, st.big ? S : nullptr);
  if (KMUL) {
    const int jy = (int)(o % cnt);
    if (ka.kq) {
      // convolution: multiply by the k-space array (hartree, bse_cplx/hartree.c:19-27)
      for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
        const int cc = t % L, i = t / L;
        const double2 q = ka.kq[(long)i * ka.nxy + (long)jy * ka.nx + x0 + cc];
        A[t] = cmul<T>(A[t], mk<T>((T)q.x, (T)q.y));
      }
    } else {
      for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
        const int cc = t % L, i = t / L;
        A[t] = cscale<T>(A[t], kin_factor<T>(ka, x0 + cc, jy, i));
      }
    }
    __syncthreads();
    fft_lines<T>(A, L, 1, L, st, tw, true, st.big ? S : nullptr);
  }
#pragma unroll 8
  for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
    const int cc = t % L, i = t / L;
    data[base + (long)i * es + cc] = A[i * L + cc];
  }
}

}  // namespace fbse

#include "fft_fast.cuh"

namespace fbse {

template <typename T> static const T *pot_of(fbse_ctx *c);
template <> const float *pot_of<float>(fbse_ctx *c) { return c->pot32; }
template <> const double *pot_of<double>(fbse_ctx *c) { return c->pot64; }

static int cols_tile(int nx, int elem)
{
  const int t = elem <= 8 ? 32 : 16;
  return nx < t ? nx : t;
}

static int max_smem()
{
  static int v = -1;
  if (v < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) v = 48 * 1024;
  }
  return v;
}

template <typename T>
static int launch_x(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, bool inv, int epi, const C<T> *phi,
                    const T *pot, T ca, T cb)
{
  const AxisPlan &p = c->ax[0];
  const int n = p.n;
  const long nlines = nblk * c->ny * c->nz;
  Stages st = stages_of(p);
  int L = 32;
  while (L > 1 && (size_t)(n + (st.big ? 2L : 1L) * L * (n | 1)) * sizeof(C<T>) > (size_t)max_smem()) L /= 2;
  const size_t smem = (size_t)(n + (st.big ? 2L : 1L) * L * (n | 1)) * sizeof(C<T>);
  const long grid = (nlines + L - 1) / L;
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
static int launch_cols(fbse_ctx *c, C<T> *data, long nblk, int axis, bool inv, bool kmul,
                       const double2 *kq = nullptr)
{
  const AxisPlan &p = c->ax[axis];
  const int n = p.n;
  const int TX = cols_tile((int)c->nx, (int)sizeof(C<T>));
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
  Stages st = stages_of(p);
  const size_t smem = (size_t)(n + (st.big ? 2L : 1L) * TX * n) * sizeof(C<T>);
  if (smem > (size_t)max_smem()) return set_err(c, FBSE_ERR_UNSUPPORTED, "FFT axis too long for shared memory");
  const long grid = nouter * nxt;
  KinArgs ka{c->k2x, c->k2y, c->k2z, c->k2xf, c->k2yf, c->k2zf, c->kemax_scaled, kq, c->nx, c->nx * c->ny};
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

template <typename T> static size_t plane_smem(fbse_ctx *c)
{
  const long nx = c->nx, ny = c->ny;
  return (size_t)(nx + ny + (nx | 1) * ny) * sizeof(C<T>);
}

template <typename T>
static int launch_plane(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, int mode, const C<T> *phi, const T *pot,
                        T ca, T cb)
{
  const size_t smem = plane_smem<T>(c);
  const long grid = nblk * c->nz;
  Stages sx = stages_of(c->ax[0]), sy = stages_of(c->ax[1]);
  if (mode == 0) {
    FBSE_CUDA(c, cudaFuncSetAttribute(k_fft_plane<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_plane<T, 0><<<grid, 1024, smem, c->stream>>>(in, out, sx, sy, roots<T>(c->ax[0]), roots<T>(c->ax[1]),
                                                       nullptr, nullptr, c->ngrid, T(1), T(0));
  } else {
    FBSE_CUDA(c, cudaFuncSetAttribute(k_fft_plane<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_plane<T, 1><<<grid, 1024, smem, c->stream>>>(in, out, sx, sy, roots<T>(c->ax[0]), roots<T>(c->ax[1]), phi,
                                                       pot, c->ngrid, ca, cb);
  }
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

// ---------------------------------------------------------------------------
// register-resident kernels (fft_fast.cuh) for axes of 64, 128, 256 points;
// fbse_tuning.fft_kernels = 1 selects the mixed-radix kernels for every axis,
// = 2 the mixed-radix line passes
// ---------------------------------------------------------------------------
static bool fast_axis_ok(fbse_ctx *c, long n) { return c->tune.fft_kernels == 0 && (n == 64 || n == 128 || n == 256); }

template <typename T> static bool fast_plane_ok(fbse_ctx *c)
{
  if (c->tune.fft_kernels != 0 || c->nx != c->ny) return false;
  if (c->nx == 64) return fast::PlaneCfg<T, 64>::smem() <= (size_t)max_smem();
  if (c->nx == 128 && sizeof(C<T>) == 8) return fast::PlaneCfg<T, 128>::smem() <= (size_t)max_smem();
  return false;
}

template <typename T, int N>
static int launch_plane_fast_n(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, int mode, const C<T> *phi,
                               const T *pot, T ca, T cb)
{
  using Cfg = fast::PlaneCfg<T, N>;
  const size_t smem = Cfg::smem();
  const long grid = nblk * c->nz;
  const C<T> *rt = roots<T>(c->ax[0]);
  if (mode == 0) {
    FBSE_CUDA(c, cudaFuncSetAttribute(fast::k_plane_fast<T, N, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    fast::k_plane_fast<T, N, 0><<<grid, Cfg::THREADS, smem, c->stream>>>(in, out, rt, nullptr, nullptr, c->ngrid,
                                                                          T(1), T(0));
  } else {
    FBSE_CUDA(c, cudaFuncSetAttribute(fast::k_plane_fast<T, N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    fast::k_plane_fast<T, N, 1><<<grid, Cfg::THREADS, smem, c->stream>>>(in, out, rt, phi, pot, c->ngrid, ca, cb);
  }
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

// the two-CTA cluster variant (fbse_tuning.fft_plane_cluster = 1) of the 128 x 128 FP32 plane
template <typename T, int N>
static int launch_plane_cl_n(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, int mode, const C<T> *phi,
                             const T *pot, T ca, T cb)
{
  using Cfg = fast::ClCfg<T, N>;
  const size_t smem = Cfg::smem();
  const long grid = 2 * nblk * c->nz;
  const C<T> *rt = roots<T>(c->ax[0]);
  if (mode == 0) {
    FBSE_CUDA(c, cudaFuncSetAttribute(fast::k_plane_cl<T, N, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fast::k_plane_cl<T, N, 0><<<grid, Cfg::THREADS, smem, c->stream>>>(in, out, rt, nullptr, nullptr, c->ngrid, T(1),
                                                                        T(0));
  } else {
    FBSE_CUDA(c, cudaFuncSetAttribute(fast::k_plane_cl<T, N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fast::k_plane_cl<T, N, 1><<<grid, Cfg::THREADS, smem, c->stream>>>(in, out, rt, phi, pot, c->ngrid, ca, cb);
  }
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <typename T>
static int launch_plane_fast(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, int mode, const C<T> *phi,
                             const T *pot, T ca, T cb)
{
  if (c->nx == 64) return launch_plane_fast_n<T, 64>(c, in, out, nblk, mode, phi, pot, ca, cb);
  if constexpr (sizeof(C<T>) == 8) {
    if (c->nx == 128 && c->tune.fft_plane_cluster == 1) return launch_plane_cl_n<T, 128>(c, in, out, nblk, mode, phi, pot, ca, cb);
  }
  if constexpr (sizeof(C<T>) == 8) {
    if (c->nx == 128) return launch_plane_fast_n<T, 128>(c, in, out, nblk, mode, phi, pot, ca, cb);
  }
  return set_err(c, FBSE_ERR_UNSUPPORTED, "no register-resident plane kernel for this size");
}

template <typename T, int N>
static int launch_cols_fast_n(fbse_ctx *c, C<T> *data, long nblk, int axis, bool inv, bool kmul, const double2 *kq)
{
  using Cfg = fast::ColsCfg<T, N>;
  const int nxt = (int)((c->nx + 31) / 32);
  long es, cnt, s1, s2, nouter;
  if (axis == 1) {
    es = c->nx; cnt = 1; s1 = c->nx * c->ny; s2 = 0; nouter = nblk * c->nz;
  } else {
    es = c->nx * c->ny; cnt = c->ny; s1 = c->ngrid; s2 = c->nx; nouter = nblk * c->ny;
  }
  const size_t smem = Cfg::smem();
  const long grid = nouter * nxt;
  const C<T> *rt = roots<T>(c->ax[axis]);
  KinArgs ka{c->k2x, c->k2y, c->k2z, c->k2xf, c->k2yf, c->k2zf, c->kemax_scaled, kq, c->nx, c->nx * c->ny};
  if (kmul) {
    FBSE_CUDA(c, cudaFuncSetAttribute(fast::k_cols_fast<T, N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    fast::k_cols_fast<T, N, true><<<grid, Cfg::THREADS, smem, c->stream>>>(data, rt, es, (int)c->nx, nxt, cnt, s1,
                                                                            s2, inv, ka);
  } else {
    FBSE_CUDA(c, cudaFuncSetAttribute(fast::k_cols_fast<T, N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
    fast::k_cols_fast<T, N, false><<<grid, Cfg::THREADS, smem, c->stream>>>(data, rt, es, (int)c->nx, nxt, cnt, s1,
                                                                             s2, inv, ka);
  }
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <typename T>
static int launch_cols_any(fbse_ctx *c, C<T> *data, long nblk, int axis, bool inv, bool kmul,
                           const double2 *kq = nullptr)
{
  switch (fast_axis_ok(c, c->ax[axis].n) ? c->ax[axis].n : 0) {
    case 64: return launch_cols_fast_n<T, 64>(c, data, nblk, axis, inv, kmul, kq);
    case 128: return launch_cols_fast_n<T, 128>(c, data, nblk, axis, inv, kmul, kq);
    case 256: return launch_cols_fast_n<T, 256>(c, data, nblk, axis, inv, kmul, kq);
    default: return launch_cols<T>(c, data, nblk, axis, inv, kmul, kq);
  }
}

int zpass_kinetic(fbse_ctx *c, float2 *data, long nblk)
{
  return launch_cols_any<float>(c, data, nblk, 2, false, true);
}

template <typename T, int N>
static int launch_x_fast_n(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, bool inv, int epi, const C<T> *phi,
                           const T *pot, T ca, T cb)
{
  using Cfg = fast::XCfg<T, N>;
  const long nlines = nblk * c->ny * c->nz;
  const size_t smem = Cfg::smem();
  const long grid = (nlines + Cfg::LINES - 1) / Cfg::LINES;
  const C<T> *rt = roots<T>(c->ax[0]);
  if (epi) {
    FBSE_CUDA(c, cudaFuncSetAttribute(fast::k_x_fast<T, N, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fast::k_x_fast<T, N, 1><<<grid, Cfg::THREADS, smem, c->stream>>>(in, out, rt, nlines, inv, phi, pot, c->ngrid,
                                                                      ca, cb);
  } else {
    FBSE_CUDA(c, cudaFuncSetAttribute(fast::k_x_fast<T, N, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    fast::k_x_fast<T, N, 0><<<grid, Cfg::THREADS, smem, c->stream>>>(in, out, rt, nlines, inv, nullptr, nullptr,
                                                                      c->ngrid, T(1), T(0));
  }
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <typename T>
static int launch_x_any(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, bool inv, int epi, const C<T> *phi,
                        const T *pot, T ca, T cb)
{
  switch (fast_axis_ok(c, c->nx) ? c->nx : 0) {
    case 64: return launch_x_fast_n<T, 64>(c, in, out, nblk, inv, epi, phi, pot, ca, cb);
    case 128: return launch_x_fast_n<T, 128>(c, in, out, nblk, inv, epi, phi, pot, ca, cb);
    case 256: return launch_x_fast_n<T, 256>(c, in, out, nblk, inv, epi, phi, pot, ca, cb);
    default: return launch_x<T>(c, in, out, nblk, inv, epi, phi, pot, ca, cb);
  }
}

// out = a (F^-1 K F in + V in) + b in with K = the capped kinetic factor, or
// the complex k-space array kq when given (then V is not applied); cb blocks
// per launch sequence
template <typename T>
static int fft_op_chunked(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *work, long nblk, double a, double b,
                          int with_v, const double2 *kq, long cb)
{
  int rc;
  const Stages sx = stages_of(c->ax[0]), sy = stages_of(c->ax[1]);
  const bool plane = !sx.big && !sy.big && plane_smem<T>(c) <= (size_t)max_smem() && c->tune.fft_kernels != 2;
  const T *pot = with_v ? pot_of<T>(c) : nullptr;
  const bool fplane = fast_plane_ok<T>(c);
  for (long b0 = 0; b0 < nblk; b0 += cb) {
    const long nb = (nblk - b0 < cb) ? nblk - b0 : cb;
    const C<T> *ci = in + b0 * c->ngrid;
    C<T> *co = out + b0 * c->ngrid;
    C<T> *wk = work;  // reused by every chunk: a chunk's intermediate passes can stay in L2
    if (fplane) {
      if ((rc = launch_plane_fast<T>(c, ci, wk, nb, 0, nullptr, nullptr, T(1), T(0)))) return rc;
      if ((rc = launch_cols_any<T>(c, wk, nb, 2, false, true, kq))) return rc;
      if ((rc = launch_plane_fast<T>(c, wk, co, nb, 1, ci, pot, (T)a, (T)b))) return rc;
    } else if (plane) {
      if ((rc = launch_plane<T>(c, ci, wk, nb, 0, nullptr, nullptr, T(1), T(0)))) return rc;
      if ((rc = launch_cols<T>(c, wk, nb, 2, false, true, kq))) return rc;
      if ((rc = launch_plane<T>(c, wk, co, nb, 1, ci, pot, (T)a, (T)b))) return rc;
    } else {
      if ((rc = launch_x_any<T>(c, ci, wk, nb, false, 0, nullptr, nullptr, T(1), T(0)))) return rc;
      if ((rc = launch_cols_any<T>(c, wk, nb, 1, false, false))) return rc;
      if ((rc = launch_cols_any<T>(c, wk, nb, 2, false, true, kq))) return rc;
      if ((rc = launch_cols_any<T>(c, wk, nb, 1, true, false))) return rc;
      if ((rc = launch_x_any<T>(c, wk, co, nb, true, 1, ci, pot, (T)a, (T)b))) return rc;
    }
  }
  return FBSE_OK;
}

// blocks per launch sequence: fixed by fbse_tuning.fft_chunk_blocks or
// autotuned (every block is transformed by the same kernels either way; a
// smaller chunk keeps its intermediate passes in L2, a larger one fills the
// GPU better)
template <typename T>
static int fft_op_apply(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *work, long nblk, double a, double b,
                        int with_v, const double2 *kq)
{
  long cb = c->tune.fft_chunk_blocks;
  if (cb == 0) {
    cb = nblk;
    if (nblk >= 4 && (const void *)in != (const void *)out) {
      std::vector<long> cands{nblk};
      for (long v : {16L, 8L, 4L, 2L})
        if (v < nblk) cands.push_back(v);
      const std::string prob = std::string(sizeof(T) == 4 ? "fp32" : "fp64") + " grid=" + std::to_string(c->nx) +
                               "x" + std::to_string(c->ny) + "x" + std::to_string(c->nz) +
                               " blocks=" + std::to_string(nblk) + (kq ? " convolution" : " kinetic");
      int rc = autotune(c, "fft blocks per launch", prob, cands,
                        [&](long v) { return fft_op_chunked<T>(c, in, out, work, nblk, a, b, with_v, kq, v); }, &cb);
      if (rc) return rc;
    }
  }
  return fft_op_chunked<T>(c, in, out, work, nblk, a, b, with_v, kq, cb < nblk ? cb : nblk);
}

template <typename T>
int kinetic_apply(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *work, long nblk, double a, double b, int with_v)
{
  return fft_op_apply<T>(c, in, out, work, nblk, a, b, with_v, nullptr);
}

template <typename T>
int conv_apply(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *work, long nblk, const double2 *kq)
{
  return fft_op_apply<T>(c, in, out, work, nblk, 1.0, 0.0, 0, kq);
}

// unnormalised forward 3D DFT of one FP64 block in place (FFTW_FORWARD of the
// reference's fftw_plan_dft_3d); work: one block of scratch
int forward_fft64(fbse_ctx *c, double2 *data, double2 *work)
{
  int rc;
  if ((rc = launch_x<double>(c, data, work, 1, false, 0, nullptr, nullptr, 1.0, 0.0))) return rc;
  if ((rc = launch_cols<double>(c, work, 1, 1, false, false))) return rc;
  if ((rc = launch_cols<double>(c, work, 1, 2, false, false))) return rc;
  FBSE_CUDA(c, cudaMemcpyAsync(data, work, c->ngrid * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream));
  return FBSE_OK;
}

template int conv_apply<float>(fbse_ctx *, const C<float> *, C<float> *, C<float> *, long, const double2 *);
template int conv_apply<double>(fbse_ctx *, const C<double> *, C<double> *, C<double> *, long, const double2 *);
template int kinetic_apply<float>(fbse_ctx *, const C<float> *, C<float> *, C<float> *, long, double, double, int);
template int kinetic_apply<double>(fbse_ctx *, const C<double> *, C<double> *, C<double> *, long, double, double, int);

}  // namespace fbse
