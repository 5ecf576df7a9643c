// Batched mixed-radix 3D FFT for the kinetic term of H.
//
// Replaces kinetic() (filter_mpi/hamiltonian.c:62-99), i.e. FFTW's
// fftw_plan_dft_3d(nz, ny, nx) forward transform, the ksqr multiply and the
// unnormalised backward transform (plans made in filter_mpi/aux.c:259-270).
//
// Every axis is transformed by a self-sorting Stockham FFT in shared memory.
// The grid sizes the reference's auto-grid produces are arbitrary (e.g.
// 57 x 52 x 45 = 3*19 x 4*13 x 9*5), so each axis is factored into radix-4/2/3
// stages with hand-written butterflies plus generic odd-prime stages;
// twiddles and butterfly roots come from one table of n roots e^{-2 pi i t/n}
// per axis, computed on the host in extended precision.
//
// Plane path (an xy plane fits in shared memory, the usual case in FP32):
//   pass 1  per (block, z): load the plane, x then y forward, store
//   pass 2  z lines in tiles of 16 x-columns: forward, multiply by
//           min(kx^2 + ky^2 + kz^2 terms, KE_max)/N computed from the indices
//           exactly as filter_mpi/init.c:318-351 builds ksqr, inverse
//   pass 3  per (block, z): y then x inverse, fused epilogue
//           out = a (T psi + V psi) + b psi
// Line path (larger planes, FP64): x, y, z-fused, y, x passes.
// Blocks are processed in chunks sized so that a chunk's scratch stays in L2
// between the passes.
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
// A view of L lines of length n in shared memory: element i of line c sits at
// base[c * ls + i * es].
// ---------------------------------------------------------------------------
template <typename T> struct Lines {
  C<T> *base;
  int es, ls;
  __device__ __forceinline__ C<T> &at(int c, int i) const { return base[c * ls + i * es]; }
};

// One Stockham stage src -> dst over L lines.  ACROSS: consecutive threads
// take consecutive lines (column tiles), otherwise consecutive butterflies of
// one line.
template <typename T, bool ACROSS>
__device__ __forceinline__ void stage(Lines<T> src, Lines<T> dst, const C<T> *__restrict__ tw, int n, int L, int p,
                                      int Ns, bool inv)
{
  const int nb = n / p;
  const int total = nb * L;
  const int twstep = n / (Ns * p);
  const int rstep = nb;  // root index of e^{-2 pi i / p}
  const T sg = inv ? T(1) : T(-1);
  for (int w = threadIdx.x; w < total; w += blockDim.x) {
    int c, j;
    if (ACROSS) { c = w % L; j = w / L; }
    else { c = w / nb; j = w - c * nb; }
    const int k = j % Ns;
    const int ob = (j / Ns) * Ns * p + k;
    auto W = [&](int t) -> C<T> { C<T> r = tw[t]; if (inv) r.y = -r.y; return r; };
    if (p == 4) {
      C<T> v0 = src.at(c, j);
      C<T> v1 = cmul<T>(src.at(c, j + nb), W(k * twstep));
      C<T> v2 = cmul<T>(src.at(c, j + 2 * nb), W(2 * k * twstep));
      C<T> v3 = cmul<T>(src.at(c, j + 3 * nb), W(3 * k * twstep));
      C<T> a = cadd<T>(v0, v2), b = csub<T>(v0, v2), cc = cadd<T>(v1, v3), d = csub<T>(v1, v3);
      C<T> id = mk<T>(-sg * d.y, sg * d.x);  // s*i*d, s = -1 forward, +1 inverse
      dst.at(c, ob) = cadd<T>(a, cc);
      dst.at(c, ob + Ns) = cadd<T>(b, id);
      dst.at(c, ob + 2 * Ns) = csub<T>(a, cc);
      dst.at(c, ob + 3 * Ns) = csub<T>(b, id);
    } else if (p == 2) {
      C<T> v0 = src.at(c, j), v1 = cmul<T>(src.at(c, j + nb), W(k * twstep));
      dst.at(c, ob) = cadd<T>(v0, v1);
      dst.at(c, ob + Ns) = csub<T>(v0, v1);
    } else if (p == 3) {
      C<T> v0 = src.at(c, j);
      C<T> v1 = cmul<T>(src.at(c, j + nb), W(k * twstep));
      C<T> v2 = cmul<T>(src.at(c, j + 2 * nb), W(2 * k * twstep));
      const T h = T(0.86602540378443864676372317075293618);
      C<T> s12 = cadd<T>(v1, v2), d12 = csub<T>(v1, v2);
      C<T> t = mk<T>(v0.x - T(0.5) * s12.x, v0.y - T(0.5) * s12.y);
      C<T> iu = mk<T>(-sg * h * d12.y, sg * h * d12.x);  // i * s*(sqrt(3)/2)*(v1 - v2)
      dst.at(c, ob) = cadd<T>(v0, s12);
      dst.at(c, ob + Ns) = cadd<T>(t, iu);
      dst.at(c, ob + 2 * Ns) = csub<T>(t, iu);
    } else {
      // generic radix: twiddle this butterfly's inputs in place (each input
      // element of a stage is read by exactly one butterfly), then a direct
      // length-p DFT with roots from the table.
      for (int r = 1; r < p; r++) src.at(c, j + r * nb) = cmul<T>(src.at(c, j + r * nb), W(r * k * twstep));
      for (int q = 0; q < p; q++) {
        C<T> acc = src.at(c, j);
        int e = 0;
        for (int r = 1; r < p; r++) {
          e += q;
          if (e >= p) e -= p;
          acc = cadd<T>(acc, cmul<T>(src.at(c, j + r * nb), W(e * rstep)));
        }
        dst.at(c, ob + q * Ns) = acc;
      }
    }
  }
}

// transform L lines held in a using b as the other Stockham buffer; returns
// true when the result ended in b (odd number of stages)
template <typename T, bool ACROSS>
__device__ bool fft_lines(Lines<T> a, Lines<T> b, const C<T> *tw, const Stages &st, int L, bool inv)
{
  int Ns = 1;
  bool inb = false;
  for (int s = 0; s < st.nst; s++) {
    if (!inb) stage<T, ACROSS>(a, b, tw, st.n, L, st.radix[s], Ns, inv);
    else stage<T, ACROSS>(b, a, tw, st.n, L, st.radix[s], Ns, inv);
    __syncthreads();
    Ns *= st.radix[s];
    inb = !inb;
  }
  return inb;
}

// ---------------------------------------------------------------------------
// plane pass: one (block, z) plane of ny x nx in shared memory.
//   MODE 0: forward x then y, store to out
//   MODE 1: inverse y then x, epilogue out = a (kin + V phi) + b phi
// The rows / columns are transformed G at a time with a small scratch as the
// second Stockham buffer, so the plane itself needs no second copy.
// ---------------------------------------------------------------------------
template <typename T>
__device__ void plane_rows(C<T> *P, C<T> *S, const C<T> *tw, const Stages &st, int nx, int ny, int G, bool inv)
{
  for (int r0 = 0; r0 < ny; r0 += G) {
    const int g = min(G, ny - r0);
    Lines<T> a{P + r0 * nx, 1, nx}, b{S, 1, nx};
    const bool inb = fft_lines<T, false>(a, b, tw, st, g, inv);
    if (inb) {
      for (int t = threadIdx.x; t < g * nx; t += blockDim.x) P[r0 * nx + t] = S[t];
      __syncthreads();
    }
  }
}

template <typename T>
__device__ void plane_cols(C<T> *P, C<T> *S, const C<T> *tw, const Stages &st, int nx, int ny, int G, bool inv)
{
  for (int c0 = 0; c0 < nx; c0 += G) {
    const int g = min(G, nx - c0);
    Lines<T> a{P + c0, nx, 1}, b{S, g, 1};
    const bool inb = fft_lines<T, true>(a, b, tw, st, g, inv);
    if (inb) {
      for (int t = threadIdx.x; t < g * ny; t += blockDim.x) {
        const int cc = t % g, i = t / g;
        P[i * nx + c0 + cc] = S[i * g + cc];
      }
      __syncthreads();
    }
  }
}

template <typename T, int MODE>
__global__ void __launch_bounds__(512) k_fft_plane(const C<T> *__restrict__ in, C<T> *__restrict__ out, Stages sx,
                                                   Stages sy, const C<T> *__restrict__ twxg,
                                                   const C<T> *__restrict__ twyg, int G,
                                                   const C<T> *__restrict__ phi, const T *__restrict__ pot,
                                                   long ngrid, T ca, T cb)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nx = sx.n, ny = sy.n;
  const int npl = nx * ny;
  C<T> *twx = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *twy = twx + nx;
  C<T> *P = twy + ny;
  C<T> *S = P + npl;
  for (int t = threadIdx.x; t < nx; t += blockDim.x) twx[t] = twxg[t];
  for (int t = threadIdx.x; t < ny; t += blockDim.x) twy[t] = twyg[t];
  const long base = (long)blockIdx.x * npl;
  for (int t = threadIdx.x; t < npl; t += blockDim.x) P[t] = in[base + t];
  __syncthreads();
  if (MODE == 0) {
    plane_rows<T>(P, S, twx, sx, nx, ny, G, false);
    plane_cols<T>(P, S, twy, sy, nx, ny, G, false);
    for (int t = threadIdx.x; t < npl; t += blockDim.x) out[base + t] = P[t];
  } else {
    plane_cols<T>(P, S, twy, sy, nx, ny, G, true);
    plane_rows<T>(P, S, twx, sx, nx, ny, G, true);
    for (int t = threadIdx.x; t < npl; t += blockDim.x) {
      const long g = base + t;
      C<T> v = P[t];
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
// x line pass (line path): L contiguous lines per CTA.  EPI = 1: fused
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
  const bool inb = fft_lines<T, false>(Lines<T>{A, 1, n}, Lines<T>{B, 1, n}, tw, st, nl, inv);
  const C<T> *r = inb ? B : A;
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
  Lines<T> la{A, L, 1}, lb{B, L, 1};
  bool inb = fft_lines<T, true>(la, lb, tw, st, L, KMUL ? false : inv);
  if (KMUL) {
    C<T> *r = inb ? B : A;
    const int jy = (int)(o % cnt);
    const double ky = ka.k2y[jy];
    for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
      const int cc = t % L, i = t / L;
      double kk = ka.k2x[x0 + cc] + ky + ka.k2z[i];
      if (kk > ka.kemax) kk = ka.kemax;
      r[t] = cscale<T>(r[t], (T)kk);
    }
    __syncthreads();
    const bool inb2 = inb ? fft_lines<T, true>(lb, la, tw, st, L, true) : fft_lines<T, true>(la, lb, tw, st, L, true);
    inb = inb ? !inb2 : inb2;
  }
  const C<T> *r = inb ? B : A;
  for (int t = threadIdx.x; t < n * L; t += blockDim.x) {
    const int cc = t % L, i = t / L;
    data[base + (long)i * es + cc] = r[i * L + cc];
  }
}

template <typename T> static const T *pot_of(fbse_ctx *c);
template <> const float *pot_of<float>(fbse_ctx *c) { return c->pot32; }
template <> const double *pot_of<double>(fbse_ctx *c) { return c->pot64; }

static int cols_tile(int nx) { return nx < 16 ? nx : 16; }
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
  KinArgs ka{c->k2x, c->k2y, c->k2z, c->kemax_scaled};
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

// rows / columns per scratch group and the plane kernel's shared memory
template <typename T> static size_t plane_smem(fbse_ctx *c, int *G)
{
  const int nx = (int)c->nx, ny = (int)c->ny;
  *G = 16;
  const int mx = nx > ny ? nx : ny;
  return (size_t)(nx + ny + (long)nx * ny + (long)(*G) * mx) * sizeof(C<T>);
}

template <typename T>
static int launch_plane(fbse_ctx *c, const C<T> *in, C<T> *out, long nblk, int mode, const C<T> *phi, const T *pot,
                        T ca, T cb)
{
  int G;
  const size_t smem = plane_smem<T>(c, &G);
  const long grid = nblk * c->nz;
  Stages sx = stages_of(c->ax[0]), sy = stages_of(c->ax[1]);
  if (mode == 0) {
    FBSE_CUDA(c, cudaFuncSetAttribute(k_fft_plane<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_plane<T, 0><<<grid, 512, smem, c->stream>>>(in, out, sx, sy, roots<T>(c->ax[0]), roots<T>(c->ax[1]), G,
                                                       nullptr, nullptr, c->ngrid, T(1), T(0));
  } else {
    FBSE_CUDA(c, cudaFuncSetAttribute(k_fft_plane<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fft_plane<T, 1><<<grid, 512, smem, c->stream>>>(in, out, sx, sy, roots<T>(c->ax[0]), roots<T>(c->ax[1]), G,
                                                       phi, pot, c->ngrid, ca, cb);
  }
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

// blocks per chunk: keep a chunk's scratch (and its input) within L2
template <typename T> static long chunk_blocks(fbse_ctx *c, long nblk)
{
  const char *e = getenv("FBSE_FFT_CHUNK_BLOCKS");
  if (e && atol(e) > 0) return atol(e) < nblk ? atol(e) : nblk;
  const double blk = (double)c->ngrid * sizeof(C<T>);
  long cb = (long)(40.0e6 / blk);
  if (cb < 1) cb = 1;
  return cb < nblk ? cb : nblk;
}

template <typename T>
int kinetic_apply(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *work, long nblk, double a, double b, int with_v)
{
  int rc, G;
  const bool plane = plane_smem<T>(c, &G) <= (size_t)max_smem() && getenv("FBSE_FFT_LINES") == nullptr;
  const T *pot = with_v ? pot_of<T>(c) : nullptr;
  const long cb = chunk_blocks<T>(c, nblk);
  for (long b0 = 0; b0 < nblk; b0 += cb) {
    const long nb = (nblk - b0 < cb) ? nblk - b0 : cb;
    const C<T> *ci = in + b0 * c->ngrid;
    C<T> *co = out + b0 * c->ngrid;
    if (plane) {
      if ((rc = launch_plane<T>(c, ci, work, nb, 0, nullptr, nullptr, T(1), T(0)))) return rc;
      if ((rc = launch_cols<T>(c, work, nb, 2, false, true))) return rc;
      if ((rc = launch_plane<T>(c, work, co, nb, 1, ci, pot, (T)a, (T)b))) return rc;
    } else {
      if ((rc = launch_x<T>(c, ci, work, nb, false, 0, nullptr, nullptr, T(1), T(0)))) return rc;
      if ((rc = launch_cols<T>(c, work, nb, 1, false, false))) return rc;
      if ((rc = launch_cols<T>(c, work, nb, 2, false, true))) return rc;
      if ((rc = launch_cols<T>(c, work, nb, 1, true, false))) return rc;
      if ((rc = launch_x<T>(c, work, co, nb, true, 1, ci, pot, (T)a, (T)b))) return rc;
    }
  }
  return FBSE_OK;
}

template int kinetic_apply<float>(fbse_ctx *, const C<float> *, C<float> *, C<float> *, long, double, double, int);
template int kinetic_apply<double>(fbse_ctx *, const C<double> *, C<double> *, C<double> *, long, double, double, int);

}  // namespace fbse
