// Register-resident FFT kernels for axis lengths n = Q * P with P threads per
// line and Q values per thread (n = 64, 128, 256).  Included by fft.cu only.
//
// Decomposition (n = t + P m, k = k1 + Q k2):
//   X[k1 + Q k2] = sum_t w_P^{t k2} [ w_n^{t k1} sum_m x[t + P m] w_Q^{m k1} ]
// Thread t of a line holds x[t + P m] (m < Q), computes the Q-point DFT over
// m and the twiddle w_n^{t k1} in registers, one exchange through shared
// memory hands thread t the values of k1 = t + P j (j < Q / P) from all P
// threads, and a P-point DFT per k1 gives X[k1 + Q k2].  The inverse of that
// output distribution runs the other way round (P-point DFTs first, one
// exchange, Q-point DFTs) and ends with thread t holding x[t + P m] again, so
// forward - multiply - inverse needs two exchanges and no reordering.
#pragma once

namespace fbse {
namespace fast {

template <int N> struct Shape { static constexpr bool ok = false; static constexpr int P = 1, Q = 1; };
template <> struct Shape<64> { static constexpr bool ok = true; static constexpr int P = 8, Q = 8; };
template <> struct Shape<128> { static constexpr bool ok = true; static constexpr int P = 8, Q = 16; };
template <> struct Shape<256> { static constexpr bool ok = true; static constexpr int P = 16, Q = 16; };

// natural-order DFT of R = 2^k values in registers, sign sg
template <typename T, int R>
__device__ __forceinline__ void dft_nat(C<T> *v, T sg)
{
  dif_pow2<T, R>(v, sg);
  C<T> o[R];
#pragma unroll
  for (int q = 0; q < R; q++) o[q] = v[bitrev(q, ilog2(R))];
#pragma unroll
  for (int q = 0; q < R; q++) v[q] = o[q];
}

// tw2[k1 * P + t] = w_n^{t k1} = roots[(t k1) mod n] (forward sign)
template <typename T, int N>
__device__ __forceinline__ void load_tw2(C<T> *tw2, const C<T> *__restrict__ roots)
{
  constexpr int P = Shape<N>::P;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw2[i] = roots[((i % P) * (i / P)) % N];
}

template <typename T>
__device__ __forceinline__ C<T> twid(const C<T> *tw2, int i, bool inv)
{
  C<T> w = tw2[i];
  if (inv) w.y = -w.y;
  return w;
}

// forward decomposition, first half: v[m] = x[t + P m] -> v[k1] = Y_t[k1]
template <typename T, int N, bool INV>
__device__ __forceinline__ void inner_q(C<T> *v, int t, const C<T> *tw2)
{
  constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
  dft_nat<T, Q>(v, INV ? T(1) : T(-1));
#pragma unroll
  for (int k1 = 1; k1 < Q; k1++) v[k1] = cmul<T>(v[k1], twid<T>(tw2, k1 * P + t, INV));
}

// forward decomposition, second half: u[j][s] = Y_s[t + P j] -> v[j P + k2] = X[t + P j + Q k2]
template <typename T, int N, bool INV>
__device__ __forceinline__ void outer_p(C<T> *v)
{
  constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
#pragma unroll
  for (int j = 0; j < Q / P; j++) dft_nat<T, P>(v + j * P, INV ? T(1) : T(-1));
}

// transposed decomposition, first half: v[j P + k2] = X[t + P j + Q k2] ->
// v[j P + n2] = V[k1 = t + P j][n2] (P-point DFTs over k2, then w_n^{n2 k1})
template <typename T, int N, bool INV>
__device__ __forceinline__ void tinner_p(C<T> *v, int t, const C<T> *tw2)
{
  constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
#pragma unroll
  for (int j = 0; j < Q / P; j++) {
    dft_nat<T, P>(v + j * P, INV ? T(1) : T(-1));
#pragma unroll
    for (int n2 = 1; n2 < P; n2++) v[j * P + n2] = cmul<T>(v[j * P + n2], twid<T>(tw2, (t + P * j) * P + n2, INV));
  }
}

// transposed decomposition, second half: v[k1] = V[k1][t] -> v[n1] = x[t + P n1]
template <typename T, int N, bool INV>
__device__ __forceinline__ void touter_q(C<T> *v)
{
  dft_nat<T, Shape<N>::Q>(v, INV ? T(1) : T(-1));
}

// ---------------------------------------------------------------------------
// plane pass (nx = ny = N): rows with P threads per row and a warp-local
// exchange in the row's own shared-memory slots, then columns with lanes on
// consecutive x and the P threads of a column in P different warps.
//   MODE 0: forward x then y;  MODE 1: inverse y then x, epilogue
//   out = a (result + V phi) + b phi
// Row slots: row r at P[r * PITCH], slot (k1, s) at k1 * P + (s ^ (k1 & (P-1))).
// ---------------------------------------------------------------------------
template <typename T, int N> struct PlaneCfg {
  static constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
  static constexpr int PITCH = N + 8;
  static constexpr int THREADS = N * P;
  static constexpr size_t smem() { return (size_t)(N + N * PITCH + (N == 128 && sizeof(T) == 4 ? 128 : 0)) * sizeof(C<T>); }
};

template <typename T, int N>
__device__ __forceinline__ void row_exchange(C<T> *row, C<T> *v, int t)
{
  constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
#pragma unroll
  for (int k1 = 0; k1 < Q; k1++) row[k1 * P + (t ^ (k1 & (P - 1)))] = v[k1];
  __syncwarp();
#pragma unroll
  for (int j = 0; j < Q / P; j++) {
    const int k1 = t + P * j;
#pragma unroll
    for (int s = 0; s < P; s++) v[j * P + s] = row[k1 * P + (s ^ (k1 & (P - 1)))];
  }
  __syncwarp();
}

// the transposed exchange: thread t holds V[t + P j][n2]; afterwards v[k1] = V[k1][t]
template <typename T, int N>
__device__ __forceinline__ void row_texchange(C<T> *row, C<T> *v, int t)
{
  constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
#pragma unroll
  for (int j = 0; j < Q / P; j++) {
    const int k1 = t + P * j;
#pragma unroll
    for (int s = 0; s < P; s++) row[k1 * P + (s ^ (k1 & (P - 1)))] = v[j * P + s];
  }
  __syncwarp();
#pragma unroll
  for (int k1 = 0; k1 < Q; k1++) v[k1] = row[k1 * P + (t ^ (k1 & (P - 1)))];
  __syncwarp();
}

// ---------------------------------------------------------------------------
// FP32 128-point rows as two 64-point transforms (even / odd split), so that
// each of the 8 threads of a row moves adjacent complex pairs with 16-byte
// accesses (x[2i], x[2i+1] with i = t + 8 m), half the global instructions
// of the direct 128-point decomposition.  With w = e^{-2 pi i / 128}:
//   forward: E, O = 64-point DFTs of x[2i], x[2i+1];
//            X[k] = E[k] + w^k O[k], X[k + 64] = E[k] - w^k O[k]
//   inverse: A[k] = X[k] + X[k + 64], B[k] = (X[k] - X[k + 64]) w^-k;
//            x[2i] = A'[i], x[2i+1] = B'[i] (64-point inverse DFTs)
// Tables in shared memory: tw64[k1 * 8 + t] = w^{2 t k1}, wk[k] = w^k (k < 64).
// ---------------------------------------------------------------------------
template <typename T, int N> struct SplitRows {
  static constexpr bool on = (N == 128 && sizeof(T) == 4);
  static constexpr int extra = on ? 128 : 0;  // complex table entries
};

__device__ __forceinline__ void load_split_tables(float2 *tw64, float2 *wk, const float2 *__restrict__ roots)
{
  for (int i = threadIdx.x; i < 64; i += blockDim.x) {
    tw64[i] = roots[(2 * (i % 8) * (i / 8)) % 128];
    wk[i] = roots[i];
  }
}

// forward row: xin = the row in global memory, row = its shared slots; X in
// natural order into row[0, 128)
__device__ __forceinline__ void row128_fwd(const float2 *__restrict__ xin, float2 *row, int t, const float2 *tw64,
                                          const float2 *wk)
{
  float2 e[8], o[8];
  const float4 *src = reinterpret_cast<const float4 *>(xin);
#pragma unroll
  for (int m = 0; m < 8; m++) {
    const float4 q = src[t + 8 * m];
    e[m] = make_float2(q.x, q.y);
    o[m] = make_float2(q.z, q.w);
  }
  inner_q<float, 64, false>(e, t, tw64);
  inner_q<float, 64, false>(o, t, tw64);
  row_exchange<float, 64>(row, e, t);
  row_exchange<float, 64>(row + 64, o, t);
  outer_p<float, 64, false>(e);
  outer_p<float, 64, false>(o);
#pragma unroll
  for (int k2 = 0; k2 < 8; k2++) {
    const int k = t + 8 * k2;
    const float2 wo = cmul<float>(o[k2], wk[k]);
    row[k] = cadd<float>(e[k2], wo);
    row[k + 64] = csub<float>(e[k2], wo);
  }
}

// inverse row from row[0, 128) (natural order): a[k2] = x[2 i], b[k2] =
// x[2 i + 1] with i = t + 8 k2 (the row's shared slots are reused)
__device__ __forceinline__ void row128_inv(float2 *row, int t, const float2 *tw64, const float2 *wk, float2 *a,
                                          float2 *b)
{
#pragma unroll
  for (int m = 0; m < 8; m++) {
    const int k = t + 8 * m;
    const float2 x0 = row[k], x1 = row[k + 64];
    a[m] = cadd<float>(x0, x1);
    b[m] = cmulc<float>(csub<float>(x0, x1), wk[k], true);
  }
  __syncwarp();
  inner_q<float, 64, true>(a, t, tw64);
  inner_q<float, 64, true>(b, t, tw64);
  row_exchange<float, 64>(row, a, t);
  row_exchange<float, 64>(row + 64, b, t);
  outer_p<float, 64, true>(a);
  outer_p<float, 64, true>(b);
}

// out[2i, 2i+1] = ca (x + V phi) + cb phi for the pairs of a row (16-byte
// accesses; V as float2 pairs)
__device__ __forceinline__ void row128_epilogue(const float2 *a, const float2 *b, int t,
                                               const float2 *__restrict__ phi, const float *__restrict__ pot,
                                               float2 *__restrict__ out, float ca, float cb)
{
  const float4 *ph4 = reinterpret_cast<const float4 *>(phi);
  const float2 *v2 = reinterpret_cast<const float2 *>(pot);
  float4 *o4 = reinterpret_cast<float4 *>(out);
#pragma unroll
  for (int k2 = 0; k2 < 8; k2++) {
    const int i = t + 8 * k2;
    const float4 ph = ph4[i];
    float2 r0 = a[k2], r1 = b[k2];
    if (pot) {
      const float2 V = v2[i];
      r0.x += V.x * ph.x;
      r0.y += V.x * ph.y;
      r1.x += V.y * ph.z;
      r1.y += V.y * ph.w;
    }
    o4[i] = make_float4(ca * r0.x + cb * ph.x, ca * r0.y + cb * ph.y, ca * r1.x + cb * ph.z, ca * r1.y + cb * ph.w);
  }
}

template <typename T, int N, int MODE>
__global__ void __launch_bounds__(PlaneCfg<T, N>::THREADS, 1)
    k_plane_fast(const C<T> *__restrict__ in, C<T> *__restrict__ out, const C<T> *__restrict__ roots,
                 const C<T> *__restrict__ phi, const T *__restrict__ pot, long ngrid, T ca, T cb)
{
  using Cfg = PlaneCfg<T, N>;
  constexpr int P = Cfg::P, Q = Cfg::Q, PITCH = Cfg::PITCH;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C<T> *tw2 = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *S = tw2 + N;
  constexpr bool SPLIT = SplitRows<T, N>::on;
  C<T> *tws = S + N * PITCH;  // SPLIT: tw64[64], wk[64]
  load_tw2<T, N>(tw2, roots);
  if constexpr (SPLIT) load_split_tables(tws, tws + 64, roots);
  const long base = (long)blockIdx.x * N * N;
  const int rr = threadIdx.x / P, rt = threadIdx.x % P;  // row phase: row, thread in row
  const int cw = threadIdx.x >> 5;
  const int ct = cw % P, cc = (cw / P) * 32 + (threadIdx.x & 31);  // column phase: thread in column, column
  C<T> v[Q];
  __syncthreads();
  if (MODE == 0) {
    // rows, forward
    C<T> *row = S + rr * PITCH;
    if constexpr (SPLIT) {
      row128_fwd(in + base + (long)rr * N, row, rt, tws, tws + 64);
    } else {
#pragma unroll
      for (int m = 0; m < Q; m++) v[m] = in[base + (long)rr * N + rt + P * m];
      inner_q<T, N, false>(v, rt, tw2);
      row_exchange<T, N>(row, v, rt);
      outer_p<T, N, false>(v);
#pragma unroll
      for (int j = 0; j < Q / P; j++)
#pragma unroll
        for (int k2 = 0; k2 < P; k2++) row[rt + P * j + Q * k2] = v[j * P + k2];
    }
    __syncthreads();
    // columns, forward
#pragma unroll
    for (int m = 0; m < Q; m++) v[m] = S[(ct + P * m) * PITCH + cc];
    inner_q<T, N, false>(v, ct, tw2);
    __syncthreads();
#pragma unroll
    for (int k1 = 0; k1 < Q; k1++) S[(k1 * P + ct) * PITCH + cc] = v[k1];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int s = 0; s < P; s++) v[j * P + s] = S[((ct + P * j) * P + s) * PITCH + cc];
    outer_p<T, N, false>(v);
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int k2 = 0; k2 < P; k2++) out[base + (long)(ct + P * j + Q * k2) * N + cc] = v[j * P + k2];
  } else {
    // columns, inverse
#pragma unroll
    for (int m = 0; m < Q; m++) v[m] = in[base + (long)(ct + P * m) * N + cc];
    inner_q<T, N, true>(v, ct, tw2);
#pragma unroll
    for (int k1 = 0; k1 < Q; k1++) S[(k1 * P + ct) * PITCH + cc] = v[k1];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int s = 0; s < P; s++) v[j * P + s] = S[((ct + P * j) * P + s) * PITCH + cc];
    outer_p<T, N, true>(v);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int k2 = 0; k2 < P; k2++) S[(ct + P * j + Q * k2) * PITCH + cc] = v[j * P + k2];
    __syncthreads();
    // rows, inverse, with the epilogue (a plane lies inside one block: one
    // modulo gives its offset in the potential)
    const long pbase = base % ngrid;
    C<T> *row = S + rr * PITCH;
    if constexpr (SPLIT) {
      C<T> a[8], b[8];
      row128_inv(row, rt, tws, tws + 64, a, b);
      const long o = (long)rr * N;
      row128_epilogue(a, b, rt, phi + base + o, pot ? pot + pbase + o : nullptr, out + base + o, ca, cb);
    } else {
#pragma unroll
      for (int m = 0; m < Q; m++) v[m] = row[rt + P * m];
      __syncwarp();
      inner_q<T, N, true>(v, rt, tw2);
      row_exchange<T, N>(row, v, rt);
      outer_p<T, N, true>(v);
#pragma unroll
      for (int j = 0; j < Q / P; j++)
#pragma unroll
        for (int k2 = 0; k2 < P; k2++) {
          const long o = (long)rr * N + rt + P * j + Q * k2;
          const long g = base + o;
          C<T> r = v[j * P + k2];
          const C<T> ph = phi[g];
          if (pot) {
            const T V = pot[pbase + o];
            r.x += V * ph.x;
            r.y += V * ph.y;
          }
          out[g] = mk<T>(ca * r.x + cb * ph.x, ca * r.y + cb * ph.y);
        }
    }
  }
}

// ---------------------------------------------------------------------------
// column pass over lines of stride es (y or z): a tile of 32 consecutive x
// columns, P warps, warp t holds rows t + P m of its lane's column.
//   KMUL false: one direction;  KMUL true: forward, kinetic factor (or the
//   complex k-space array kq), inverse -- two exchanges.
// Tile o: base = (o / cnt) * s1 + (o % cnt) * s2 + 32 xt.
// ---------------------------------------------------------------------------
template <typename T, int N> struct ColsCfg {
  static constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
  static constexpr int THREADS = 32 * P;
  // FP32 with 8 warps: ask for 3 CTAs per SM (24 warps) instead of the 2 that
  // the unconstrained register count allows
  static constexpr int MINB = (sizeof(T) == 4 && THREADS == 256) ? 3 : 1;
  static constexpr size_t smem() { return (size_t)(N + 32 * N) * sizeof(C<T>); }
};

template <typename T, int N, bool KMUL>
__global__ void __launch_bounds__(ColsCfg<T, N>::THREADS, ColsCfg<T, N>::MINB)
    k_cols_fast(C<T> *__restrict__ data, const C<T> *__restrict__ roots, long es, int nxc, int nxt, long cnt,
                long s1, long s2, bool inv, KinArgs ka)
{
  constexpr int P = ColsCfg<T, N>::P, Q = ColsCfg<T, N>::Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C<T> *tw2 = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *S = tw2 + N;  // S[row * 32 + lane]
  load_tw2<T, N>(tw2, roots);
  const long o = blockIdx.x / nxt;
  const int x0 = (blockIdx.x % nxt) * 32;
  const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
  const bool act = x0 + lane < nxc;
  const long base = (o / cnt) * s1 + (o % cnt) * s2 + x0 + lane;
  C<T> v[Q];
  __syncthreads();
#pragma unroll
  for (int m = 0; m < Q; m++) v[m] = act ? data[base + (long)(t + P * m) * es] : mk<T>(T(0), T(0));
  const bool fi = KMUL ? false : inv;
  if (fi) inner_q<T, N, true>(v, t, tw2);
  else inner_q<T, N, false>(v, t, tw2);
#pragma unroll
  for (int k1 = 0; k1 < Q; k1++) S[(k1 * P + t) * 32 + lane] = v[k1];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < Q / P; j++)
#pragma unroll
    for (int s = 0; s < P; s++) v[j * P + s] = S[((t + P * j) * P + s) * 32 + lane];
  if (fi) outer_p<T, N, true>(v);
  else outer_p<T, N, false>(v);
  if (KMUL) {
    const int jy = (int)(o % cnt);
    const int x = act ? x0 + lane : x0;
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int k2 = 0; k2 < P; k2++) {
        const int k = t + P * j + Q * k2;
        if (ka.kq) {
          // convolution: multiply by the k-space array (hartree, bse_cplx/hartree.c:19-27)
          const double2 q = ka.kq[(long)k * ka.nxy + (long)jy * ka.nx + x];
          v[j * P + k2] = cmul<T>(v[j * P + k2], mk<T>((T)q.x, (T)q.y));
        } else {
          v[j * P + k2] = cscale<T>(v[j * P + k2], kin_factor<T>(ka, x, jy, k));
        }
      }
    tinner_p<T, N, true>(v, t, tw2);
    // slots (k1, n2) of this thread's own k1 rows: no other thread reads them before the barrier
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int n2 = 0; n2 < P; n2++) S[((t + P * j) * P + n2) * 32 + lane] = v[j * P + n2];
    __syncthreads();
#pragma unroll
    for (int k1 = 0; k1 < Q; k1++) v[k1] = S[(k1 * P + t) * 32 + lane];
    touter_q<T, N, true>(v);
    if (act) {
#pragma unroll
      for (int m = 0; m < Q; m++) data[base + (long)(t + P * m) * es] = v[m];
    }
  } else if (act) {
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int k2 = 0; k2 < P; k2++) data[base + (long)(t + P * j + Q * k2) * es] = v[j * P + k2];
  }
}

// ---------------------------------------------------------------------------
// x line pass: 256 threads, 256 / P contiguous lines per CTA, warp-local
// exchange in per-line slots (line stride N + 8).  EPI: inverse with the
// epilogue out = a (result + V phi) + b phi.
// ---------------------------------------------------------------------------
template <typename T, int N> struct XCfg {
  static constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
  static constexpr int THREADS = 256, LINES = THREADS / P, PITCH = N + 8;
  static constexpr size_t smem() { return (size_t)(N + LINES * PITCH) * sizeof(C<T>); }
};

template <typename T, int N, int EPI>
__global__ void __launch_bounds__(256)
    k_x_fast(const C<T> *__restrict__ in, C<T> *__restrict__ out, const C<T> *__restrict__ roots, long nlines,
             bool inv, const C<T> *__restrict__ phi, const T *__restrict__ pot, long ngrid, T ca, T cb)
{
  using Cfg = XCfg<T, N>;
  constexpr int P = Cfg::P, Q = Cfg::Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C<T> *tw2 = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *S = tw2 + N;
  load_tw2<T, N>(tw2, roots);
  __syncthreads();
  const int li = threadIdx.x / P, t = threadIdx.x % P;
  const long line = (long)blockIdx.x * Cfg::LINES + li;
  const bool act = line < nlines;  // a tail line repeats line 0 and stores nothing
  const long off = (act ? line : 0) * N;
  const long pbase = EPI == 1 ? off % ngrid : 0;  // a line lies inside one block
  C<T> v[Q];
#pragma unroll
  for (int m = 0; m < Q; m++) v[m] = in[off + t + P * m];
  C<T> *row = S + li * Cfg::PITCH;
  if (inv) {
    inner_q<T, N, true>(v, t, tw2);
    row_exchange<T, N>(row, v, t);
    outer_p<T, N, true>(v);
  } else {
    inner_q<T, N, false>(v, t, tw2);
    row_exchange<T, N>(row, v, t);
    outer_p<T, N, false>(v);
  }
#pragma unroll
  for (int j = 0; j < Q / P; j++)
#pragma unroll
    for (int k2 = 0; k2 < P; k2++) {
      const long o = t + P * j + Q * k2;
      const long g = off + o;
      C<T> r = v[j * P + k2];
      if (!act) continue;
      if (EPI == 1) {
        const C<T> ph = phi[g];
        if (pot) {
          const T V = pot[pbase + o];
          r.x += V * ph.x;
          r.y += V * ph.y;
        }
        r = mk<T>(ca * r.x + cb * ph.x, ca * r.y + cb * ph.y);
      }
      out[g] = r;
    }
}

}  // namespace fast
}  // namespace fbse

#include <cooperative_groups.h>

namespace fbse {
namespace fast {

// ---------------------------------------------------------------------------
// plane pass split over a cluster of two CTAs (two SMs), each holding half
// of the plane's rows in its shared memory: half the footprint of the
// one-CTA plane kernel, so two clusters share an SM and one's loads overlap
// the other's arithmetic.  Rows are transformed where they live; the column
// phase of CTA q covers columns [N/2 q, N/2 (q+1)) and reads the other half
// of each column from the partner's shared memory.
// ---------------------------------------------------------------------------
template <typename T, int N> struct ClCfg {
  static constexpr int P = Shape<N>::P, Q = Shape<N>::Q;
  static constexpr int HR = N / 2;                 // rows per CTA
  static constexpr int PITCH = N + 8;
  static constexpr int THREADS = HR * P;           // row phase: P threads per row
  static constexpr int CW = HR;                    // columns per CTA
  static constexpr size_t smem() { return (size_t)(N + HR * PITCH + SplitRows<T, N>::extra) * sizeof(C<T>); }
};

template <typename T, int N, int MODE>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(ClCfg<T, N>::THREADS, 2)
    k_plane_cl(const C<T> *__restrict__ in, C<T> *__restrict__ out, const C<T> *__restrict__ roots,
               const C<T> *__restrict__ phi, const T *__restrict__ pot, long ngrid, T ca, T cb)
{
  using Cfg = ClCfg<T, N>;
  constexpr int P = Cfg::P, Q = Cfg::Q, PITCH = Cfg::PITCH, HR = Cfg::HR, CW = Cfg::CW;
  namespace cgr = cooperative_groups;
  cgr::cluster_group cluster = cgr::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C<T> *tw2 = reinterpret_cast<C<T> *>(smem_raw);
  C<T> *H = tw2 + N;  // HR rows x PITCH; reused as the column slots S2[slot * CW + c]
  const unsigned q = cluster.block_rank();
  C<T> *const Hp = cluster.map_shared_rank(H, 1 - q);
  C<T> *const H0 = q == 0 ? H : Hp;  // rows [0, N/2)
  C<T> *const H1 = q == 0 ? Hp : H;  // rows [N/2, N)
  constexpr bool SPLIT = SplitRows<T, N>::on;
  C<T> *tws = H + HR * PITCH;  // SPLIT: tw64[64], wk[64]
  load_tw2<T, N>(tw2, roots);
  if constexpr (SPLIT) load_split_tables(tws, tws + 64, roots);
  const long base = (long)(blockIdx.x / 2) * N * N;
  const int rr = threadIdx.x / P, rt = threadIdx.x % P;        // row phase: local row, thread in row
  const int cw = threadIdx.x >> 5;
  const int ct = cw % P, cl = (cw / P) * 32 + (threadIdx.x & 31);  // column phase: thread in column, local column
  const int cgl = (int)q * CW + cl;                            // global column
  C<T> v[Q];
  __syncthreads();
  if (MODE == 0) {
    // rows N/2 q + rr, forward
    const long rbase = base + (long)((int)q * HR + rr) * N;
    C<T> *row = H + rr * PITCH;
    if constexpr (SPLIT) {
      row128_fwd(in + rbase, row, rt, tws, tws + 64);
    } else {
#pragma unroll
      for (int m = 0; m < Q; m++) v[m] = in[rbase + rt + P * m];
      inner_q<T, N, false>(v, rt, tw2);
      row_exchange<T, N>(row, v, rt);
      outer_p<T, N, false>(v);
#pragma unroll
      for (int j = 0; j < Q / P; j++)
#pragma unroll
        for (int k2 = 0; k2 < P; k2++) row[rt + P * j + Q * k2] = v[j * P + k2];
    }
    cluster.sync();
    // columns, forward: rows R = ct + P m from the CTA that holds them
#pragma unroll
    for (int m = 0; m < Q; m++) {
      const int R = ct + P * m;
      v[m] = (R < HR ? H0 : H1)[(R % HR) * PITCH + cgl];
    }
    inner_q<T, N, false>(v, ct, tw2);
    cluster.sync();  // the partner has read its half of every column
#pragma unroll
    for (int k1 = 0; k1 < Q; k1++) H[(k1 * P + ct) * CW + cl] = v[k1];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int s = 0; s < P; s++) v[j * P + s] = H[((ct + P * j) * P + s) * CW + cl];
    outer_p<T, N, false>(v);
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int k2 = 0; k2 < P; k2++) out[base + (long)(ct + P * j + Q * k2) * N + cgl] = v[j * P + k2];
  } else {
    // columns, inverse
#pragma unroll
    for (int m = 0; m < Q; m++) v[m] = in[base + (long)(ct + P * m) * N + cgl];
    inner_q<T, N, true>(v, ct, tw2);
#pragma unroll
    for (int k1 = 0; k1 < Q; k1++) H[(k1 * P + ct) * CW + cl] = v[k1];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int s = 0; s < P; s++) v[j * P + s] = H[((ct + P * j) * P + s) * CW + cl];
    outer_p<T, N, true>(v);
    cluster.sync();  // both CTAs are done with their column slots
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int k2 = 0; k2 < P; k2++) {
        const int R = ct + P * j + Q * k2;
        (R < HR ? H0 : H1)[(R % HR) * PITCH + cgl] = v[j * P + k2];
      }
    cluster.sync();
    // rows N/2 q + rr, inverse, with the epilogue
    const long o0 = (long)((int)q * HR + rr) * N;
    const long pbase = base % ngrid;
    C<T> *row = H + rr * PITCH;
    if constexpr (SPLIT) {
      C<T> a[8], b[8];
      row128_inv(row, rt, tws, tws + 64, a, b);
      row128_epilogue(a, b, rt, phi + base + o0, pot ? pot + pbase + o0 : nullptr, out + base + o0, ca, cb);
    } else {
#pragma unroll
      for (int m = 0; m < Q; m++) v[m] = row[rt + P * m];
      __syncwarp();
      inner_q<T, N, true>(v, rt, tw2);
      row_exchange<T, N>(row, v, rt);
      outer_p<T, N, true>(v);
#pragma unroll
      for (int j = 0; j < Q / P; j++)
#pragma unroll
        for (int k2 = 0; k2 < P; k2++) {
          const long o = o0 + rt + P * j + Q * k2;
          const long g = base + o;
          C<T> r = v[j * P + k2];
          const C<T> ph = phi[g];
          if (pot) {
            const T V = pot[pbase + o];
            r.x += V * ph.x;
            r.y += V * ph.y;
          }
          out[g] = mk<T>(ca * r.x + cb * ph.x, ca * r.y + cb * ph.y);
        }
    }
  }
}

}  // namespace fast
}  // namespace fbse
