// In-register DFT helpers and the kinetic factor shared by the FFT kernels
// (fft.cu, fft_fast.cuh) and the fused H psi kernel (hpsi_pipe.cu).
#pragma once

#include "fbse_internal.cuh"

namespace fbse {

// ---------------------------------------------------------------------------
// in-register DFTs
// ---------------------------------------------------------------------------
// cos(2 pi m / 16), m = 0..15 (exact constants of the 16th roots of unity)
__host__ __device__ constexpr double c16(int m)
{
  return m == 0 ? 1.0 : m == 1 ? 0.92387953251128675613 : m == 2 ? 0.70710678118654752440
       : m == 3 ? 0.38268343236508977173 : m == 4 ? 0.0 : m == 5 ? -0.38268343236508977173
       : m == 6 ? -0.70710678118654752440 : m == 7 ? -0.92387953251128675613 : m == 8 ? -1.0
       : m == 9 ? -0.92387953251128675613 : m == 10 ? -0.70710678118654752440
       : m == 11 ? -0.38268343236508977173 : m == 12 ? 0.0 : m == 13 ? 0.38268343236508977173
       : m == 14 ? 0.70710678118654752440 : 0.92387953251128675613;
}
__host__ __device__ constexpr double s16(int m) { return c16((m + 12) & 15); }  // sin(2 pi m / 16)

__host__ __device__ constexpr int bitrev(int x, int bits)
{
  int r = 0;
  for (int i = 0; i < bits; i++) r |= ((x >> i) & 1) << (bits - 1 - i);
  return r;
}
__host__ __device__ constexpr int ilog2(int r) { return r <= 1 ? 0 : 1 + ilog2(r / 2); }

// radix-2 decimation in frequency on R = 2^k values; the result is left in
// bit-reversed order (the caller writes v[bitrev(q)] to output q)
template <typename T, int R>
__device__ __forceinline__ void dif_pow2(C<T> *v, T sg)
{
#pragma unroll
  for (int h = R / 2; h >= 1; h >>= 1) {
#pragma unroll
    for (int blk = 0; blk < R; blk += 2 * h) {
#pragma unroll
      for (int t = 0; t < h; t++) {
        const C<T> a = v[blk + t], b = v[blk + t + h];
        v[blk + t] = cadd<T>(a, b);
        const C<T> d = csub<T>(a, b);
        const int m = t * (16 / (2 * h));  // e^{sg 2 pi i t / (2h)} = 16th root m
        if (m == 0) {
          v[blk + t + h] = d;
        } else if (m == 4) {  // sg * i
          v[blk + t + h] = mk<T>(-sg * d.y, sg * d.x);
        } else {
          const T cr = (T)c16(m), ci = sg * (T)s16(m);
          v[blk + t + h] = mk<T>(d.x * cr - d.y * ci, d.x * ci + d.y * cr);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// kinetic factor of the z pass
// ---------------------------------------------------------------------------
struct KinArgs {
  const double *k2x, *k2y, *k2z;
  const float *k2xf, *k2yf, *k2zf;  // FP32 copies: the mixed path's factor is formed in FP32
  double kemax;
  const double2 *kq;  // when set: multiply by this complex k-space array instead
  long nx, nxy;
};

// min(0.5 k^2, KE_max) / N from the per-axis tables, in the working precision
template <typename T> __device__ __forceinline__ T kin_factor(const KinArgs &ka, int x, int y, int z);
template <> __device__ __forceinline__ double kin_factor<double>(const KinArgs &ka, int x, int y, int z)
{
  const double kk = ka.k2x[x] + ka.k2y[y] + ka.k2z[z];
  return kk > ka.kemax ? ka.kemax : kk;
}
template <> __device__ __forceinline__ float kin_factor<float>(const KinArgs &ka, int x, int y, int z)
{
  const float kk = ka.k2xf[x] + ka.k2yf[y] + ka.k2zf[z];
  const float cap = (float)ka.kemax;
  return kk > cap ? cap : kk;
}

}  // namespace fbse
