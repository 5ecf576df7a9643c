// Learned residual preconditioner and residual refinement (no counterpart in
// the reference, whose only remedy for unconverged states is to filter again
// with more starts and terms: retryFilter, filter_mpi/mod_output.c:131-147).
//
// Network (per real field f of a residual: the real or imaginary part of one
// spin block of r = (H - E) psi):
//   x0 = [f / rms(f), f / rms(f) * (V - E) / 1 Ha]          2 channels, BF16
//   a1 = tanh(W1 * x0), a2 = tanh(W2 * a1), a3 = tanh(W3 * a2)  16 channels, BF16
//   y  = W4 * a3                                               1 channel, FP32
//   correction = f + y * rms(f)       (residual connection: W4 = 0 gives f)
// "*" is a 3x3x3 convolution over the grid with zero padding and no bias, so
// the correction is an odd function of the residual.  Weights are FP32 in
// the layout [c_out][c_in][27] per layer, k = (dz * 3 + dy) * 3 + dx.
//
// Kernels: one convolution kernel serves the forward pass (tanh or linear
// epilogue) and the backward data pass (flipped, transposed weights; the
// epilogue multiplies by 1 - a^2 of the stored activation); a weight-gradient
// kernel accumulates dW over a fixed set of persistent CTAs (the tile -> CTA
// map does not depend on the device, so the sums are deterministic) and one
// kernel sums the CTAs' partials in order.  Arithmetic is FP32, partial sums of
// gradients and losses FP64.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "fbse_async.cuh"
#include "fbse_internal.cuh"

namespace fbse {

int pack_states(fbse_ctx *c, const double *src, void *dst, long nsrc);
int unpack_states(fbse_ctx *c, const void *src, double *dst, long ndst);
int ortho_diag_sigma(fbse_ctx *c, double *psitot, long n, long *n_kept, double *eval, double *sigma);
int normalize_all(fbse_ctx *c, double *psitot, long n, double *norms);

namespace pc {

constexpr int kC = 16;  // hidden channels
constexpr int kLayers = 4;
constexpr int kCin[kLayers] = {2, kC, kC, kC};
constexpr int kCout[kLayers] = {kC, kC, kC, 1};
constexpr long kWOff[kLayers + 1] = {0, 2 * kC * 27, 2 * kC * 27 + kC * kC * 27, 2 * kC * 27 + 2 * kC * kC * 27,
                                     2 * kC * 27 + 2 * kC * kC * 27 + kC * 27};
static_assert(kWOff[kLayers] == FBSE_PRECOND_NWEIGHTS, "weight count");
constexpr double kVScale = 1.0;  // (V - E) / 1 Ha

// output tile of the convolution kernels: 32 x 8 x 4 points, 256 threads, 4
// consecutive x points per thread
constexpr int TX = 32, TY = 8, TZ = 4, HX = TX + 2, HY = TY + 2, HZ = TZ + 2, HALO = HX * HY * HZ;
constexpr int kThreads = 256;
constexpr int kWgCtas = 512;  // persistent CTAs of the weight-gradient kernel

struct Geo {
  int nx, ny, nz;
  long n;  // nx * ny * nz
  int tx, ty, tz;  // tiles per axis
  int ntx, px;     // tensor-core path: 128-point x tiles, padded row length (see h8_index)
  __host__ __device__ long tiles() const { return (long)tx * ty * tz; }
};

// The inference path keeps the hidden activations channel-minor for the tensor
// cores: [field][channel half][z][y][x + 1][8 channels] in BF16, each row
// padded to ntx * 128 + 2 points with zeros at x = -1 and beyond nx, so that
// the 130 points a 128-point output tile needs are one contiguous,
// 16-byte-aligned run per channel half.
__host__ __device__ __forceinline__ long h8_index(const Geo &g, long f, int c, int z, int y, int x)
{
  return ((((f * 2 + c / 8) * g.nz + z) * g.ny + y) * (long)g.px + (x + 1)) * 8 + c % 8;
}

__device__ __forceinline__ float ld_f(const float *p) { return *p; }
__device__ __forceinline__ float ld_f(const __nv_bfloat16 *p) { return __bfloat162float(*p); }

// the halo of tile (tile) for channels [c0, c0 + cc) of field f into xs[cc][HALO]
template <typename TI, bool H8 = false>
__device__ void load_halo(const TI *__restrict__ in, int cin, long f, int c0, int cc, const Geo &g, int bx, int by,
                          int bz, float *xs)
{
  const int x0 = bx * TX - 1, y0 = by * TY - 1, z0 = bz * TZ - 1;
  for (int i = threadIdx.x; i < cc * HALO; i += blockDim.x) {
    const int ch = i / HALO, h = i % HALO;
    const int hx = h % HX, hy = (h / HX) % HY, hz = h / (HX * HY);
    const int x = x0 + hx, y = y0 + hy, z = z0 + hz;
    float v = 0.f;
    if (x >= 0 && x < g.nx && y >= 0 && y < g.ny && z >= 0 && z < g.nz)
      v = H8 ? ld_f(in + h8_index(g, f, c0 + ch, z, y, x))
             : ld_f(in + ((f * cin + c0 + ch) * g.n + ((long)z * g.ny + y) * g.nx + x));
    xs[i] = v;
  }
}

// out[f][co][p] = epi(sum_ci sum_k w[ci][k][co] in[f][ci][p + off_k])
// MODE 0: BF16 tanh(acc); 1: FP32 acc; 2: FP32 acc * (1 - a^2), a = act[f][co][p];
// 3: BF16 tanh(acc) in the channel-minor layout (h8_index).  H8: the input is
// in the channel-minor layout.
template <int CIN, int COUT, int MODE, typename TI, bool H8 = false>
__global__ void __launch_bounds__(kThreads) k_conv(const TI *__restrict__ in, const float *__restrict__ w, void *out,
                                                   const __nv_bfloat16 *__restrict__ act, Geo g)
{
  constexpr int CC = CIN < 4 ? CIN : 4;
  extern __shared__ float sm[];
  float *ws = sm;                      // [CIN][27][COUT]
  float *xs = sm + CIN * 27 * COUT;    // [CC][HALO]
  const long tile = blockIdx.x % g.tiles();
  const long f = blockIdx.x / g.tiles();
  const int bx = (int)(tile % g.tx), by = (int)((tile / g.tx) % g.ty), bz = (int)(tile / ((long)g.tx * g.ty));
  const int t = threadIdx.x, px = (t % 8) * 4, py = (t / 8) % 8, pz = t / 64;
  for (int i = t; i < CIN * 27 * COUT; i += kThreads) ws[i] = w[i];
  float acc[4][COUT];
#pragma unroll
  for (int q = 0; q < 4; q++)
#pragma unroll
    for (int o = 0; o < COUT; o++) acc[q][o] = 0.f;
  for (int c0 = 0; c0 < CIN; c0 += CC) {
    __syncthreads();
    load_halo<TI, H8>(in, CIN, f, c0, CC, g, bx, by, bz, xs);
    __syncthreads();
#pragma unroll 1
    for (int cc = 0; cc < CC; cc++) {
#pragma unroll
      for (int kz = 0; kz < 3; kz++)
#pragma unroll
        for (int ky = 0; ky < 3; ky++) {
          const float *row = xs + cc * HALO + ((pz + kz) * HY + (py + ky)) * HX + px;
          float r[6];
#pragma unroll
          for (int q = 0; q < 6; q++) r[q] = row[q];
#pragma unroll
          for (int kx = 0; kx < 3; kx++) {
            const float *wk = ws + ((c0 + cc) * 27 + (kz * 3 + ky) * 3 + kx) * COUT;
#pragma unroll
            for (int o = 0; o < COUT; o++) {
              const float wv = wk[o];
#pragma unroll
              for (int q = 0; q < 4; q++) acc[q][o] = fmaf(wv, r[q + kx], acc[q][o]);
            }
          }
        }
    }
  }
  const int z = bz * TZ + pz, y = by * TY + py;
  if (z >= g.nz || y >= g.ny) return;
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const int x = bx * TX + px + q;
    if (x >= g.nx) continue;
    const long p = ((long)z * g.ny + y) * g.nx + x;
#pragma unroll
    for (int o = 0; o < COUT; o++) {
      const long e = (f * COUT + o) * g.n + p;
      if (MODE == 0) {
        reinterpret_cast<__nv_bfloat16 *>(out)[e] = __float2bfloat16(tanhf(acc[q][o]));
      } else if (MODE == 3) {
        reinterpret_cast<__nv_bfloat16 *>(out)[h8_index(g, f, o, z, y, x)] = __float2bfloat16(tanhf(acc[q][o]));
      } else if (MODE == 1) {
        reinterpret_cast<float *>(out)[e] = acc[q][o];
      } else {
        const float a = __bfloat162float(act[e]);
        reinterpret_cast<float *>(out)[e] = acc[q][o] * (1.f - a * a);
      }
    }
  }
}

// partial dW[co][ci][k] = sum over this CTA's tiles of dy[f][co][p] x[f][ci][p + off_k];
// CTA b takes tiles b, b + gridDim.x, ... of all fields (a fixed order)
template <int CIN, int COUT, typename TI>
__global__ void __launch_bounds__(kThreads) k_conv_wgrad(const TI *__restrict__ x, const float *__restrict__ dy,
                                                         Geo g, long nf, double *__restrict__ part)
{
  constexpr int NO = COUT * CIN * 27;
  constexpr int PER = (NO + kThreads - 1) / kThreads;
  constexpr int DYS = TX * TY * TZ + 1;  // padded row: lanes with different c_out hit different banks
  extern __shared__ float sm[];
  float *xs = sm;                  // [CIN][HALO]
  float *dys = sm + CIN * HALO;    // [COUT][DYS]
  float acc[PER];
#pragma unroll
  for (int i = 0; i < PER; i++) acc[i] = 0.f;
  const long total = nf * g.tiles();
  for (long tt = blockIdx.x; tt < total; tt += gridDim.x) {
    const long tile = tt % g.tiles(), f = tt / g.tiles();
    const int bx = (int)(tile % g.tx), by = (int)((tile / g.tx) % g.ty), bz = (int)(tile / ((long)g.tx * g.ty));
    __syncthreads();
    load_halo<TI>(x, CIN, f, 0, CIN, g, bx, by, bz, xs);
    for (int i = threadIdx.x; i < COUT * TX * TY * TZ; i += kThreads) {
      const int co = i / (TX * TY * TZ), pp = i % (TX * TY * TZ);
      const int xx = bx * TX + pp % TX, yy = by * TY + (pp / TX) % TY, zz = bz * TZ + pp / (TX * TY);
      float v = 0.f;
      if (xx < g.nx && yy < g.ny && zz < g.nz) v = dy[(f * COUT + co) * g.n + ((long)zz * g.ny + yy) * g.nx + xx];
      dys[co * DYS + pp] = v;
    }
    __syncthreads();
    // the summation over the tile's points in a fixed order per thread
#pragma unroll
    for (int i = 0; i < PER; i++) {
      const int o = threadIdx.x + kThreads * i;
      if (o >= NO) continue;
      const int co = o / (CIN * 27), ci = (o / 27) % CIN, k = o % 27;
      const float *xr = xs + ci * HALO + ((k / 9) * HY + (k / 3) % 3) * HX + k % 3;
      const float *dr = dys + co * DYS;
      float s = 0.f;
      for (int hz = 0; hz < TZ; hz++)
        for (int hy = 0; hy < TY; hy++) {
          const float *xrow = xr + (hz * HY + hy) * HX, *drow = dr + (hz * TY + hy) * TX;
#pragma unroll 8
          for (int hx = 0; hx < TX; hx++) s = fmaf(drow[hx], xrow[hx], s);
        }
      acc[i] += s;
    }
  }
#pragma unroll
  for (int i = 0; i < PER; i++) {
    const int o = threadIdx.x + kThreads * i;
    if (o < NO) part[(long)blockIdx.x * NO + o] = (double)acc[i];
  }
}


// ---------------------------------------------------------------------------
// 16 -> 16 channel convolution on the tensor cores (tcgen05, kind::f16), the
// two hidden layers of the inference path.  One CTA walks the rows y of one
// (field, z, 128-point x tile).  An output row is a 128 x 16 tile
//   D[x][c_out] = sum over the 27 offsets of  A_k[x][c_in] W_k[c_out][c_in],
// A_k the input row (z + dz, y + dy) shifted by dx, read straight from a ring
// of input rows in shared memory (no im2col): in the channel-minor layout
// eight consecutive points of one channel half are one 128-byte core matrix,
// so the shifted operand is the same descriptor with its start moved by 16
// bytes per point.  The FP32 weights enter as two BF16 parts (hi + lo), 54
// MMAs of M = 128, N = 16, K = 16 per row into 16 FP32 columns of tensor
// memory; the four warps read the accumulator back (one lane per point),
// apply tanh and store BF16.  Input rows arrive by bulk copies two rows ahead
// of their first use; every wait is bounded, and on a timeout the kernel sets
// the context's error flag, waits (bounded) for what it issued, frees its
// tensor memory and returns.
// ---------------------------------------------------------------------------
namespace tcc {
using namespace fbse::async;
constexpr int kRowPts = 128 + 2;
constexpr int kHalfBytes = kRowPts * 16;    // one channel half of an input row: 2080 B
constexpr int kRowBytes = 2 * kHalfBytes;   // both halves
constexpr int kSlots = 4;                   // ring of y rows
constexpr int kSlotBytes = 3 * kRowBytes;   // rows z - 1, z, z + 1
constexpr int kWTile = 512;                 // one weight tile: 16 x 16 BF16
constexpr int kWBytes = 2 * 27 * kWTile;    // hi / lo tiles of one layer
// slack after the ring: an operand's 16 core matrices span 15 x 128 + 2080 B
// from its start, and they would span 15 x 2080 + 128 B with the two
// descriptor strides exchanged; the slack keeps both inside this CTA's memory
constexpr int kGuard = 15 * kHalfBytes + 256;
constexpr size_t kSmem = kWBytes + kSlots * kSlotBytes + kGuard;

// shared-memory matrix descriptor, K-major, no swizzle: core matrices of 8
// rows x 16 bytes, lbo between core matrices along K, sbo along M (or N)
__device__ __forceinline__ uint64_t desc_none(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // fixed 0b001; swizzle bits 61-63 stay 0
  return d;
}

// instruction descriptor: D = F32, A = B = BF16, both K-major, N = 16, M = 128
__host__ __device__ constexpr uint32_t idesc_bf16()
{
  return (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t acc)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc_bf16()), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t *bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__global__ void __launch_bounds__(128, 1) k_conv16_tc(const __nv_bfloat16 *__restrict__ in,
                                                      const __nv_bfloat16 *__restrict__ wtc,
                                                      __nv_bfloat16 *__restrict__ out, Geo g, int *status)
{
  extern __shared__ __align__(128) unsigned char sm_raw[];
  unsigned char *wsm = sm_raw;            // [hi / lo][27][c_in half][c_out][8 c_in]
  unsigned char *ring = sm_raw + kWBytes;  // [slot][dz][c half][130 points][8 channels]
  __shared__ __align__(8) uint64_t full_bar[kSlots], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  const int warp = threadIdx.x >> 5;
  const long blk = blockIdx.x;
  const int xt = (int)(blk % g.ntx), z = (int)((blk / g.ntx) % g.nz);
  const long f = blk / ((long)g.ntx * g.nz);
  const int x0 = xt * 128;
  for (int i = threadIdx.x; i < kWBytes / 16; i += blockDim.x)
    reinterpret_cast<uint4 *>(wsm)[i] = reinterpret_cast<const uint4 *>(wtc)[i];
  if (threadIdx.x == 0) {
    for (int sl = 0; sl < kSlots; sl++) mbar_init(&full_bar[sl], 1);
    mbar_init(&done_bar, 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  int nvalid = 0;
  for (int dz = 0; dz < 3; dz++) nvalid += (z + dz - 1 >= 0 && z + dz - 1 < g.nz);
  // producer: input row yy of the rows z - 1, z, z + 1 into slot yy % kSlots
  auto load_row = [&](int yy) {
    uint64_t *bar = &full_bar[yy % kSlots];
    unsigned char *slot = ring + (yy % kSlots) * kSlotBytes;
    mbar_expect_tx(bar, (uint32_t)(nvalid * kRowBytes));
    for (int dz = 0; dz < 3; dz++) {
      const int zz = z + dz - 1;
      if (zz < 0 || zz >= g.nz) continue;
      for (int h = 0; h < 2; h++)
        bulk_copy(slot + dz * kRowBytes + h * kHalfBytes, in + h8_index(g, f, 8 * h, zz, yy, x0 - 1), kHalfBytes,
                  bar);
    }
  };
  int loaded = -1, waited = -1;  // rows issued by the producer / awaited by the MMA thread
  if (threadIdx.x == 0) {
    load_row(0);
    loaded = 0;
    if (g.ny > 1) {
      load_row(1);
      loaded = 1;
    }
  }
  int committed = -1;
  for (int y = 0; y < g.ny; y++) {
    // the slot of row y + 2 held row y - 2, last read by row y - 1 (done)
    if (threadIdx.x == 0 && y + 2 < g.ny) {
      load_row(y + 2);
      loaded = y + 2;
    }
    if (threadIdx.x == 32) {
      bool ok = true;
      for (int yy = waited + 1; yy <= y + 1 && yy < g.ny && ok; yy++) {
        ok = mbar_wait(&full_bar[yy % kSlots], (uint32_t)((yy / kSlots) & 1));
        if (ok) waited = yy;
      }
      if (!ok) {
        atomicExch(&fail, 1);
      } else {
        asm volatile("tcgen05.fence::after_thread_sync;");
        uint32_t acc = 0;
        for (int dy = 0; dy < 3; dy++) {
          const int yy = y + dy - 1;
          if (yy < 0 || yy >= g.ny) continue;
          for (int dz = 0; dz < 3; dz++) {
            const int zz = z + dz - 1;
            if (zz < 0 || zz >= g.nz) continue;
            const uint32_t base = smem_u32(ring + (yy % kSlots) * kSlotBytes + dz * kRowBytes);
            for (int dx = 0; dx < 3; dx++) {
              const uint64_t a = desc_none(base + dx * 16, kHalfBytes, 128);
              const int k = (dz * 3 + dy) * 3 + dx;
              for (int hl = 0; hl < 2; hl++) {
                mma_bf16(tmem, a, desc_none(smem_u32(wsm + (hl * 27 + k) * kWTile), 256, 128), acc);
                acc = 1;
              }
            }
          }
        }
        commit(&done_bar);
        committed = y;
      }
    }
    __syncthreads();
    if (fail) break;
    // epilogue: lane = point, 16 FP32 columns = output channels
    bool ok = mbar_wait(&done_bar, (uint32_t)(y & 1));
    ok = __all_sync(0xffffffffu, ok);
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (ok) {
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int x = x0 + threadIdx.x;
      if (x < g.nx) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
          __align__(16) __nv_bfloat16 v[8];
#pragma unroll
          for (int j = 0; j < 8; j++) v[j] = __float2bfloat16(tanhf(__uint_as_float(r[8 * h + j])));
          *reinterpret_cast<uint4 *>(out + h8_index(g, f, 8 * h, z, y, x)) = *reinterpret_cast<uint4 *>(v);
        }
      }
    } else {
      atomicExch(&fail, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (fail) break;
  }
  if (fail) {
    if (threadIdx.x == 0) {
      atomicExch(status, 1);
      // copies still in flight land before the CTA leaves (bounded)
      for (int yy = (waited > loaded - 3 ? waited + 1 : loaded - 2); yy <= loaded; yy++)
        if (yy >= 0) mbar_wait(&full_bar[yy % kSlots], (uint32_t)((yy / kSlots) & 1));
    }
    // MMAs still in flight finish before their tensor memory is released (bounded)
    if (threadIdx.x == 32 && committed >= 0) mbar_wait(&done_bar, (uint32_t)(committed & 1));
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem));
}

// weight tiles of one 16 -> 16 layer: w[co][ci][27] FP32 -> hi and lo BF16
// parts, tile (part, k) laid out [ci half][co][8 ci]
__global__ void k_prep_wtc(const float *__restrict__ w, __nv_bfloat16 *__restrict__ out)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 16 * 16 * 27; i += gridDim.x * blockDim.x) {
    const int co = i / (16 * 27), ci = (i / 27) % 16, k = i % 27;
    const float v = w[i];
    const __nv_bfloat16 hi = __float2bfloat16(v);
    const __nv_bfloat16 lo = __float2bfloat16(v - __bfloat162float(hi));
    const int o = k * 256 + (ci / 8) * 128 + co * 8 + ci % 8;
    out[o] = hi;
    out[27 * 256 + o] = lo;
  }
}

}  // namespace tcc

// out[o] = sum_b part[b][o] in order b = 0, 1, ...
__global__ void k_sum_parts(const double *__restrict__ part, int nb, int no, double *__restrict__ out)
{
  for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < no; o += gridDim.x * blockDim.x) {
    double s = 0;
    for (int b = 0; b < nb; b++) s += part[(long)b * no + o];
    out[o] = s;
  }
}

// forward layout [ci][k][co] and the flipped, transposed layout of the data
// gradient [co][26 - k][ci] (a convolution from COUT to CIN channels) of
// layer weights w[co][ci][k]
__global__ void k_prep_w(const float *__restrict__ w, int cin, int cout, float *__restrict__ wf,
                         float *__restrict__ wb)
{
  const int n = cin * cout * 27;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int co = i / (cin * 27), ci = (i / 27) % cin, k = i % 27;
    wf[(ci * 27 + k) * cout + co] = w[i];
    wb[(co * 27 + (26 - k)) * cin + ci] = w[i];
  }
}

// mean squares of the fields of n psitot states: rms[f], f = state * fps + comp
// (comp = spin * (cplx + 1) + part); one CTA per field, fixed-order reduction
__global__ void k_field_rms(const double *__restrict__ psi, long ngrid, int nspin, int cplx, double *__restrict__ rms)
{
  const int fps = nspin * (cplx + 1);
  const long f = blockIdx.x, st = f / fps, comp = f % fps;
  const long spin = comp / (cplx + 1), part = comp % (cplx + 1);
  const long stlen = (long)(cplx + 1) * nspin * ngrid;
  const double *base = psi + st * stlen;
  double s = 0;
  for (long p = threadIdx.x; p < ngrid; p += blockDim.x) {
    const double v = cplx ? base[(spin * ngrid + p) * 2 + part] : base[spin * ngrid + p];
    s += v * v;
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) rms[f] = sqrt(red[0] / (double)ngrid);
}

// network input x0[f][2][p] (BF16) and, with corr, the target of y,
// t[f][p] = (corr - f) / rms (the output adds f back)
__global__ void k_field_in(const double *__restrict__ psi, const double *__restrict__ corr, long nf, long ngrid,
                           int nspin, int cplx, const double *__restrict__ pot, const double *__restrict__ ene,
                           const double *__restrict__ rms, __nv_bfloat16 *__restrict__ x0, float *__restrict__ tgt)
{
  const int fps = nspin * (cplx + 1);
  const long stlen = (long)(cplx + 1) * nspin * ngrid;
  const long total = nf * ngrid;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long f = i / ngrid, p = i % ngrid, st = f / fps, comp = f % fps;
    const long spin = comp / (cplx + 1), part = comp % (cplx + 1);
    const long e = st * stlen + (cplx ? (spin * ngrid + p) * 2 + part : spin * ngrid + p);
    const double r = rms[f] > 0 ? 1.0 / rms[f] : 0.0;
    const double v = psi[e] * r;
    x0[(f * 2) * ngrid + p] = __float2bfloat16((float)v);
    x0[(f * 2 + 1) * ngrid + p] = __float2bfloat16((float)(v * (pot[p] - ene[st]) / kVScale));
    if (tgt) tgt[i] = (float)((corr[e] - psi[e]) * r);
  }
}

// out (psitot layout) = resid + y * rms
__global__ void k_field_out(const float *__restrict__ y, const double *__restrict__ resid, long nf, long ngrid,
                            int nspin, int cplx, const double *__restrict__ rms, double *__restrict__ out)
{
  const int fps = nspin * (cplx + 1);
  const long stlen = (long)(cplx + 1) * nspin * ngrid;
  const long total = nf * ngrid;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const long f = i / ngrid, p = i % ngrid, st = f / fps, comp = f % fps;
    const long spin = comp / (cplx + 1), part = comp % (cplx + 1);
    const long e = st * stlen + (cplx ? (spin * ngrid + p) * 2 + part : spin * ngrid + p);
    out[e] = resid[e] + (double)y[i] * rms[f];
  }
}

// loss partials and dL/dy for L = mean (y - t)^2; CTA b sums elements b, b + G, ... in order
__global__ void k_mse(const float *__restrict__ y, const float *__restrict__ t, long total, float *__restrict__ dy,
                      double *__restrict__ part)
{
  double s = 0;
  const float sc = 2.f / (float)total;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const float d = y[i] - t[i];
    s += (double)d * d;
    dy[i] = sc * d;
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                       const double *__restrict__ g, int n, float lr, float b1c, float b2c)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = (float)g[i];
    m[i] = 0.9f * m[i] + 0.1f * gi;
    v[i] = 0.999f * v[i] + 0.001f * gi * gi;
    w[i] -= lr * (m[i] / b1c) / (sqrtf(v[i] / b2c) + 1e-8f);
  }
}

// r = hpsi - e psi (psitot layout, FP64); r may be hpsi itself
__global__ void k_residual(const double *__restrict__ psi, const double *hpsi, const double *__restrict__ e, long n,
                           long stlen, double *r)
{
  const long total = n * stlen;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x)
    r[i] = hpsi[i] - e[i / stlen] * psi[i];
}

}  // namespace pc
}  // namespace fbse

struct fbse_precond {
  fbse_ctx *c = nullptr;
  float *w = nullptr, *m = nullptr, *v = nullptr;  // weights and Adam moments (device)
  float *wf = nullptr, *wb = nullptr;              // per-layer forward / backward layouts (device)
  double *g = nullptr;                             // gradient (device, FP64 sums)
  __nv_bfloat16 *wtc = nullptr;                    // tensor-core weight tiles of the two hidden layers
  long step = 0;
  // activations and scratch, grown on demand
  void *buf = nullptr;
  size_t buf_bytes = 0;
};

namespace fbse {
namespace pc {

static unsigned blocks_for(long n) { return (unsigned)std::max<long>(1, std::min<long>((n + 255) / 256, 152L * 32)); }

template <int CIN, int COUT, int MODE, typename TI, bool H8 = false>
static int conv(fbse_precond *P, const TI *in, const float *w, void *out, const __nv_bfloat16 *act, const Geo &g,
                long nf)
{
  fbse_ctx *c = P->c;
  constexpr int CC = CIN < 4 ? CIN : 4;
  const size_t smem = (size_t)(CIN * 27 * COUT + CC * HALO) * sizeof(float);
  FBSE_CUDA(c, cudaFuncSetAttribute(k_conv<CIN, COUT, MODE, TI, H8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  k_conv<CIN, COUT, MODE, TI, H8><<<(unsigned)(nf * g.tiles()), kThreads, smem, c->stream>>>(in, w, out, act, g);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

// one hidden layer on the tensor cores (channel-minor input and output)
static int conv_tc(fbse_precond *P, const __nv_bfloat16 *in, const __nv_bfloat16 *wtc, __nv_bfloat16 *out,
                   const Geo &g, long nf)
{
  fbse_ctx *c = P->c;
  FBSE_CUDA(c, cudaFuncSetAttribute(tcc::k_conv16_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tcc::kSmem));
  tcc::k_conv16_tc<<<(unsigned)(nf * g.nz * g.ntx), 128, tcc::kSmem, c->stream>>>(in, wtc, out, g, c->dstatus);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <int CIN, int COUT, typename TI>
static int wgrad(fbse_precond *P, const TI *x, const float *dy, const Geo &g, long nf, double *part, double *gout)
{
  fbse_ctx *c = P->c;
  const size_t smem = (size_t)(CIN * HALO + COUT * (TX * TY * TZ + 1)) * sizeof(float);
  FBSE_CUDA(c, cudaFuncSetAttribute(k_conv_wgrad<CIN, COUT, TI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
  k_conv_wgrad<CIN, COUT, TI><<<kWgCtas, kThreads, smem, c->stream>>>(x, dy, g, nf, part);
  FBSE_CHECK_LAUNCH(c);
  k_sum_parts<<<(COUT * CIN * 27 + 255) / 256, 256, 0, c->stream>>>(part, kWgCtas, COUT * CIN * 27, gout);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

static Geo geo(fbse_ctx *c)
{
  Geo g;
  g.nx = (int)c->nx;
  g.ny = (int)c->ny;
  g.nz = (int)c->nz;
  g.n = c->ngrid;
  g.tx = (g.nx + TX - 1) / TX;
  g.ty = (g.ny + TY - 1) / TY;
  g.tz = (g.nz + TZ - 1) / TZ;
  g.ntx = (g.nx + 127) / 128;
  g.px = g.ntx * 128 + 2;
  return g;
}

// scratch layout for nf fields of the context's grid
struct Bufs {
  double *rms, *ene, *lpart, *wpart;
  __nv_bfloat16 *x0, *a1, *a2, *a3;
  float *y, *t, *d4, *d3, *d2, *d1;
  __nv_bfloat16 *h1, *h2, *h3;  // inference: channel-minor hidden activations
  size_t h_bytes;
};

static int bufs(fbse_precond *P, long nf, long nstates, bool train, Bufs *b)
{
  fbse_ctx *c = P->c;
  const long N = c->ngrid;
  auto al = [](size_t x) { return (x + 255) / 256 * 256; };
  size_t off[16], tot = 0;
  int k = 0;
  auto add = [&](size_t bytes) { off[k++] = tot; tot += al(bytes); };
  add(nf * sizeof(double));                        // rms
  add(std::max<long>(nstates, 1) * sizeof(double));  // ene
  add(1025 * sizeof(double));                      // loss partials and their sum
  add((size_t)kWgCtas * kC * kC * 27 * sizeof(double));  // weight-gradient partials
  add((size_t)nf * 2 * N * 2);                     // x0
  add((size_t)nf * kC * N * 2);                    // a1
  add((size_t)nf * kC * N * 2);                    // a2
  add((size_t)nf * kC * N * 2);                    // a3
  add((size_t)nf * N * 4);                         // y
  const Geo gg = geo(c);
  const size_t hb = (size_t)nf * 2 * gg.nz * gg.ny * gg.px * 8 * 2;
  if (!train) {
    add(hb);                                       // h1
    add(hb);                                       // h2
    add(hb);                                       // h3
  }
  if (train) {
    add((size_t)nf * N * 4);                       // t
    add((size_t)nf * N * 4);                       // d4
    add((size_t)nf * kC * N * 4);                  // d3
    add((size_t)nf * kC * N * 4);                  // d2
    add((size_t)nf * kC * N * 4);                  // d1
  }
  int rc = ensure(c, &P->buf, &P->buf_bytes, tot);
  if (rc) return rc;
  char *B = static_cast<char *>(P->buf);
  b->rms = (double *)(B + off[0]);
  b->ene = (double *)(B + off[1]);
  b->lpart = (double *)(B + off[2]);
  b->wpart = (double *)(B + off[3]);
  b->x0 = (__nv_bfloat16 *)(B + off[4]);
  b->a1 = (__nv_bfloat16 *)(B + off[5]);
  b->a2 = (__nv_bfloat16 *)(B + off[6]);
  b->a3 = (__nv_bfloat16 *)(B + off[7]);
  b->y = (float *)(B + off[8]);
  b->t = train ? (float *)(B + off[9]) : nullptr;
  b->d4 = train ? (float *)(B + off[10]) : nullptr;
  b->d3 = train ? (float *)(B + off[11]) : nullptr;
  b->d2 = train ? (float *)(B + off[12]) : nullptr;
  b->d1 = train ? (float *)(B + off[13]) : nullptr;
  b->h1 = train ? nullptr : (__nv_bfloat16 *)(B + off[9]);
  b->h2 = train ? nullptr : (__nv_bfloat16 *)(B + off[10]);
  b->h3 = train ? nullptr : (__nv_bfloat16 *)(B + off[11]);
  b->h_bytes = train ? 0 : hb;
  return FBSE_OK;
}

static int prep_weights(fbse_precond *P)
{
  fbse_ctx *c = P->c;
  for (int l = 0; l < kLayers; l++) {
    k_prep_w<<<32, 256, 0, c->stream>>>(P->w + kWOff[l], kCin[l], kCout[l], P->wf + kWOff[l], P->wb + kWOff[l]);
    FBSE_CHECK_LAUNCH(c);
  }
  return FBSE_OK;
}

// inputs (and targets) of the n states, then the forward pass; y holds the output
static int forward(fbse_precond *P, const double *resid, const double *corr, const double *ene_host, long n,
                   bool train, Bufs *b, long *nf_out)
{
  fbse_ctx *c = P->c;
  const int fps = c->nspin * (c->is_complex + 1);
  const long nf = n * fps, N = c->ngrid;
  int rc = bufs(P, nf, n, train, b);
  if (rc) return rc;
  *nf_out = nf;
  FBSE_CUDA(c, h2d(c->stream, b->ene, ene_host, n * sizeof(double)));
  if ((rc = prep_weights(P))) return rc;
  k_field_rms<<<(unsigned)nf, 256, 0, c->stream>>>(resid, N, c->nspin, c->is_complex, b->rms);
  FBSE_CHECK_LAUNCH(c);
  k_field_in<<<blocks_for(nf * N), 256, 0, c->stream>>>(resid, corr, nf, N, c->nspin, c->is_complex, c->pot64, b->ene,
                                                        b->rms, b->x0, train ? b->t : nullptr);
  FBSE_CHECK_LAUNCH(c);
  const Geo g = geo(c);
  if (!train) {
    // inference: the hidden layers on the tensor cores in the channel-minor
    // layout (zero padding columns: the kernels write interior points only)
    FBSE_CUDA(c, cudaMemsetAsync(b->h1, 0, 3 * ((b->h_bytes + 255) / 256 * 256), c->stream));
    for (int l = 1; l <= 2; l++) {
      tcc::k_prep_wtc<<<27, 256, 0, c->stream>>>(P->w + kWOff[l], P->wtc + (l - 1) * (tcc::kWBytes / 2));
      FBSE_CHECK_LAUNCH(c);
    }
    if ((rc = conv<2, kC, 3>(P, b->x0, P->wf + kWOff[0], b->h1, nullptr, g, nf))) return rc;
    if ((rc = conv_tc(P, b->h1, P->wtc, b->h2, g, nf))) return rc;
    if ((rc = conv_tc(P, b->h2, P->wtc + tcc::kWBytes / 2, b->h3, g, nf))) return rc;
    return conv<kC, 1, 1, __nv_bfloat16, true>(P, b->h3, P->wf + kWOff[3], b->y, nullptr, g, nf);
  }
  if ((rc = conv<2, kC, 0>(P, b->x0, P->wf + kWOff[0], b->a1, nullptr, g, nf))) return rc;
  if ((rc = conv<kC, kC, 0>(P, b->a1, P->wf + kWOff[1], b->a2, nullptr, g, nf))) return rc;
  if ((rc = conv<kC, kC, 0>(P, b->a2, P->wf + kWOff[2], b->a3, nullptr, g, nf))) return rc;
  return conv<kC, 1, 1>(P, b->a3, P->wf + kWOff[3], b->y, nullptr, g, nf);
}

// loss (host) and the gradient into P->g (device)
static int backward(fbse_precond *P, const Bufs &b, long nf, double *loss)
{
  fbse_ctx *c = P->c;
  const long N = c->ngrid, total = nf * N;
  const Geo g = geo(c);
  int rc;
  k_mse<<<1024, 256, 0, c->stream>>>(b.y, b.t, total, b.d4, b.lpart);
  FBSE_CHECK_LAUNCH(c);
  k_sum_parts<<<1, 32, 0, c->stream>>>(b.lpart, 1024, 1, b.lpart + 1024);
  FBSE_CHECK_LAUNCH(c);
  // weight gradients need the layer inputs and output gradients; data
  // gradients run through the flipped, transposed weights
  if ((rc = wgrad<kC, 1>(P, b.a3, b.d4, g, nf, b.wpart, P->g + kWOff[3]))) return rc;
  if ((rc = conv<1, kC, 2>(P, b.d4, P->wb + kWOff[3], b.d3, b.a3, g, nf))) return rc;
  if ((rc = wgrad<kC, kC>(P, b.a2, b.d3, g, nf, b.wpart, P->g + kWOff[2]))) return rc;
  if ((rc = conv<kC, kC, 2>(P, b.d3, P->wb + kWOff[2], b.d2, b.a2, g, nf))) return rc;
  if ((rc = wgrad<kC, kC>(P, b.a1, b.d2, g, nf, b.wpart, P->g + kWOff[1]))) return rc;
  if ((rc = conv<kC, kC, 2>(P, b.d2, P->wb + kWOff[1], b.d1, b.a1, g, nf))) return rc;
  if ((rc = wgrad<2, kC>(P, b.x0, b.d1, g, nf, b.wpart, P->g + kWOff[0]))) return rc;
  double l = 0;
  FBSE_CUDA(c, d2h(c->stream, &l, b.lpart + 1024, sizeof(double)));
  *loss = l / (double)total;
  return FBSE_OK;
}

}  // namespace pc

static int precond_check(fbse_precond *p, const void *a, long n)
{
  if (!p || !p->c) return FBSE_ERR_ARG;
  if (!a || n < 1) return set_err(p->c, FBSE_ERR_ARG, "precond: null states or n < 1");
  if (p->c->nx > 65535 || p->c->ny > 65535 || p->c->nz > 65535)
    return set_err(p->c, FBSE_ERR_UNSUPPORTED, "precond: grid too large");
  return FBSE_OK;
}

// r_i = H psi_i - e_i psi_i for n psitot rows (device, FP64 layout), H psi in
// the context's precision; e device
static int residual_dev(fbse_ctx *c, const double *psi, long n, const double *e_dev, double *r)
{
  const long stlen = (long)(c->is_complex + 1) * c->nspin * c->ngrid;
  const long len = (long)c->nspin * c->ngrid;
  const size_t wbytes = (c->precision == FBSE_MIXED ? sizeof(float2) : sizeof(double2)) * (size_t)len;
  const long chunk = 16;
  void *w0 = nullptr;
  if (cudaMalloc(&w0, 2 * chunk * wbytes) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_OOM, "residual: H psi scratch");
  }
  void *w1 = static_cast<char *>(w0) + chunk * wbytes;
  int rc = FBSE_OK;
  for (long s0 = 0; s0 < n && !rc; s0 += chunk) {
    const long ns = std::min(chunk, n - s0);
    const long nw = c->is_complex ? ns : (ns + 1) / 2;
    if ((rc = pack_states(c, psi + s0 * stlen, w0, ns))) break;
    rc = c->precision == FBSE_MIXED ? hpsi_apply<float>(c, (float2 *)w0, (float2 *)w1, nw, 1.0, 0.0)
                                    : hpsi_apply<double>(c, (double2 *)w0, (double2 *)w1, nw, 1.0, 0.0);
    if (rc) break;
    if ((rc = unpack_states(c, w1, r + s0 * stlen, ns))) break;
  }
  if (!rc) {
    pc::k_residual<<<pc::blocks_for(n * stlen), 256, 0, c->stream>>>(psi, r, e_dev, n, stlen, r);
    rc = launch_status(c);
    FBSE_COUNT(1);
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(w0);
  return rc;
}

static int residual_host_e(fbse_ctx *c, const double *psi, long n, const double *e_host, double *r)
{
  double *ed = nullptr;
  if (cudaMalloc(&ed, n * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_OOM, "residual: energies");
  }
  int rc = h2d(c->stream, ed, e_host, n * sizeof(double)) == cudaSuccess ? FBSE_OK
                                                                          : set_err(c, FBSE_ERR_CUDA, "residual");
  if (!rc) rc = residual_dev(c, psi, n, ed, r);
  cudaStreamSynchronize(c->stream);
  cudaFree(ed);
  return rc;
}

// one round of refinement; returns the new pair count in *n_out
static int refine_round(fbse_ctx *c, fbse_precond *P, double *psitot, long n, long cap, double tol, double *eval,
                        double *sigma, long *n_out)
{
  const long stlen = (long)(c->is_complex + 1) * c->nspin * c->ngrid;
  std::vector<long> sel;
  for (long i = 0; i < n && n + (long)sel.size() < cap; i++)
    if (sigma[i] > tol) sel.push_back(i);
  *n_out = n;
  if (sel.empty()) return FBSE_OK;
  const long nd = (long)sel.size();
  int rc = FBSE_OK;
  // the selected states after the n rows, their residuals, then P(r) there
  double *dst = psitot + n * stlen;
  for (long k = 0; k < nd; k++)
    FBSE_CUDA(c, cudaMemcpyAsync(dst + k * stlen, psitot + sel[k] * stlen, stlen * sizeof(double),
                                 cudaMemcpyDeviceToDevice, c->stream));
  void *rb = nullptr;
  if ((rc = cached(c, kSlotHpsi, (size_t)nd * stlen * sizeof(double), &rb))) return rc;
  double *res = static_cast<double *>(rb);
  std::vector<double> e(nd);
  for (long k = 0; k < nd; k++) e[k] = eval[sel[k]];
  if ((rc = residual_host_e(c, dst, nd, e.data(), res))) return rc;
  if (P) {
    if ((rc = fbse_precond_apply(P, res, e.data(), nd, dst))) return rc;
  } else {
    FBSE_CUDA(c, cudaMemcpyAsync(dst, res, nd * stlen * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  }
  // unit norms: a residual's norm is sigma (1e-3 and below), so its overlap
  // eigenvalue would fall under the Rayleigh-Ritz step's relative cut and the
  // new direction would be dropped
  if ((rc = normalize_all(c, dst, nd, nullptr))) return rc;
  // Rayleigh-Ritz on the n pairs and the nd new directions
  long nk = 0;
  if ((rc = ortho_diag_sigma(c, psitot, n + nd, &nk, eval, sigma))) return rc;
  *n_out = nk;
  return FBSE_OK;
}

}  // namespace fbse

using namespace fbse;

extern "C" {

int fbse_precond_create(fbse_ctx *c, fbse_precond **out, const float *weights, long seed)
{
  if (!c || !out) return c ? set_err(c, FBSE_ERR_ARG, "fbse_precond_create: null") : FBSE_ERR_ARG;
  *out = nullptr;
  fbse_precond *P = new fbse_precond();
  P->c = c;
  const size_t nw = FBSE_PRECOND_NWEIGHTS;
  void *m = nullptr;
  if (cudaMalloc(&m, nw * sizeof(float) * 5 + nw * sizeof(double) + 2 * pc::tcc::kWBytes) != cudaSuccess) {
    cudaGetLastError();
    delete P;
    return set_err(c, FBSE_ERR_OOM, "fbse_precond_create");
  }
  P->w = static_cast<float *>(m);
  P->m = P->w + nw;
  P->v = P->m + nw;
  P->wf = P->v + nw;
  P->wb = P->wf + nw;
  P->g = reinterpret_cast<double *>(P->wb + nw);
  P->wtc = reinterpret_cast<__nv_bfloat16 *>(P->g + nw);
  std::vector<float> w(nw);
  if (weights) {
    std::copy(weights, weights + nw, w.begin());
  } else {
    // uniform in +-sqrt(3 / fan_in) (unit variance through each layer), the
    // last layer at a tenth of that so that P(r) = r + y rms starts near r;
    // drawn with the reference's own generator (ran_nrc) from the seed
    long s = -std::labs(seed) - 1;
    for (int l = 0; l < pc::kLayers; l++) {
      const double a = std::sqrt(3.0 / (pc::kCin[l] * 27.0)) * (l == pc::kLayers - 1 ? 0.1 : 1.0);
      for (long i = pc::kWOff[l]; i < pc::kWOff[l + 1]; i++) w[i] = (float)(a * (2.0 * fbse_ran(&s) - 1.0));
    }
  }
  int rc = FBSE_OK;
  if (cudaMemcpy(P->w, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(P->m, 0, 2 * nw * sizeof(float)) != cudaSuccess)
    rc = set_err(c, FBSE_ERR_CUDA, "fbse_precond_create: upload");
  if (rc) {
    cudaFree(m);
    delete P;
    return rc;
  }
  *out = P;
  return FBSE_OK;
}

void fbse_precond_destroy(fbse_precond *p)
{
  if (!p) return;
  // waits for the whole device rather than the context's stream: the context
  // may already be destroyed (destruction order is the caller's)
  cudaDeviceSynchronize();
  cudaFree(p->w);
  if (p->buf) cudaFree(p->buf);
  delete p;
}

int fbse_precond_get_weights(fbse_precond *p, float *w)
{
  if (!p || !w) return p ? set_err(p->c, FBSE_ERR_ARG, "fbse_precond_get_weights: null") : FBSE_ERR_ARG;
  if (d2h(p->c->stream, w, p->w, FBSE_PRECOND_NWEIGHTS * sizeof(float)) != cudaSuccess)
    return set_err(p->c, FBSE_ERR_CUDA, "fbse_precond_get_weights");
  return FBSE_OK;
}

int fbse_precond_set_weights(fbse_precond *p, const float *w)
{
  if (!p || !w) return p ? set_err(p->c, FBSE_ERR_ARG, "fbse_precond_set_weights: null") : FBSE_ERR_ARG;
  if (h2d(p->c->stream, p->w, w, FBSE_PRECOND_NWEIGHTS * sizeof(float)) != cudaSuccess ||
      cudaStreamSynchronize(p->c->stream) != cudaSuccess)
    return set_err(p->c, FBSE_ERR_CUDA, "fbse_precond_set_weights");
  return FBSE_OK;
}

int fbse_precond_apply(fbse_precond *p, const double *resid, const double *ene, long n, double *out)
{
  int rc = precond_check(p, resid, n);
  if (rc) return rc;
  if (!out || !ene || out == resid) return set_err(p->c, FBSE_ERR_ARG, "fbse_precond_apply: out / ene");
  fbse_ctx *c = p->c;
  // states per pass: activations of at most ~4 GB
  const long fps = c->nspin * (c->is_complex + 1);
  const double per_state = (double)fps * c->ngrid * (2 * 2 + 3 * pc::kC * 2 + 4);
  const long chunk = std::max<long>(1, std::min<long>(n, (long)(4.0e9 / per_state)));
  const long stlen = (long)(c->is_complex + 1) * c->nspin * c->ngrid;
  for (long s0 = 0; s0 < n; s0 += chunk) {
    const long ns = std::min(chunk, n - s0);
    pc::Bufs b;
    long nf = 0;
    if ((rc = pc::forward(p, resid + s0 * stlen, nullptr, ene + s0, ns, false, &b, &nf))) return rc;
    pc::k_field_out<<<pc::blocks_for(nf * c->ngrid), 256, 0, c->stream>>>(
        b.y, resid + s0 * stlen, nf, c->ngrid, c->nspin, c->is_complex, b.rms, out + s0 * stlen);
    FBSE_CHECK_LAUNCH(c);
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return set_err(c, FBSE_ERR_CUDA, "fbse_precond_apply");
  return check_dev_status(c);
}

int fbse_precond_grad(fbse_precond *p, const double *resid, const double *corr, const double *ene, long n,
                      double *loss, float *grad)
{
  int rc = precond_check(p, resid, n);
  if (rc) return rc;
  if (!corr || !ene || !loss) return set_err(p->c, FBSE_ERR_ARG, "fbse_precond_grad: null");
  pc::Bufs b;
  long nf = 0;
  if ((rc = pc::forward(p, resid, corr, ene, n, true, &b, &nf))) return rc;
  if ((rc = pc::backward(p, b, nf, loss))) return rc;
  if (grad) {
    std::vector<double> g(FBSE_PRECOND_NWEIGHTS);
    if (d2h(p->c->stream, g.data(), p->g, g.size() * sizeof(double)) != cudaSuccess)
      return set_err(p->c, FBSE_ERR_CUDA, "fbse_precond_grad: download");
    for (size_t i = 0; i < g.size(); i++) grad[i] = (float)g[i];
  }
  return FBSE_OK;
}

int fbse_precond_train_step(fbse_precond *p, const double *resid, const double *corr, const double *ene, long n,
                            double lr, double *loss)
{
  int rc = fbse_precond_grad(p, resid, corr, ene, n, loss, nullptr);
  if (rc) return rc;
  if (!(lr > 0)) return set_err(p->c, FBSE_ERR_ARG, "fbse_precond_train_step: lr must be positive");
  p->step++;
  const float b1c = (float)(1.0 - std::pow(0.9, (double)p->step));
  const float b2c = (float)(1.0 - std::pow(0.999, (double)p->step));
  fbse_ctx *c = p->c;
  pc::k_adam<<<64, 256, 0, c->stream>>>(p->w, p->m, p->v, p->g, FBSE_PRECOND_NWEIGHTS, (float)lr, b1c, b2c);
  FBSE_CHECK_LAUNCH(c);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return set_err(c, FBSE_ERR_CUDA, "fbse_precond_train_step");
  return FBSE_OK;
}

int fbse_residual(fbse_ctx *c, const double *psitot, long n, const double *ene, double *out)
{
  if (!c || !psitot || !ene || !out || n < 1 || out == psitot)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_residual: arguments") : FBSE_ERR_ARG;
  const int rc = residual_host_e(c, psitot, n, ene, out);
  return rc ? rc : check_dev_status(c);
}

int fbse_refine(fbse_ctx *c, fbse_precond *p, double *psitot, long n, long cap, int steps, double tol, long *n_out,
                double *eval, double *sigma)
{
  if (!c || !psitot || !n_out || !eval || !sigma || n < 1 || cap < n || steps < 0)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_refine: arguments") : FBSE_ERR_ARG;
  if (p && p->c != c) return set_err(c, FBSE_ERR_ARG, "fbse_refine: preconditioner of another context");
  long cur = n;
  for (int s = 0; s < steps; s++) {
    long nk = cur;
    const int rc = refine_round(c, p, psitot, cur, cap, tol, eval, sigma, &nk);
    if (rc) return rc;
    if (nk == cur && s > 0) break;
    cur = nk;
  }
  *n_out = cur;
  return check_dev_status(c);
}

}  // extern "C"
