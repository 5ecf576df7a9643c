// Real "NT" GEMM on the 5th-generation tensor cores (tcgen05, TMEM
// accumulators) with three-term split-TF32 products:
//   C[i][j] = sum_k A[i][k] B[j][k],  A = Ah + Al, B = Bh + Bl (TF32 parts),
//   C ~ Ah Bh^T + Ah Bl^T + Al Bh^T  (the Al Bl^T term is below FP32 rounding)
// accumulated in FP32 in tensor memory, split over K into FP32 partial
// tiles that are summed in FP64 afterwards.
//
// Operands are "tile images": 128 rows x 32 FP32 (16 KB) blocks in the exact
// shared-memory layout the MMA reads (K-major, 128-byte swizzle: the 16-byte
// chunk c of row r sits at chunk c ^ (r % 8)), stored [row block][k block].
// A prep kernel writes them from the complex working arrays, with the
// element map of the product wanted (plain, conjugated or swapped parts), so
// the GEMM kernel only moves whole tiles with bulk asynchronous copies.
//
// CTA: 128 threads.  Thread 0 issues the copies (two stages of A 128 x 32 and
// B 256 x 32, hi and lo parts: 96 KB each), thread 32 issues the MMAs
// (M = 128, N = 256, K = 8 per instruction) and commits them to the stage's
// "free" barrier; after the last k block all four warps read the 128 x 256
// FP32 accumulator out of tensor memory (each warp its 32 lanes).  Every
// wait is bounded: on a timeout the kernel records an error code, waits
// (bounded) for its own copies and MMAs, frees its tensor memory and returns.
#include <cstdint>
#include <cstdlib>

#include "fbse_internal.cuh"
#include "fbse_async.cuh"

namespace fbse {
namespace tc {

using namespace fbse::async;

constexpr int kBM = 128, kBN = 256, kBK = 32;   // CTA tile: M x N, k block (FP32 elements)
constexpr int kTileBytes = kBM * kBK * 4;        // one 128 x 32 image: 16 KB
constexpr int kStageBytes = 6 * kTileBytes;      // Ah, Al (1 image each), Bh, Bl (2 each)
constexpr int kStages = 2;
// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), leading byte offset unused (1)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);       // start address
  d |= (uint64_t)1 << 16;                        // leading byte offset (unused for this layout)
  d |= (uint64_t)(1024 >> 4) << 32;              // stride byte offset
  d |= (uint64_t)1 << 46;                        // fixed 0b001
  d |= (uint64_t)2 << 61;                        // 128-byte swizzle
  return d;
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, N = 256, M = 128
__host__ __device__ constexpr uint32_t idesc_tf32()
{
  return (1u << 4)                   // D format F32
         | (2u << 7)                 // A format TF32
         | (2u << 10)                // B format TF32
         | ((uint32_t)(kBN >> 3) << 17)
         | ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t acc)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc_tf32()), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// C partials: part[split][i][j] for i < mp (rows, multiple of 128), j < np
// (multiple of 256).  A images: [mp/128][nkb], B images: [np/128][nkb].
// The CTA (bx, by, bz) covers rows 128 bx, columns 256 by and k blocks
// [kb0, kb1) of split bz.
__global__ void __launch_bounds__(128, 1)
    k_tc_gemm_nt(const float *__restrict__ Ah, const float *__restrict__ Al, const float *__restrict__ Bh,
                 const float *__restrict__ Bl, long nkb, long kb_per_split, float *__restrict__ part, long mp,
                 long np, int terms, int *__restrict__ status)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte alignment of the stage buffers (the swizzle atom)
  unsigned char *base = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
  unsigned char *stage = base;
  __shared__ __align__(8) uint64_t full_bar[kStages], free_bar[kStages], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long kb0 = (long)blockIdx.z * kb_per_split;
  const long kb1 = min(nkb, kb0 + kb_per_split);
  const long nk = kb1 - kb0;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; s++) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&free_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    // 256 FP32 columns x 128 lanes of tensor memory for the accumulator
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  const float *ah = Ah + ((long)blockIdx.x * nkb) * (kTileBytes / 4);
  const float *al = Al + ((long)blockIdx.x * nkb) * (kTileBytes / 4);
  const float *bh = Bh + ((long)(2 * blockIdx.y) * nkb) * (kTileBytes / 4);
  const float *bl = Bl + ((long)(2 * blockIdx.y) * nkb) * (kTileBytes / 4);
  const long rowblk = nkb * (kTileBytes / 4);  // floats between row blocks of B
  int ok = 1;
  long issued = 0;
  if (threadIdx.x == 0) {
    // producer: stage k block kb into buffer s = it % kStages
    for (long it = 0; it < nk && ok; it++) {
      const int s = (int)(it % kStages);
      if (it >= kStages) ok = mbar_wait(&free_bar[s], (uint32_t)(((it / kStages) - 1) & 1));
      if (!ok) break;
      unsigned char *buf = stage + (long)s * kStageBytes;
      const long kb = kb0 + it;
      mbar_expect_tx(&full_bar[s], kStageBytes);
      bulk_copy(buf + 0 * kTileBytes, ah + kb * (kTileBytes / 4), kTileBytes, &full_bar[s]);
      bulk_copy(buf + 1 * kTileBytes, al + kb * (kTileBytes / 4), kTileBytes, &full_bar[s]);
      bulk_copy(buf + 2 * kTileBytes, bh + kb * (kTileBytes / 4), kTileBytes, &full_bar[s]);
      bulk_copy(buf + 3 * kTileBytes, bh + rowblk + kb * (kTileBytes / 4), kTileBytes, &full_bar[s]);
      bulk_copy(buf + 4 * kTileBytes, bl + kb * (kTileBytes / 4), kTileBytes, &full_bar[s]);
      bulk_copy(buf + 5 * kTileBytes, bl + rowblk + kb * (kTileBytes / 4), kTileBytes, &full_bar[s]);
      issued = it + 1;
    }
    if (!ok) atomicExch(&fail, 1);
  } else if (threadIdx.x == 32) {
    // MMA issuer
    for (long it = 0; it < nk && ok; it++) {
      const int s = (int)(it % kStages);
      ok = mbar_wait(&full_bar[s], (uint32_t)((it / kStages) & 1));
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t b0 = smem_u32(stage + (long)s * kStageBytes);
      const uint32_t a_hi = b0, a_lo = b0 + kTileBytes, b_hi = b0 + 2 * kTileBytes, b_lo = b0 + 4 * kTileBytes;
#pragma unroll
      for (int kk = 0; kk < kBK / 8; kk++) {  // K = 8 TF32 (32 bytes) per instruction
        const uint32_t off = kk * 32;
        const uint32_t first = (it == 0 && kk == 0) ? 0u : 1u;
        mma_tf32(tmem, sw128_desc(a_hi + off), sw128_desc(b_hi + off), first);
        if (terms > 1) {
          mma_tf32(tmem, sw128_desc(a_hi + off), sw128_desc(b_lo + off), 1u);
          mma_tf32(tmem, sw128_desc(a_lo + off), sw128_desc(b_hi + off), 1u);
        }
      }
      mma_commit(&free_bar[s]);  // the stage is free once these MMAs have read it
    }
    mma_commit(&done_bar);  // and the accumulator is final once every MMA issued is done
    if (!ok) atomicExch(&fail, 1);
  }
  __syncwarp();
  // everyone waits for the accumulator (bounded)
  const bool done = nk > 0 ? mbar_wait(&done_bar, 0u) : true;
  asm volatile("tcgen05.fence::after_thread_sync;");
  __syncthreads();
  if (!done || fail) {
    if (threadIdx.x == 0) {
      atomicExch(status, 1);
      // let the copies this CTA issued land before it leaves (bounded)
      for (long it = (issued > kStages ? issued - kStages : 0); it < issued; it++)
        mbar_wait(&full_bar[it % kStages], (uint32_t)((it / kStages) & 1));
    }
  } else if (nk == 0) {
    const long row = (long)blockIdx.x * kBM + warp * 32 + lane;
    float *dst = part + ((long)blockIdx.z * mp + row) * np + (long)blockIdx.y * kBN;
    for (int j = 0; j < kBN; j++) dst[j] = 0.0f;
  } else {
    // epilogue: warp w reads lanes 32 w .. 32 w + 31 (rows), 32 columns at a time
    const long row = (long)blockIdx.x * kBM + warp * 32 + lane;
    float *dst = part + ((long)blockIdx.z * mp + row) * np + (long)blockIdx.y * kBN;
#pragma unroll 1
    for (int c0 = 0; c0 < kBN; c0 += 32) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
            "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
            "=r"(r[30]), "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 32; j += 4)
        *reinterpret_cast<float4 *>(dst + c0 + j) =
            make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]), __uint_as_float(r[j + 2]),
                        __uint_as_float(r[j + 3]));
    }
  }
  // after a timed-out wait, MMAs this CTA issued may still write the
  // accumulator: the issuing thread waits once more (bounded) before the
  // tensor memory is released; the host treats status = 1 as fatal for the
  // context's tensor-core path
  if (!done && nk > 0 && threadIdx.x == 32) mbar_wait(&done_bar, 0u);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
}

// ---------------------------------------------------------------------------
// tile images.  Source: nrows complex rows of length L (interleaved re, im),
// FP32 or FP64.  Real element k of row i (k < 2L) is, by mode:
//   0: (re, im)        1: (re, -im)        2: (im, re)        3: (-im, re)
// i.e. the row is multiplied into a real dot product with interleaved rows.
// Images cover rows < mp (zero beyond nrows) and k < 32 nkb (zero beyond 2L).
// ---------------------------------------------------------------------------
// round to the nearest TF32 value (10 mantissa bits, ties away from zero) and
// clear the 13 low bits, so that x - tf32(x) is exactly the part the tensor
// core does not see
__device__ __forceinline__ float tf32_round(float x)
{
  uint32_t u = __float_as_uint(x);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
  return __uint_as_float(u);
}

template <typename S>
__global__ void k_tc_images(const S *__restrict__ src, long nrows, long L, int mode, long mp, long nkb, long k0,
                            float *__restrict__ hi, float *__restrict__ lo)
{
  // one thread per (row, 4-element chunk) of the padded operand: 8 chunks per k block
  const long nchunks = mp * nkb * 8;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nchunks; t += (long)gridDim.x * blockDim.x) {
    const long row = t / (nkb * 8);
    const long rem = t - row * nkb * 8;
    const long kb = rem / 8;
    const int c = (int)(rem % 8);  // 16-byte chunk within the 128-byte row
    float h[4], l[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      const long k = k0 + kb * kBK + c * 4 + e;  // real index
      float v = 0.0f;
      if (row < nrows && k < 2 * L) {
        const long p = k >> 1;
        const int part = (int)(k & 1);
        const S re = src[(row * L + p) * 2], im = src[(row * L + p) * 2 + 1];
        S x;
        if (mode == 0) x = part ? im : re;
        else if (mode == 1) x = part ? -im : re;
        else if (mode == 2) x = part ? re : im;
        else x = part ? re : -im;
        v = (float)x;
      }
      h[e] = tf32_round(v);
      l[e] = tf32_round(v - h[e]);
    }
    const long rb = row / kBM;
    const int r = (int)(row % kBM);
    const long img = (rb * nkb + kb) * (kTileBytes / 4);
    const long o = img + (long)r * kBK + (long)((c ^ (r & 7)) * 4);
    *reinterpret_cast<float4 *>(hi + o) = make_float4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<float4 *>(lo + o) = make_float4(l[0], l[1], l[2], l[3]);
  }
}

// out[i][j] = scale * (sum over splits of P0[i][j] (real part), P1 (imaginary))
__global__ void k_tc_reduce(const float *__restrict__ P0, const float *__restrict__ P1, int nsplit, long mp, long np,
                            int m, int n, double scale, double2 *__restrict__ out)
{
  const long total = (long)m * n;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long i = e / n, j = e % n;
    double re = 0, im = 0;
    for (int s = 0; s < nsplit; s++) {
      re += (double)P0[((long)s * mp + i) * np + j];
      im += (double)P1[((long)s * mp + i) * np + j];
    }
    out[e] = make_double2(re * scale, im * scale);
  }
}

}  // namespace tc

// ---------------------------------------------------------------------------
// complex products on the tensor cores
//   out[i][j] = scale * sum_r f(A[i][r]) g(B[j][r])
// conj_a: A conjugated (the Gram form <a_i|b_j>), else the plain product
// (the BSE contraction).  A: ma rows, B: nb rows, L complex columns, in FP32
// or FP64 (converted to FP32, then split into TF32 parts).
// ---------------------------------------------------------------------------
static unsigned grid_of(long n)
{
  long g = (n + 255) / 256;
  if (g > 152L * 16) g = 152L * 16;
  return (unsigned)(g < 1 ? 1 : g);
}

template <typename S>
int tc_complex_nt(fbse_ctx *c, const S *A, int ma, const S *B, int nb, long L, bool conj_a, double scale,
                  double2 *out)
{
  using namespace tc;
  if (c->tc_poisoned)
    return set_err(c, FBSE_ERR_CUDA, "tensor-core path disabled: an earlier tensor-core wait timed out in this context");
  const long mp = ((ma + kBM - 1) / kBM) * kBM;
  const long np = ((nb + kBN - 1) / kBN) * kBN;
  const long nkb_all = (2 * L + kBK - 1) / kBK;
  // the images of a K chunk (A hi/lo, two B modes hi/lo) within 24 GB
  // (fbse_tuning.tc_image_bytes sets another budget)
  const double budget = c->tune.tc_image_bytes > 0 ? c->tune.tc_image_bytes : 24.0e9;
  long nkb_c = std::max<long>(1, (long)(budget / ((2.0 * mp + 4.0 * np) * kBK * 4.0)));
  if (nkb_c > nkb_all) nkb_c = nkb_all;
  const long nchunk = (nkb_all + nkb_c - 1) / nkb_c;
  // splits per chunk: at most 64 k blocks (768 accumulating MMAs) per split --
  // the tensor core's FP32 accumulation truncates, so its error grows with the
  // number of MMAs summed into one accumulator -- with the FP32 partials of
  // all chunks within 16 GB and at least two CTAs per SM
  const long tiles = (mp / kBM) * (np / kBN);
  long sps = std::max<long>(1, (nkb_c + 63) / 64);
  const long max_total = std::max<long>(nchunk, (long)(16.0e9 / (2.0 * 4.0 * mp * np)));
  if (sps * nchunk > max_total) sps = std::max<long>(1, max_total / nchunk);
  const long want = std::min<long>(nkb_c, (2 * 152 + tiles - 1) / tiles);
  if (sps < want) sps = want;
  const long kbs = (nkb_c + sps - 1) / sps;
  sps = (nkb_c + kbs - 1) / kbs;
  const long nsplit = sps * nchunk;
  const size_t img_a = (size_t)mp * nkb_c * kBK, img_b = (size_t)np * nkb_c * kBK;  // floats
  const size_t part_n = (size_t)nsplit * mp * np;
  // operand images, partial tiles and the wait status, kept in the context
  // between calls (grown on demand, released by fbse_destroy)
  const size_t need = (2 * img_a + 4 * img_b + 2 * part_n) * sizeof(float) + 256;
  void *scratch = nullptr;
  if (cached(c, kSlotTc, need, &scratch)) return set_err(c, FBSE_ERR_OOM, "tensor-core GEMM scratch");
  float *buf = static_cast<float *>(scratch);
  int *status = reinterpret_cast<int *>(static_cast<char *>(scratch) + need - 256);
  float *ah = buf, *al = ah + img_a;
  float *b0h = al + img_a, *b0l = b0h + img_b, *b1h = b0l + img_b, *b1l = b1h + img_b;
  float *p0 = b1l + img_b, *p1 = p0 + part_n;
  int rc = FBSE_OK;
  // launch errors end the call through the cleanup below (no early return)
  auto launched = [&](int nk) {
    FBSE_COUNT(nk);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, std::string("tensor-core launch: ") + cudaGetErrorString(e));
    return e == cudaSuccess;
  };
  const int terms = 3;  // hi x hi + hi x lo + lo x hi
  do {
    if (cudaMemsetAsync(status, 0, sizeof(int), c->stream) != cudaSuccess) { rc = set_err(c, FBSE_ERR_CUDA, "memset"); break; }
    const size_t smem = (size_t)kStages * kStageBytes + 1024;
    if (cudaFuncSetAttribute(tc::k_tc_gemm_nt, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess) { rc = set_err(c, FBSE_ERR_CUDA, "tensor-core GEMM attribute"); break; }
    // real dot products of interleaved rows:
    //   plain  re = A(re, im) . B(re, -im)   im = A(re, im) . B(im, re)
    //   conj_a re = A(re, im) . B(re, im)    im = A(re, -im) . B(im, re)
    const int mb0 = conj_a ? 0 : 1, mb1 = 2;
    for (long ch = 0; ch < nchunk && !rc; ch++) {
      const long k0 = ch * nkb_c * kBK;
      const long nkb = std::min<long>(nkb_c, nkb_all - ch * nkb_c);
      const long nsp = (nkb + kbs - 1) / kbs;
      float *q0 = p0 + (size_t)ch * sps * mp * np, *q1 = p1 + (size_t)ch * sps * mp * np;
      if (nsp < sps) {  // a short last chunk: its unused partial slots must read as zero
        const size_t tail = (size_t)(sps - nsp) * mp * np * sizeof(float);
        if (cudaMemsetAsync(q0 + (size_t)nsp * mp * np, 0, tail, c->stream) != cudaSuccess ||
            cudaMemsetAsync(q1 + (size_t)nsp * mp * np, 0, tail, c->stream) != cudaSuccess) {
          rc = set_err(c, FBSE_ERR_CUDA, "tensor-core product: partial clear");
          break;
        }
      }
      tc::k_tc_images<S><<<grid_of(mp * nkb * 8), 256, 0, c->stream>>>(A, ma, L, 0, mp, nkb, k0, ah, al);
      tc::k_tc_images<S><<<grid_of(np * nkb * 8), 256, 0, c->stream>>>(B, nb, L, mb0, np, nkb, k0, b0h, b0l);
      tc::k_tc_images<S><<<grid_of(np * nkb * 8), 256, 0, c->stream>>>(B, nb, L, mb1, np, nkb, k0, b1h, b1l);
      if (!launched(3)) break;
      dim3 g((unsigned)(mp / kBM), (unsigned)(np / kBN), (unsigned)nsp);
      tc::k_tc_gemm_nt<<<g, 128, smem, c->stream>>>(ah, al, b0h, b0l, nkb, kbs, q0, mp, np, terms, status);
      if (!launched(1)) break;
      if (conj_a) {
        tc::k_tc_images<S><<<grid_of(mp * nkb * 8), 256, 0, c->stream>>>(A, ma, L, 1, mp, nkb, k0, ah, al);
        if (!launched(1)) break;
      }
      tc::k_tc_gemm_nt<<<g, 128, smem, c->stream>>>(ah, al, b1h, b1l, nkb, kbs, q1, mp, np, terms, status);
      if (!launched(1)) break;
    }
    if (rc) break;
    tc::k_tc_reduce<<<grid_of((long)ma * nb), 256, 0, c->stream>>>(p0, p1, (int)nsplit, mp, np, ma, nb, scale, out);
    if (!launched(1)) break;
    int hs = 0;
    if (d2h(c->stream, &hs, status, sizeof(int)) != cudaSuccess) { rc = set_err(c, FBSE_ERR_CUDA, "tensor-core GEMM"); break; }
    if (hs) {
      c->tc_poisoned = 1;
      rc = set_err(c, FBSE_ERR_NOCONV, "tensor-core GEMM: a wait timed out");
    }
  } while (0);
  cudaStreamSynchronize(c->stream);
  return rc;
}

template int tc_complex_nt<float>(fbse_ctx *, const float *, int, const float *, int, long, bool, double, double2 *);
template int tc_complex_nt<double>(fbse_ctx *, const double *, int, const double *, int, long, bool, double,
                                   double2 *);

}  // namespace fbse
