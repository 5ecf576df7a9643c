// H psi for 128 x 128 x nz grids in FP32 with the projectors fused into the
// xy plane passes of the 3D FFT.  Included by hpsi_fused.cu.
//
// The separate projector kernels read psi and read-modify-write H psi at the
// covered grid points (about half the grid here) with dependent index -> value
// loads; here the plane passes do that work on the plane they hold in shared
// memory:
//   plane_fwd(b, z)  load plane z of block b (state x spin); gather the
//                    projector sums of the plane's table entries from shared
//                    memory (one partial per segment of entries of one atom);
//                    x then y forward; store
//   (z pass)         the existing z lines kernel: forward, min(k^2/2, KE_max)/N,
//                    inverse
//   proj_red(s, k)   sum the partials of atoms 32k .. 32k+31 of state s over
//                    their segments, apply L.S (SO) or the channel sign (NL)
//   plane_inv(b, z)  y then x inverse; add the projector terms of the plane's
//                    entries in shared memory; epilogue
//                    out = a (result + V psi) + b psi, stored once
// The plane launches run z-major (CTA i: plane i / nblk of block i % nblk), so
// the CTAs that read one plane's slice of the table run together and find it
// in L2.  The FFT arithmetic is that of k_plane_fast (same butterflies,
// twiddles and order).  The projector terms are summed in a fixed order (per
// segment in entry order, segments of an atom in plane order, entries of a
// grid point in increasing atom order), so H psi is the same on every run and
// for every batch size; it differs from the separate kernels' in rounding only.
#pragma once

namespace fbse {
namespace fused {

// plane edge, atoms whose spheres meet one plane, entries of one grid point
// (fbse_internal.cuh, shared with the table builder)
constexpr int N = kPipeN, P = 8, Q = 16, PITCH = N + 8, THREADS = N * P;
constexpr int kPlaneAtoms = kPipePlaneAtoms, kMaxLayers = kPipeMaxLayers;

// plane-major projector table (ProjDev::fz_*): entries of plane z in the
// order (layer, atom slot, grid point); layer = rank of the entry's atom among
// the atoms covering its point, so a layer holds each point at most once
struct ProjTable {
  const unsigned *ent;  // x | y << 7 | slot << 16
  const float *y;       // [3][nent]: Y_1,-1 = (y0, y1), Y_10 = (y2, 0), Y_1,1 = (-y0, y1)
  const float *so, *nl;  // [nproj][nent]
  const int *lay;        // [nz][kMaxLayers + 1]: entry offsets of the layers
  const int *atoms;      // [nz][kPlaneAtoms]: atom of each slot
  const int *natoms;     // [nz]
  const int *seg_beg;    // [nseg + 1]
  const int *plane_seg;  // [nz + 1]: first segment of each plane
  const int *aseg_beg, *aseg;  // atom -> its segments in increasing order
  const double2 *LS;
  const int *sgn;
  long nent, nseg, nat;
  int nproj;
};

struct FusedArgs {
  const float2 *in;
  float2 *out, *wk, *coef;
  float *part;
  const float *pot;
  const float2 *rx;
  ProjTable tb;
  long ngrid;
  int nblk, nspin;
  float ca, cb, dv;
};

// L2 eviction priority of the projector table: each plane's slice is read by
// the nblk CTAs of that plane, so it is loaded with an evict-last policy
__device__ __forceinline__ unsigned long long pol_keep()
{
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
// read-only table entries, kept in L2
__device__ __forceinline__ float ld_tab(const float *p, unsigned long long pol)
{
  float v;
  asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ unsigned ld_tab(const unsigned *p, unsigned long long pol)
{
  unsigned v;
  asm("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}

// sum of v[i] over the 32 lanes, lane l left with the total of v[l] (31 shuffles)
__device__ __forceinline__ float transpose_sum(float (&v)[32], int lane)
{
#pragma unroll
  for (int h = 16; h >= 1; h >>= 1) {
    const bool up = (lane & h) != 0;
#pragma unroll
    for (int i = 0; i < h; i++) {
      const float send = up ? v[i] : v[i + h];
      const float keep = up ? v[i + h] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, h);
    }
  }
  return v[0];
}

template <int CH> struct Chan {
  static constexpr int n = (CH & 1) + ((CH >> 1) & 1);
};

// ---------------------------------------------------------------------------
// plane_fwd(b, z)
// ---------------------------------------------------------------------------
template <int CH>
__device__ __forceinline__ void plane_fwd(const FusedArgs &A, float2 *S, const float2 *twx, int b, int z,
                                         unsigned long long keep)
{
  constexpr int NCH = Chan<CH>::n;
  const int tid = threadIdx.x;
  const long pl = (long)z * N * N;
  const float2 *src = A.in + (long)b * A.ngrid + pl;
  float2 *dst = A.wk + (long)b * A.ngrid + pl;
  const int rr = tid / P, rt = tid % P;
  const int cw = tid >> 5, ct = cw % P, cc = (cw / P) * 32 + (tid & 31);
  float2 v[Q];
#pragma unroll
  for (int m = 0; m < Q; m++) v[m] = src[rr * N + rt + P * m];
  if constexpr (CH != 0) {
#pragma unroll
    for (int m = 0; m < Q; m++) S[rr * PITCH + rt + P * m] = v[m];
    __syncthreads();
    // projector sums of this plane's segments: warp w takes segments w, w + 32, ...
    const ProjTable &tb = A.tb;
    const int lane = tid & 31;
    const int sg1 = tb.plane_seg[z + 1];
    for (int sg = tb.plane_seg[z] + (tid >> 5); sg < sg1; sg += 32) {
      const int e0 = tb.seg_beg[sg], e1 = tb.seg_beg[sg + 1];
#pragma unroll
      for (int k = 0; k < 2; k++) {
        if (!(CH & (1 << k))) continue;
        const float *rad = k == 0 ? tb.so : tb.nl;
        float acc[32];
#pragma unroll
        for (int i = 0; i < 32; i++) acc[i] = 0.f;
        for (int e = e0 + lane; e < e1; e += 32) {
          const unsigned pk = ld_tab(tb.ent + e, keep);
          const float2 ps = S[((pk >> 7) & 127) * PITCH + (pk & 127)];
          const float y0 = ld_tab(tb.y + e, keep), y1 = ld_tab(tb.y + tb.nent + e, keep),
                      y2 = ld_tab(tb.y + 2 * tb.nent + e, keep);
          // psi conj(Y_m)
          float tr[3], ti[3];
          tr[0] = ps.x * y0 + ps.y * y1;
          ti[0] = ps.y * y0 - ps.x * y1;
          tr[1] = ps.x * y2;
          ti[1] = ps.y * y2;
          tr[2] = -ps.x * y0 + ps.y * y1;
          ti[2] = -ps.y * y0 - ps.x * y1;
#pragma unroll
          for (int p = 0; p < 5; p++) {
            if (p >= tb.nproj) continue;
            const float bp = ld_tab(rad + p * tb.nent + e, keep);
#pragma unroll
            for (int m = 0; m < 3; m++) {
              acc[2 * (p * 3 + m)] += bp * tr[m];
              acc[2 * (p * 3 + m) + 1] += bp * ti[m];
            }
          }
        }
        const float tot = transpose_sum(acc, lane);
        const int slot = (CH == 3) ? k : 0;
        if (lane < 30) A.part[((long)b * tb.nseg + sg) * (30 * NCH) + slot * 30 + lane] = tot;
      }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < Q; m++) v[m] = S[rr * PITCH + rt + P * m];
    __syncwarp();
  }
  // rows, forward (k_plane_fast MODE 0)
  fast::inner_q<float, N, false>(v, rt, twx);
  float2 *row = S + rr * PITCH;
  fast::row_exchange<float, N>(row, v, rt);
  fast::outer_p<float, N, false>(v);
#pragma unroll
  for (int j = 0; j < Q / P; j++)
#pragma unroll
    for (int k2 = 0; k2 < P; k2++) row[rt + P * j + Q * k2] = v[j * P + k2];
  __syncthreads();
  // columns, forward
#pragma unroll
  for (int m = 0; m < Q; m++) v[m] = S[(ct + P * m) * PITCH + cc];
  fast::inner_q<float, N, false>(v, ct, twx);
  __syncthreads();
#pragma unroll
  for (int k1 = 0; k1 < Q; k1++) S[(k1 * P + ct) * PITCH + cc] = v[k1];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < Q / P; j++)
#pragma unroll
    for (int s = 0; s < P; s++) v[j * P + s] = S[((ct + P * j) * P + s) * PITCH + cc];
  fast::outer_p<float, N, false>(v);
#pragma unroll
  for (int j = 0; j < Q / P; j++)
#pragma unroll
    for (int k2 = 0; k2 < P; k2++) dst[(long)(ct + P * j + Q * k2) * N + cc] = v[j * P + k2];
}

// ---------------------------------------------------------------------------
// proj_red(st, k): warp w sums atom 32 k + w over its segments, then L.S / sign;
// coef[((st nat + a) 2 + ch) 30 + p 6 + j] as k_proj_gather writes it
// ---------------------------------------------------------------------------
template <int CH>
__device__ __forceinline__ void proj_red(const FusedArgs &A, float2 *S, int st, int k)
{
  constexpr int NCH = Chan<CH>::n;
  const ProjTable &tb = A.tb;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long a = (long)k * 32 + w;
  if (a >= tb.nat) return;
  float2 *cf = S + w * 32;
  const int ns = A.nspin, npj = tb.nproj;
#pragma unroll
  for (int kk = 0; kk < 2; kk++) {
    if (!(CH & (1 << kk))) continue;
    const int slot = (CH == 3) ? kk : 0;
    if (lane < 15 * ns) {
      const int sp = lane / 15, q = lane % 15;
      const long blk = (long)st * ns + sp;
      float sr = 0.f, si = 0.f;
      for (int i = tb.aseg_beg[a]; i < tb.aseg_beg[a + 1]; i++) {
        const float *pp = A.part + (blk * tb.nseg + tb.aseg[i]) * (30 * NCH) + slot * 30 + 2 * q;
        sr += pp[0];
        si += pp[1];
      }
      cf[sp * 15 + q] = make_float2(sr * A.dv, si * A.dv);
    }
    __syncwarp();
    if (lane < 30) {
      const int p = lane / 6, j = lane % 6;
      float2 d = make_float2(0.f, 0.f);
      if (kk == 0) {
        // d[p][j] = sum_j' LS[j'][j] c[p][j'], j' = 3 s' + m'   (phamiltonian.c:249-290)
        for (int jp = 0; jp < 3 * ns; jp++) {
          const double2 l = tb.LS[jp * 6 + j];
          const float2 c = cf[(jp / 3) * 15 + p * 3 + jp % 3];
          d.x += (float)l.x * c.x - (float)l.y * c.y;
          d.y += (float)l.x * c.y + (float)l.y * c.x;
        }
      } else if (j / 3 < ns) {
        const float sg = (p < npj) ? (float)tb.sgn[a * npj + p] : 0.f;
        d = cscale<float>(cf[(j / 3) * 15 + p * 3 + j % 3], sg);
      }
      A.coef[((st * tb.nat + a) * 2 + kk) * 30 + lane] = d;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// plane_inv(b, z)
// ---------------------------------------------------------------------------
template <int CH>
__device__ __forceinline__ void plane_inv(const FusedArgs &A, float2 *S, float2 *dsm, const float2 *twx, int b, int z,
                                         unsigned long long keep)
{
  constexpr int NCH = Chan<CH>::n;
  const int tid = threadIdx.x;
  const long pl = (long)z * N * N;
  const float2 *src = A.wk + (long)b * A.ngrid + pl;
  const int st = b / A.nspin, sp = b % A.nspin;
  const ProjTable &tb = A.tb;
  if constexpr (CH != 0) {
    // this plane's coefficients for output spin sp: dsm[(slot NCH + c) 15 + p 3 + m]
    const int na = tb.natoms[z];
    for (int i = tid; i < na * 15 * NCH; i += THREADS) {
      const int sl = i / (15 * NCH), r = i % (15 * NCH), c = r / 15, q = r % 15;
      const int ch = (CH == 3) ? c : (CH == 1 ? 0 : 1);
      const long a = tb.atoms[z * kPlaneAtoms + sl];
      dsm[i] = A.coef[((st * tb.nat + a) * 2 + ch) * 30 + (q / 3) * 6 + 3 * sp + q % 3];
    }
  }
  const int rr = tid / P, rt = tid % P;
  const int cw = tid >> 5, ct = cw % P, cc = (cw / P) * 32 + (tid & 31);
  float2 v[Q];
  // columns, inverse (k_plane_fast MODE 1)
#pragma unroll
  for (int m = 0; m < Q; m++) v[m] = src[(long)(ct + P * m) * N + cc];
  fast::inner_q<float, N, true>(v, ct, twx);
#pragma unroll
  for (int k1 = 0; k1 < Q; k1++) S[(k1 * P + ct) * PITCH + cc] = v[k1];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < Q / P; j++)
#pragma unroll
    for (int s = 0; s < P; s++) v[j * P + s] = S[((ct + P * j) * P + s) * PITCH + cc];
  fast::outer_p<float, N, true>(v);
  __syncthreads();
#pragma unroll
  for (int j = 0; j < Q / P; j++)
#pragma unroll
    for (int k2 = 0; k2 < P; k2++) S[(ct + P * j + Q * k2) * PITCH + cc] = v[j * P + k2];
  __syncthreads();
  // rows, inverse
  float2 *row = S + rr * PITCH;
#pragma unroll
  for (int m = 0; m < Q; m++) v[m] = row[rt + P * m];
  __syncwarp();
  fast::inner_q<float, N, true>(v, rt, twx);
  fast::row_exchange<float, N>(row, v, rt);
  fast::outer_p<float, N, true>(v);
  if constexpr (CH != 0) {
    // the plane in shared memory, then the projector terms layer by layer
    // (a layer holds each grid point once, so its updates do not collide)
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int k2 = 0; k2 < P; k2++) row[rt + P * j + Q * k2] = v[j * P + k2];
    __syncthreads();
    const int *lay = tb.lay + z * (kMaxLayers + 1);
    for (int L = 0; L < kMaxLayers; L++) {
      const int e0 = lay[L], e1 = lay[L + 1];
      if (e0 == e1) break;
      for (int e = e0 + tid; e < e1; e += THREADS) {
        const unsigned pk = ld_tab(tb.ent + e, keep);
        const float y0 = ld_tab(tb.y + e, keep), y1 = ld_tab(tb.y + tb.nent + e, keep),
                    y2 = ld_tab(tb.y + 2 * tb.nent + e, keep);
        const float2 *d = dsm + (pk >> 16) * (15 * NCH);
        // q_m = sum_p b_p d[p][3 sp + m] over the channels, p in increasing order
        float qr[3] = {0.f, 0.f, 0.f}, qi[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int p = 0; p < 5; p++) {
          if (p >= tb.nproj) continue;
          const float bs = (CH & 1) ? ld_tab(tb.so + p * tb.nent + e, keep) : 0.f;
          const float bn = (CH & 2) ? ld_tab(tb.nl + p * tb.nent + e, keep) : 0.f;
#pragma unroll
          for (int m = 0; m < 3; m++) {
            if (CH & 1) {
              const float2 r = d[p * 3 + m];
              qr[m] += bs * r.x;
              qi[m] += bs * r.y;
            }
            if (CH & 2) {
              const float2 r = d[(NCH - 1) * 15 + p * 3 + m];
              qr[m] += bn * r.x;
              qi[m] += bn * r.y;
            }
          }
        }
        // sum_m Y_m q_m
        float vr = y0 * qr[0] - y1 * qi[0];
        float vi = y0 * qi[0] + y1 * qr[0];
        vr += y2 * qr[1];
        vi += y2 * qi[1];
        vr += -y0 * qr[2] - y1 * qi[2];
        vi += -y0 * qi[2] + y1 * qr[2];
        float2 *o = S + ((pk >> 7) & 127) * PITCH + (pk & 127);
        float2 cur = *o;
        cur.x += vr;
        cur.y += vi;
        *o = cur;
      }
      __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < Q / P; j++)
#pragma unroll
      for (int k2 = 0; k2 < P; k2++) v[j * P + k2] = row[rt + P * j + Q * k2];
  }
  // epilogue: out = a (result + V psi) + b psi
  const long gb = (long)b * A.ngrid + pl;
#pragma unroll
  for (int j = 0; j < Q / P; j++)
#pragma unroll
    for (int k2 = 0; k2 < P; k2++) {
      const long o = (long)rr * N + rt + P * j + Q * k2;
      float2 r = v[j * P + k2];
      const float2 ph = A.in[gb + o];
      if (A.pot) {
        const float V = A.pot[pl + o];
        r.x += V * ph.x;
        r.y += V * ph.y;
      }
      __stcs(A.out + gb + o, make_float2(A.ca * r.x + A.cb * ph.x, A.ca * r.y + A.cb * ph.y));
    }
}

template <int CH>
__global__ void __launch_bounds__(THREADS, 1) k_plane_proj_fwd(const __grid_constant__ FusedArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *twx = reinterpret_cast<float2 *>(smem_raw);
  float2 *S = twx + N;
  fast::load_tw2<float, N>(twx, A.rx);
  const unsigned long long keep = pol_keep();
  __syncthreads();
  plane_fwd<CH>(A, S, twx, (int)(blockIdx.x % A.nblk), (int)(blockIdx.x / A.nblk), keep);
}

template <int CH>
__global__ void __launch_bounds__(THREADS, 1) k_proj_red(const __grid_constant__ FusedArgs A)
{
  __shared__ float2 cf[32 * 32];
  proj_red<CH>(A, cf, (int)blockIdx.y, (int)blockIdx.x);
}

template <int CH>
__global__ void __launch_bounds__(THREADS, 1) k_plane_proj_inv(const __grid_constant__ FusedArgs A)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2 *twx = reinterpret_cast<float2 *>(smem_raw);
  float2 *S = twx + N;
  float2 *dsm = S + N * PITCH;
  fast::load_tw2<float, N>(twx, A.rx);
  const unsigned long long keep = pol_keep();
  __syncthreads();
  plane_inv<CH>(A, S, dsm, twx, (int)(blockIdx.x % A.nblk), (int)(blockIdx.x / A.nblk), keep);
}

template <int CH> constexpr size_t plane_proj_smem(bool inv)
{
  return (size_t)(N + N * PITCH + (inv ? kPlaneAtoms * 15 * Chan<CH>::n : 0)) * sizeof(float2);
}

}  // namespace fused
}  // namespace fbse
