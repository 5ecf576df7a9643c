// H psi on the GPU: local potential, spin-orbit and
// nonlocal projectors, and the Newton scale-and-shift of p_hnorm.
//
// Projectors replace p_spin_orbit_proj_pot and p_nonlocal_proj_pot
// (filter_mpi/phamiltonian.c:140-312, 316-444; k = 0).  For one atom a and
// radial channel p the reference forms
//   c[p][j'] = dv sum_pts b_p(r) conj(Y_m'(r)) psi_s'(r),   j' = 3 s' + m'
// and scatters b_p(r) Y_m(r) sum_j' LS[j'][j] c[p][j'] into spin s of the
// output (SO); the NL operator is the same with b^NL_p, a sign per channel and
// no spin mixing.  Here one CTA per (atom, channel, group of states) gathers
// the coefficients with one warp per (state, spin) (register accumulation,
// warp reduction; the warps of a CTA share every table entry through L1) and
// applies L.S (or the NL sign).  The scatter runs one thread per grid point
// covered by any sphere (overlapping spheres of neighbouring atoms make it a
// reduction, which the reference does with "omp atomic",
// phamiltonian.c:295-303): each point's entries are summed in a fixed order,
// so H psi is bit-identical from run to run.
#include <cstdlib>

#include "fbse_internal.cuh"

namespace fbse {

// Table entries i = a*npts + e in structure-of-arrays form (one coalesced
// load per quantity for 32 consecutive entries): y1[m*ne + i] = Y_1m as a
// complex, sop/nlp[p*ne + i] = radial value of channel p.
template <typename T> struct ProjView {
  const int *cnt, *jxyz, *sgn;
  const C<T> *y1;
  const T *sop, *nlp;
  const double2 *LS;
  long npts, ne;
  int nproj;
};

template <typename T> static ProjView<T> view(fbse_ctx *c);
template <> ProjView<double> view<double>(fbse_ctx *c)
{
  const ProjDev &p = c->proj;
  return {p.nl_cnt, p.jxyz, p.sgn, reinterpret_cast<const double2 *>(p.y1), p.sop, p.nlp, p.LS, p.npts,
          p.nat * p.npts, p.nproj};
}
template <> ProjView<float> view<float>(fbse_ctx *c)
{
  const ProjDev &p = c->proj;
  return {p.nl_cnt, p.jxyz, p.sgn, reinterpret_cast<const float2 *>(p.y1f), p.sopf, p.nlpf, p.LS, p.npts,
          p.nat * p.npts, p.nproj};
}

constexpr int kSW = 4;              // warps per CTA
constexpr int kProjThreads = 32 * kSW;
constexpr int kNC = 30;             // 5 radial channels x (2 spins x 3 m)

// gather: one warp per (state, spin s'); each lane accumulates the 15
// coefficients b_p conj(Y_m) psi_s' of its points, kGU points per iteration so
// that the dependent loads (grid index, then psi) of several points are in
// flight together; the grid indices of the next iteration are loaded before
// the current iteration's arithmetic, so only the psi load is on the critical
// path.  W warps per CTA (W / nspin states) share every table entry through
// L1.  Then L.S (or the NL sign) per state:
//   coef[((st*nat + a)*2 + ch)*30 + p*6 + j]
template <typename T, int kGU, int MINB, int W>
__global__ void __launch_bounds__(32 * W, MINB) k_proj_gather(const C<T> *__restrict__ psi, C<T> *__restrict__ coef,
                                                              ProjView<T> pv, long nat, long nstates, long ngrid,
                                                              int nspin, int ch0, double dv)
{
  const long a = blockIdx.x;
  const int ch = ch0 + blockIdx.y;  // 0: SO, 1: NL
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int spc = W / nspin;  // states per CTA
  const long st = (long)blockIdx.z * spc + wid / nspin;
  const int sp = wid % nspin;
  const bool live = st < nstates;
  const int np = pv.cnt[a];
  const C<T> *ps = psi + (live ? st : 0) * nspin * ngrid + (long)sp * ngrid;
  const T *rad = (ch == 0) ? pv.sop : pv.nlp;
  const int npj = pv.nproj;
  const long ebase = a * pv.npts;
  T acc[30];
#pragma unroll
  for (int i = 0; i < 30; i++) acc[i] = T(0);
  if (live) {
    int jn[kGU];
#pragma unroll
    for (int u = 0; u < kGU; u++) {
      const int g = lane + 32 * u;
      jn[u] = g < np ? pv.jxyz[ebase + g] : -1;
    }
    for (int g0 = lane; g0 < np; g0 += 32 * kGU) {
      int jx[kGU];
      C<T> v[kGU];
#pragma unroll
      for (int u = 0; u < kGU; u++) {
        jx[u] = jn[u];
        v[u] = jx[u] >= 0 ? ps[jx[u]] : mk<T>(T(0), T(0));
      }
#pragma unroll
      for (int u = 0; u < kGU; u++) {
        const int g = g0 + 32 * (kGU + u);
        jn[u] = g < np ? pv.jxyz[ebase + g] : -1;
      }
#pragma unroll
      for (int u = 0; u < kGU; u++) {
        if (jx[u] < 0) continue;
        const long e = ebase + g0 + 32 * u;
        T b[5];
#pragma unroll
        for (int p = 0; p < 5; p++) b[p] = (p < npj) ? rad[p * pv.ne + e] : T(0);
#pragma unroll
        for (int m = 0; m < 3; m++) {
          const C<T> y = pv.y1[m * pv.ne + e];
          // psi * conj(Y)
          const T tr = v[u].x * y.x + v[u].y * y.y;
          const T ti = v[u].y * y.x - v[u].x * y.y;
#pragma unroll
          for (int p = 0; p < 5; p++) {
            acc[2 * (p * 3 + m)] += b[p] * tr;
            acc[2 * (p * 3 + m) + 1] += b[p] * ti;
          }
        }
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 30; i++) {
    T x = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    acc[i] = x;
  }
  __shared__ C<T> cf[W][15];
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < 15; i++) cf[wid][i] = mk<T>(acc[2 * i] * (T)dv, acc[2 * i + 1] * (T)dv);
  }
  __syncthreads();
  for (int o = threadIdx.x; o < spc * kNC; o += blockDim.x) {
    const int ls = o / kNC, q = o % kNC;
    const long sg = (long)blockIdx.z * spc + ls;
    if (sg >= nstates) continue;
    const int p = q / 6, j = q % 6;
    C<T> d = mk<T>(0, 0);
    if (ch == 0) {
      // d[p][j] = sum_j' LS[j'][j] c[p][j'], j' = 3 s' + m'   (phamiltonian.c:249-290)
      for (int jp = 0; jp < 3 * nspin; jp++) {
        const double2 l = pv.LS[jp * 6 + j];
        const C<T> cc = cf[ls * nspin + jp / 3][p * 3 + jp % 3];
        d.x += (T)l.x * cc.x - (T)l.y * cc.y;
        d.y += (T)l.x * cc.y + (T)l.y * cc.x;
      }
    } else if (j / 3 < nspin) {
      // sign of the channel (phamiltonian.c:399-401), block diagonal in spin
      const T sgn = (p < npj) ? (T)pv.sgn[a * npj + p] : T(0);
      d = cscale<T>(cf[ls * nspin + j / 3][p * 3 + j % 3], sgn);
    }
    coef[((sg * nat + a) * 2 + ch) * kNC + q] = d;
  }
}

// point-major view of the table for the scatter (ProjDev::cov_j ...)
template <typename T> struct PtView {
  const int *cov_j, *cov_beg, *atom;
  const C<T> *y1;
  const T *sop, *nlp;
  long ncov, nent;
  int nproj;
};

template <typename T> static PtView<T> ptview(fbse_ctx *c);
template <> PtView<double> ptview<double>(fbse_ctx *c)
{
  const ProjDev &p = c->proj;
  return {p.cov_j, p.cov_beg, p.pe_atom, reinterpret_cast<const double2 *>(p.pe_y1), p.pe_sop, p.pe_nlp, p.ncov,
          p.nent, p.nproj};
}
template <> PtView<float> ptview<float>(fbse_ctx *c)
{
  const ProjDev &p = c->proj;
  return {p.cov_j, p.cov_beg, p.pe_atom, reinterpret_cast<const float2 *>(p.pe_y1f), p.pe_sopf, p.pe_nlpf, p.ncov,
          p.nent, p.nproj};
}

// scatter: out_s(r) += scale * sum_(a covering r) sum_m Y_m(r) sum_p b_p(r) d_a[p][3 s + m]
// over the active channels.  One thread owns one covered point for kG states:
// it sums the point's entries in increasing atom order and writes the point
// once, so the result is the same on every run and for every batch size (the
// reference adds with "omp atomic", phamiltonian.c:295-303, whose order
// varies).  The lanes of a warp mostly share their atom, so the coefficient
// loads are broadcasts.
// the six coefficients d[p][0..5] (j = 3 s + m) of one channel, 16-byte loads
__device__ __forceinline__ void ld_row6(const float2 *d, float2 q[6])
{
  const float4 *v = reinterpret_cast<const float4 *>(d);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float4 t = __ldg(v + i);
    q[2 * i] = make_float2(t.x, t.y);
    q[2 * i + 1] = make_float2(t.z, t.w);
  }
}
__device__ __forceinline__ void ld_row6(const double2 *d, double2 q[6])
{
#pragma unroll
  for (int i = 0; i < 6; i++) q[i] = __ldg(d + i);
}

template <typename T, bool SO, bool NL, int kG>
__global__ void __launch_bounds__(256) k_proj_scatter(C<T> *__restrict__ out, const C<T> *__restrict__ coef,
                                                      PtView<T> pv, long nat, long nstates, long ngrid, int nspin,
                                                      T scale)
{
  const long k = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (k >= pv.ncov) return;
  const long s0 = (long)blockIdx.y * kG;
  const int ng = (int)(nstates - s0 < kG ? nstates - s0 : kG);
  const long j = pv.cov_j[k];
  const int e0 = pv.cov_beg[k], e1 = pv.cov_beg[k + 1];
  const int npj = pv.nproj;
  // the outputs this thread updates, loaded before the sums so that their
  // DRAM latency overlaps the coefficient work
  C<T> o[kG][2];
#pragma unroll
  for (int g = 0; g < kG; g++)
#pragma unroll
    for (int s = 0; s < 2; s++)
      if (g < ng && s < nspin) o[g][s] = out[((s0 + g) * nspin + s) * ngrid + j];
  T ar[kG][2], ai[kG][2];
#pragma unroll
  for (int g = 0; g < kG; g++) {
    ar[g][0] = ar[g][1] = T(0);
    ai[g][0] = ai[g][1] = T(0);
  }
  for (int e = e0; e < e1; e++) {
    const long a = pv.atom[e];
    T yr[3], yi[3];
#pragma unroll
    for (int m = 0; m < 3; m++) {
      const C<T> y = pv.y1[m * pv.nent + e];
      yr[m] = y.x;
      yi[m] = y.y;
    }
    T bs[5], bn[5];
#pragma unroll
    for (int p = 0; p < 5; p++) {
      bs[p] = (SO && p < npj) ? pv.sop[p * pv.nent + e] : T(0);
      bn[p] = (NL && p < npj) ? pv.nlp[p * pv.nent + e] : T(0);
    }
#pragma unroll
    for (int g = 0; g < kG; g++) {
      if (g >= ng) continue;
      const C<T> *d = coef + (((s0 + g) * nat + a) * 2) * kNC;
      // q[j] = sum_p b_p d[p][j], j = 3 s + m, p in increasing order
      T qr[6], qi[6];
#pragma unroll
      for (int q = 0; q < 6; q++) qr[q] = qi[q] = T(0);
#pragma unroll
      for (int p = 0; p < 5; p++) {
        if (p >= npj) continue;
        C<T> rs[6], rn[6];
        if (SO) ld_row6(d + p * 6, rs);
        if (NL) ld_row6(d + kNC + p * 6, rn);
#pragma unroll
        for (int q = 0; q < 6; q++) {
          if (SO) {
            qr[q] += bs[p] * rs[q].x;
            qi[q] += bs[p] * rs[q].y;
          }
          if (NL) {
            qr[q] += bn[p] * rn[q].x;
            qi[q] += bn[p] * rn[q].y;
          }
        }
      }
#pragma unroll
      for (int s = 0; s < 2; s++) {
        if (s >= nspin) continue;
        T vr = 0, vi = 0;
#pragma unroll
        for (int m = 0; m < 3; m++) {
          vr += yr[m] * qr[3 * s + m] - yi[m] * qi[3 * s + m];
          vi += yr[m] * qi[3 * s + m] + yi[m] * qr[3 * s + m];
        }
        ar[g][s] += vr;
        ai[g][s] += vi;
      }
    }
  }
#pragma unroll
  for (int g = 0; g < kG; g++) {
#pragma unroll
    for (int s = 0; s < 2; s++) {
      if (g >= ng || s >= nspin) continue;
      C<T> v = o[g][s];
      v.x += scale * ar[g][s];
      v.y += scale * ai[g][s];
      out[((s0 + g) * nspin + s) * ngrid + j] = v;
    }
  }
}

// scatter over chunks of covered points (ProjDev::chunk_beg ...): one CTA
// per chunk (at most kScatterChunkPoints points, kScatterChunkAtoms atoms),
// one thread per point, all states in groups of kG.  The coefficients of the
// chunk's atoms for a group's states are staged in shared memory once (16-byte
// copies of the chunk's own atoms) and shared by every point; the table values
// of a point's first entry stay in registers across the groups (NPJ: the
// number of radial channels when it is 5, else 0 and read at run time).  The
// arithmetic of each (state, point) is that of k_proj_scatter, in the same
// order.
template <typename T> struct Row6 {
  static __device__ __forceinline__ void ld(const C<T> *d, C<T> r[6])
  {
#pragma unroll
    for (int i = 0; i < 6; i++) r[i] = d[i];
  }
};
template <> struct Row6<float> {
  static __device__ __forceinline__ void ld(const float2 *d, float2 r[6])
  {
    const float4 *v = reinterpret_cast<const float4 *>(d);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const float4 t = v[i];
      r[2 * i] = make_float2(t.x, t.y);
      r[2 * i + 1] = make_float2(t.z, t.w);
    }
  }
};

template <typename T, bool SO, bool NL, int kG, int NPJ>
__global__ void __launch_bounds__(kScatterChunkPoints) k_proj_scatter_chunk(
    C<T> *__restrict__ out, const C<T> *__restrict__ coef, PtView<T> pv, const int *__restrict__ chunk_beg,
    const int *__restrict__ chunk_atoms, const unsigned char *__restrict__ slot, long nat, long nstates, long ngrid,
    int nspin, T scale)
{
  constexpr int NCH = (SO ? 1 : 0) + (NL ? 1 : 0);
  constexpr int ROW = NCH * kNC;                          // coefficients per (state, atom)
  constexpr int U16 = ROW * (int)sizeof(C<T>) / 16;       // 16-byte units per (state, atom)
  constexpr int kCache = 1;                               // entries whose table values stay in registers
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C<T> *dsm = reinterpret_cast<C<T> *>(smem_raw);  // [kG][kScatterChunkAtoms][ROW]
  const int c = blockIdx.x;
  const int p0 = chunk_beg[c], np = chunk_beg[c + 1] - p0;
  const int t = threadIdx.x;
  const bool live = t < np;
  const long k = p0 + (live ? t : 0);
  const long j = pv.cov_j[k];
  const int e0 = pv.cov_beg[k], e1 = live ? pv.cov_beg[k + 1] : e0;
  const int npj = NPJ ? NPJ : pv.nproj;
  const int ch0 = SO ? 0 : 1;
  int na = 0;  // the chunk's atoms come first, unused slots are -1
  while (na < kScatterChunkAtoms && chunk_atoms[c * kScatterChunkAtoms + na] >= 0) na++;
  auto table = [&](int e, T yr[3], T yi[3], T bs[5], T bn[5]) {
#pragma unroll
    for (int m = 0; m < 3; m++) {
      const C<T> y = pv.y1[m * pv.nent + e];
      yr[m] = y.x;
      yi[m] = y.y;
    }
#pragma unroll
    for (int p = 0; p < 5; p++) {
      bs[p] = (SO && p < npj) ? pv.sop[p * pv.nent + e] : T(0);
      bn[p] = (NL && p < npj) ? pv.nlp[p * pv.nent + e] : T(0);
    }
  };
  T cyr[kCache][3], cyi[kCache][3], cbs[kCache][5], cbn[kCache][5];
  int csl[kCache];
#pragma unroll
  for (int q = 0; q < kCache; q++) {
    if (e0 + q < e1) {
      table(e0 + q, cyr[q], cyi[q], cbs[q], cbn[q]);
      csl[q] = slot[e0 + q];
    }
  }
  for (long s0 = 0; s0 < nstates; s0 += kG) {
    const int ng = (int)(nstates - s0 < kG ? nstates - s0 : kG);
    __syncthreads();
#pragma unroll
    for (int g = 0; g < kG; g++) {
      if (g >= ng) break;
      for (int i = t; i < na * U16; i += blockDim.x) {
        const int sa = i / U16, u = i - sa * U16;
        const int a = chunk_atoms[c * kScatterChunkAtoms + sa];
        reinterpret_cast<float4 *>(dsm + (g * kScatterChunkAtoms + sa) * ROW)[u] =
            reinterpret_cast<const float4 *>(coef + (((s0 + g) * nat + a) * 2 + ch0) * kNC)[u];
      }
    }
    __syncthreads();
    if (!live) continue;
    C<T> o[kG][2];
#pragma unroll
    for (int g = 0; g < kG; g++)
#pragma unroll
      for (int s = 0; s < 2; s++)
        if (g < ng && s < nspin) o[g][s] = out[((s0 + g) * nspin + s) * ngrid + j];
    T ar[kG][2], ai[kG][2];
#pragma unroll
    for (int g = 0; g < kG; g++) {
      ar[g][0] = ar[g][1] = T(0);
      ai[g][0] = ai[g][1] = T(0);
    }
    for (int e = e0; e < e1; e++) {
      int sl;
      T yr[3], yi[3], bs[5], bn[5];
      if (e == e0) {
#pragma unroll
        for (int m = 0; m < 3; m++) {
          yr[m] = cyr[0][m];
          yi[m] = cyi[0][m];
        }
#pragma unroll
        for (int p = 0; p < 5; p++) {
          bs[p] = cbs[0][p];
          bn[p] = cbn[0][p];
        }
        sl = csl[0];
      } else {
        table(e, yr, yi, bs, bn);
        sl = slot[e];
      }
#pragma unroll
      for (int g = 0; g < kG; g++) {
        if (g >= ng) continue;
        const C<T> *d = dsm + (g * kScatterChunkAtoms + sl) * ROW;
        T qr[6], qi[6];
#pragma unroll
        for (int q = 0; q < 6; q++) qr[q] = qi[q] = T(0);
#pragma unroll
        for (int p = 0; p < 5; p++) {
          if (p >= npj) continue;
          C<T> rs[6], rn[6];
          if (SO) Row6<T>::ld(d + p * 6, rs);
          if (NL) Row6<T>::ld(d + (SO ? kNC : 0) + p * 6, rn);
#pragma unroll
          for (int q = 0; q < 6; q++) {
            if (SO) {
              qr[q] += bs[p] * rs[q].x;
              qi[q] += bs[p] * rs[q].y;
            }
            if (NL) {
              qr[q] += bn[p] * rn[q].x;
              qi[q] += bn[p] * rn[q].y;
            }
          }
        }
#pragma unroll
        for (int s = 0; s < 2; s++) {
          if (s >= nspin) continue;
          T vr = 0, vi = 0;
#pragma unroll
          for (int m = 0; m < 3; m++) {
            vr += yr[m] * qr[3 * s + m] - yi[m] * qi[3 * s + m];
            vi += yr[m] * qi[3 * s + m] + yi[m] * qr[3 * s + m];
          }
          ar[g][s] += vr;
          ai[g][s] += vi;
        }
      }
    }
#pragma unroll
    for (int g = 0; g < kG; g++)
#pragma unroll
      for (int s = 0; s < 2; s++) {
        if (g >= ng || s >= nspin) continue;
        C<T> v = o[g][s];
        v.x += scale * ar[g][s];
        v.y += scale * ai[g][s];
        out[((s0 + g) * nspin + s) * ngrid + j] = v;
      }
  }
}

template <typename T, int kGU>
static void launch_gather(fbse_ctx *c, dim3 g, const C<T> *in, C<T> *coef, const ProjView<T> &pv, long nstates, int ch0)
{
  // FP32 (mixed path): a register cap for 8 CTAs per SM (more warps in flight
  // instead of more loads per warp); FP64: no cap (the cap spills there)
  constexpr int kMinB = sizeof(T) == 4 ? 8 : 1;
  k_proj_gather<T, kGU, kMinB, kSW><<<g, kProjThreads, 0, c->stream>>>(in, coef, pv, c->proj.nat, nstates, c->ngrid,
                                                                      c->nspin, ch0, c->dv);
}

template <typename T, bool SO, bool NL, int kG, int NPJ>
static int launch_scatter_chunk2(fbse_ctx *c, C<T> *out, const C<T> *coef, const PtView<T> &pt, long nstates, T sc)
{
  const ProjDev &p = c->proj;
  constexpr int NCH = (SO ? 1 : 0) + (NL ? 1 : 0);
  const size_t smem = (size_t)kG * kScatterChunkAtoms * NCH * kNC * sizeof(C<T>);
  FBSE_CUDA(c, cudaFuncSetAttribute(k_proj_scatter_chunk<T, SO, NL, kG, NPJ>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_proj_scatter_chunk<T, SO, NL, kG, NPJ><<<(unsigned)p.nchunk, kScatterChunkPoints, smem, c->stream>>>(
      out, coef, pt, p.chunk_beg, p.chunk_atoms, p.pe_slot, p.nat, nstates, c->ngrid, c->nspin, sc);
  return FBSE_OK;
}

template <typename T, bool SO, bool NL, int kG>
static int launch_scatter_chunk1(fbse_ctx *c, C<T> *out, const C<T> *coef, const PtView<T> &pt, long nstates, T sc)
{
  if (pt.nproj == 5) return launch_scatter_chunk2<T, SO, NL, kG, 5>(c, out, coef, pt, nstates, sc);
  return launch_scatter_chunk2<T, SO, NL, kG, 0>(c, out, coef, pt, nstates, sc);
}

template <typename T, int kG>
static int launch_scatter_chunk(fbse_ctx *c, C<T> *out, const C<T> *coef, const PtView<T> &pt, long nstates, T sc)
{
  if (c->so && c->nl) return launch_scatter_chunk1<T, true, true, kG>(c, out, coef, pt, nstates, sc);
  if (c->so) return launch_scatter_chunk1<T, true, false, kG>(c, out, coef, pt, nstates, sc);
  return launch_scatter_chunk1<T, false, true, kG>(c, out, coef, pt, nstates, sc);
}

template <typename T, int kG>
static void launch_scatter(fbse_ctx *c, C<T> *out, const C<T> *coef, const PtView<T> &pt, long nstates, T sc)
{
  const ProjDev &p = c->proj;
  dim3 gs((unsigned)((p.ncov + 255) / 256), (unsigned)((nstates + kG - 1) / kG));
  if (c->so && c->nl)
    k_proj_scatter<T, true, true, kG><<<gs, 256, 0, c->stream>>>(out, coef, pt, p.nat, nstates, c->ngrid, c->nspin, sc);
  else if (c->so)
    k_proj_scatter<T, true, false, kG><<<gs, 256, 0, c->stream>>>(out, coef, pt, p.nat, nstates, c->ngrid, c->nspin, sc);
  else
    k_proj_scatter<T, false, true, kG><<<gs, 256, 0, c->stream>>>(out, coef, pt, p.nat, nstates, c->ngrid, c->nspin, sc);
}

// the gather half of proj_apply: the projector coefficients of in into the
// context's coefficient buffer, on the context's stream
template <typename T>
static int proj_gather(fbse_ctx *c, const C<T> *in, long nstates, long st0 = 0)
{
  // st0: the states' offset in the coefficient buffer (sized for st0 + nstates)
  const ProjDev &p = c->proj;
  const size_t need = (size_t)(st0 + nstates) * p.nat * 2 * kNC * sizeof(C<T>);
  int rc = ensure(c, &c->coef, &c->coef_bytes, need);
  if (rc) return rc;
  C<T> *coef = reinterpret_cast<C<T> *>(c->coef) + st0 * p.nat * 2 * kNC;
  const long spc = kSW / c->nspin;
  const long ggroups = (nstates + spc - 1) / spc;
  if (ggroups > 65535 || p.nat > 2147483647L || nstates > 65535)
    return set_err(c, FBSE_ERR_UNSUPPORTED, "projector grid too large");
  const int ch0 = c->so ? 0 : 1;
  const int nch = (c->so ? 1 : 0) + (c->nl ? 1 : 0);
  dim3 gg((unsigned)p.nat, (unsigned)nch, (unsigned)ggroups);
  const ProjView<T> pv = view<T>(c);
  const std::string prob = std::string(sizeof(T) == 4 ? "fp32" : "fp64") + " states=" + std::to_string(nstates) +
                           " atoms=" + std::to_string(p.nat) + " points=" + std::to_string(p.ncov) +
                           (c->so ? " SO" : "") + (c->nl ? " NL" : "");
  // points per lane per iteration (the same sums in the same order for every
  // choice); the gather writes only coef, so candidates run in place
  long gu = c->tune.gather_points;
  auto gather = [&](long v) -> int {
    if (v == 1) launch_gather<T, 1>(c, gg, in, coef, pv, nstates, ch0);
    else if (v == 4) launch_gather<T, 4>(c, gg, in, coef, pv, nstates, ch0);
    else launch_gather<T, 2>(c, gg, in, coef, pv, nstates, ch0);
    return launch_status(c);
  };
  if (gu == 0 && (rc = autotune(c, "projector gather points per lane", prob, {1, 2, 4}, gather, &gu))) return rc;
  if ((rc = gather(gu))) return rc;
  FBSE_COUNT(1);
  return FBSE_OK;
}

// the scatter half: out += scale * (projector terms of the gathered
// coefficients).  scratch (optional, nstates states): where the autotuner may
// time scatter candidates; without it the scatter runs its default shape
// until a call that has scratch.
template <typename T>
static int proj_scatter(fbse_ctx *c, C<T> *out, long nstates, double scale, C<T> *scratch, long st0 = 0)
{
  const ProjDev &p = c->proj;
  if (p.ncov == 0) return FBSE_OK;
  int rc;
  const C<T> *coef = reinterpret_cast<const C<T> *>(c->coef) + st0 * p.nat * 2 * kNC;
  const std::string prob = std::string(sizeof(T) == 4 ? "fp32" : "fp64") + " states=" + std::to_string(nstates) +
                           " atoms=" + std::to_string(p.nat) + " points=" + std::to_string(p.ncov) +
                           (c->so ? " SO" : "") + (c->nl ? " NL" : "");
  const PtView<T> pt = ptview<T>(c);
  const T sc = (T)scale;
  // v = 1, 2, 4, 8: one thread per point and v states; v = 16 + g: one CTA
  // per chunk of points, all states in groups of g with the chunk's
  // coefficients in shared memory.  Each (state, point) is summed in the same
  // order for every choice; candidates are timed on the scratch states
  long kg = c->tune.scatter_states;
  auto scatter = [&](C<T> *dst, long v) -> int {
    int r = FBSE_OK;
    if (v == 1) launch_scatter<T, 1>(c, dst, coef, pt, nstates, sc);
    else if (v == 2) launch_scatter<T, 2>(c, dst, coef, pt, nstates, sc);
    else if (v == 8) launch_scatter<T, 8>(c, dst, coef, pt, nstates, sc);
    else if (v == 18) r = launch_scatter_chunk<T, 2>(c, dst, coef, pt, nstates, sc);
    else if (v == 20) r = launch_scatter_chunk<T, 4>(c, dst, coef, pt, nstates, sc);
    else launch_scatter<T, 4>(c, dst, coef, pt, nstates, sc);
    return r ? r : launch_status(c);
  };
  if (kg == 0) {
    if (scratch) {
      if ((rc = autotune(c, "projector scatter states per thread (16 + g: chunked, g per group)", prob,
                         {1, 2, 4, 8, 18, 20}, [&](long v) { return scatter(scratch, v); }, &kg)))
        return rc;
    } else {
      kg = 4;
    }
  }
  if ((rc = scatter(out, kg))) return rc;
  FBSE_COUNT(1);
  return FBSE_OK;
}

static bool has_proj(fbse_ctx *c) { return (c->so || c->nl) && c->proj.nat > 0; }

// out += scale * (V_SO + V_NL) in for nstates states
template <typename T>
int proj_apply(fbse_ctx *c, const C<T> *in, C<T> *out, long nstates, double scale, C<T> *scratch)
{
  if (!has_proj(c)) return FBSE_OK;
  int rc = proj_gather<T>(c, in, nstates);
  return rc ? rc : proj_scatter<T>(c, out, nstates, scale, scratch);
}

// one part of a split H psi: gather, FFT passes, scatter of nstates states
// whose coefficients sit at state offset st0, on the context's current stream
template <typename T>
static int hpsi_part(fbse_ctx *c, const C<T> *in, C<T> *out, C<T> *wk, long nstates, double a, double b, long st0)
{
  int rc = proj_gather<T>(c, in, nstates, st0);
  if (!rc) rc = kinetic_apply<T>(c, in, out, wk, nstates * c->nspin, a, b, 1);
  // the FFT scratch is free again: the scatter's autotuner may time on it
  return rc ? rc : proj_scatter<T>(c, out, nstates, a, wk, st0);
}

template <typename T>
int hpsi_apply(fbse_ctx *c, const C<T> *in, C<T> *out, long nstates, double a, double b)
{
  if constexpr (sizeof(T) == 4) {
    if (hpsi_fused_ok(c)) return hpsi_fused_apply(c, in, out, nstates, a, b);
  }
  const size_t need = (size_t)nstates * c->nspin * c->ngrid * sizeof(C<T>);
  int rc = ensure(c, &c->wk, &c->wk_bytes, need);
  if (rc) return rc;
  C<T> *wk = reinterpret_cast<C<T> *>(c->wk);
  const long nblk = nstates * c->nspin;
  // with the projectors on and input and output apart, the batch runs as
  // parts (two by default) on the context's streams, each gather -> FFT
  // passes -> scatter, so that one part's projector kernels (latency bound)
  // and tail waves overlap the other parts' kernels; every state sees the
  // same kernels either way
  const char *i0 = reinterpret_cast<const char *>(in), *o0 = reinterpret_cast<const char *>(out);
  const bool apart = i0 + need <= o0 || o0 + need <= i0;
  const long parts = std::min<long>(nstates, c->tune.hpsi_streams == 0 ? 2 : c->tune.hpsi_streams);
  if (has_proj(c) && apart && parts >= 2 && c->side[0]) {
    // buffers sized on the main stream: no part reallocates under another
    if ((rc = ensure(c, &c->coef, &c->coef_bytes, (size_t)nstates * c->proj.nat * 2 * kNC * sizeof(C<T>))))
      return rc;
    FBSE_CUDA(c, cudaEventRecord(c->ev_fork, c->stream));
    cudaStream_t main = c->stream;
    // parts 1.. on the side streams, part 0 on the context's stream
    // (a first call's autotuners time their candidates on the stream of the part they serve)
    for (long k = parts - 1; k >= 0; k--) {
      const long s0 = nstates * k / parts, s1 = nstates * (k + 1) / parts;
      const long off = s0 * c->nspin * c->ngrid;
      if (k > 0) {
        FBSE_CUDA(c, cudaStreamWaitEvent(c->side[k - 1], c->ev_fork, 0));
        c->stream = c->side[k - 1];
      }
      rc = hpsi_part<T>(c, in + off, out + off, wk + off, s1 - s0, a, b, s0);
      c->stream = main;
      if (rc) {
        // parts already enqueued finish before the caller may free or reuse buffers
        for (int q = 0; q < fbse_ctx::kSide; q++) cudaStreamSynchronize(c->side[q]);
        return rc;
      }
      if (k > 0) FBSE_CUDA(c, cudaEventRecord(c->ev_join[k - 1], c->side[k - 1]));
    }
    for (long k = 1; k < parts; k++) FBSE_CUDA(c, cudaStreamWaitEvent(c->stream, c->ev_join[k - 1], 0));
    return FBSE_OK;
  }
  if ((rc = kinetic_apply<T>(c, in, out, wk, nblk, a, b, 1))) return rc;
  return proj_apply<T>(c, in, out, nstates, a, wk);
}

template int proj_apply<float>(fbse_ctx *, const C<float> *, C<float> *, long, double, C<float> *);
template int proj_apply<double>(fbse_ctx *, const C<double> *, C<double> *, long, double, C<double> *);
template int hpsi_apply<float>(fbse_ctx *, const C<float> *, C<float> *, long, double, double);
template int hpsi_apply<double>(fbse_ctx *, const C<double> *, C<double> *, long, double, double);

}  // namespace fbse
