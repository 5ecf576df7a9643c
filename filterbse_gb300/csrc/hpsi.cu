// H psi on the GPU: local potential, spin-orbit and
// nonlocal projectors, and the Newton scale-and-shift of p_hnorm.
//
// Projectors replace p_spin_orbit_proj_pot and p_nonlocal_proj_pot
// (filter_mpi/phamiltonian.c:140-312, 316-444; k = 0).  For one atom a and
// radial channel p the reference forms
//   c[p][j'] = dv sum_pts b_p(r) conj(Y_m'(r)) psi_s'(r),   j' = 3 s' + m'
// and scatters b_p(r) Y_m(r) sum_j' LS[j'][j] c[p][j'] into spin s of the
// output (SO); the NL operator is the same with b^NL_p, a sign per channel and
// no spin mixing.  Here one CTA per (atom, channel, group of 4 states) gathers
// the 30 coefficients of each state in one warp (register accumulation, warp
// reduction) -- the 4 warps share every table entry through L1, so the table
// is read once per 4 states -- and applies L.S (or the NL sign).  The scatter
// kernel has the same shape and adds the contribution with atomics
// (overlapping spheres of neighbouring atoms make it a reduction; the
// reference uses "omp atomic" for the same reason, phamiltonian.c:295-303).
#include "fbse_internal.cuh"

namespace fbse {

template <typename T> struct ProjView {
  const int *cnt, *jxyz, *sgn;
  const T *y1, *sop, *nlp;
  const double2 *LS;
  long npts;
  int nproj;
};

template <typename T> static ProjView<T> view(fbse_ctx *c);
template <> ProjView<double> view<double>(fbse_ctx *c)
{
  const ProjDev &p = c->proj;
  return {p.nl_cnt, p.jxyz, p.sgn, p.y1, p.sop, p.nlp, p.LS, p.npts, p.nproj};
}
template <> ProjView<float> view<float>(fbse_ctx *c)
{
  const ProjDev &p = c->proj;
  return {p.nl_cnt, p.jxyz, p.sgn, p.y1f, p.sopf, p.nlpf, p.LS, p.npts, p.nproj};
}

constexpr int kSW = 4;              // states (warps) per CTA
constexpr int kProjThreads = 32 * kSW;
constexpr int kNC = 30;             // 5 radial channels x (2 spins x 3 m)

// gather: coef[((st*nat + a)*2 + ch)*30 + p*6 + j]
template <typename T>
__global__ void __launch_bounds__(kProjThreads) k_proj_gather(const C<T> *__restrict__ psi, C<T> *__restrict__ coef,
                                                              ProjView<T> pv, long nat, long nstates, long ngrid,
                                                              int nspin, int ch0, double dv)
{
  const long a = blockIdx.x;
  const int ch = ch0 + blockIdx.y;  // 0: SO, 1: NL
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long st = (long)blockIdx.z * kSW + wid;
  const bool live = st < nstates;
  const int np = pv.cnt[a];
  const C<T> *ps = psi + (live ? st : 0) * nspin * ngrid;
  const T *rad = (ch == 0) ? pv.sop : pv.nlp;
  T acc[2 * kNC];
#pragma unroll
  for (int i = 0; i < 2 * kNC; i++) acc[i] = T(0);
  if (live) {
    for (int g = lane; g < np; g += 32) {
      const long e = a * pv.npts + g;
      const int jx = pv.jxyz[e];
      T yr[3], yi[3], b[5];
#pragma unroll
      for (int m = 0; m < 3; m++) { yr[m] = pv.y1[e * 6 + 2 * m]; yi[m] = pv.y1[e * 6 + 2 * m + 1]; }
#pragma unroll
      for (int p = 0; p < 5; p++) b[p] = (p < pv.nproj) ? rad[e * pv.nproj + p] : T(0);
#pragma unroll
      for (int s = 0; s < 2; s++) {
        if (s < nspin) {
          const C<T> v = ps[s * ngrid + jx];
#pragma unroll
          for (int m = 0; m < 3; m++) {
            // psi * conj(Y)
            const T tr = v.x * yr[m] + v.y * yi[m];
            const T ti = v.y * yr[m] - v.x * yi[m];
#pragma unroll
            for (int p = 0; p < 5; p++) {
              acc[2 * (p * 6 + s * 3 + m)] += b[p] * tr;
              acc[2 * (p * 6 + s * 3 + m) + 1] += b[p] * ti;
            }
          }
        }
      }
    }
  }
  __shared__ C<T> cf[kSW][kNC];
#pragma unroll
  for (int i = 0; i < 2 * kNC; i++) {
    T v = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    acc[i] = v;
  }
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < kNC; i++) cf[wid][i] = mk<T>(acc[2 * i] * (T)dv, acc[2 * i + 1] * (T)dv);
  }
  __syncwarp();
  if (live && lane < kNC) {
    const int p = lane / 6, j = lane % 6;
    C<T> d = mk<T>(0, 0);
    if (ch == 0) {
      // d[p][j] = sum_j' LS[j'][j] c[p][j']   (phamiltonian.c:249-290)
      for (int jp = 0; jp < 6; jp++) {
        const double2 l = pv.LS[jp * 6 + j];
        const C<T> cc = cf[wid][p * 6 + jp];
        d.x += (T)l.x * cc.x - (T)l.y * cc.y;
        d.y += (T)l.x * cc.y + (T)l.y * cc.x;
      }
    } else {
      // sign of the channel (phamiltonian.c:399-401), block diagonal in spin
      const T sg = (p < pv.nproj) ? (T)pv.sgn[a * pv.nproj + p] : T(0);
      d = cscale<T>(cf[wid][lane], sg);
    }
    coef[((st * nat + a) * 2 + ch) * kNC + lane] = d;
  }
}

__device__ __forceinline__ void atomic_add_c(float2 *p, float2 v)
{
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}
__device__ __forceinline__ void atomic_add_c(double2 *p, double2 v)
{
  atomicAdd(&p->x, v.x);
  atomicAdd(&p->y, v.y);
}

// scatter: out_s(r) += scale * sum_p b_p(r) sum_m Y_m(r) d[p][3 s + m] over the active channels
template <typename T>
__global__ void __launch_bounds__(kProjThreads) k_proj_scatter(C<T> *__restrict__ out, const C<T> *__restrict__ coef,
                                                               ProjView<T> pv, long nat, long nstates, long ngrid,
                                                               int nspin, int use_so, int use_nl, T scale)
{
  const long a = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long st = (long)blockIdx.y * kSW + wid;
  __shared__ C<T> d[kSW][2][kNC];
  if (st < nstates) {
    for (int i = lane; i < 2 * kNC; i += 32) d[wid][i / kNC][i % kNC] = coef[((st * nat + a) * 2) * kNC + i];
  }
  __syncwarp();
  if (st >= nstates) return;
  const int np = pv.cnt[a];
  C<T> *po = out + st * nspin * ngrid;
  for (int g = lane; g < np; g += 32) {
    const long e = a * pv.npts + g;
    const int jx = pv.jxyz[e];
    T yr[3], yi[3];
#pragma unroll
    for (int m = 0; m < 3; m++) { yr[m] = pv.y1[e * 6 + 2 * m]; yi[m] = pv.y1[e * 6 + 2 * m + 1]; }
    for (int s = 0; s < nspin; s++) {
      T vr = 0, vi = 0;
      for (int ch = 0; ch < 2; ch++) {
        if ((ch == 0 && !use_so) || (ch == 1 && !use_nl)) continue;
        const T *rad = (ch == 0) ? pv.sop : pv.nlp;
        for (int p = 0; p < pv.nproj; p++) {
          const T b = rad[e * pv.nproj + p];
          T sr = 0, si = 0;
#pragma unroll
          for (int m = 0; m < 3; m++) {
            const C<T> q = d[wid][ch][p * 6 + s * 3 + m];
            sr += yr[m] * q.x - yi[m] * q.y;
            si += yr[m] * q.y + yi[m] * q.x;
          }
          vr += b * sr;
          vi += b * si;
        }
      }
      atomic_add_c(&po[s * ngrid + jx], mk<T>(scale * vr, scale * vi));
    }
  }
}

template <typename T>
int proj_apply(fbse_ctx *c, const C<T> *in, C<T> *out, long nstates, double scale)
{
  const ProjDev &p = c->proj;
  if (!(c->so || c->nl) || p.nat == 0) return FBSE_OK;
  const size_t need = (size_t)nstates * p.nat * 2 * kNC * sizeof(C<T>);
  int rc = ensure(c, &c->coef, &c->coef_bytes, need);
  if (rc) return rc;
  C<T> *coef = reinterpret_cast<C<T> *>(c->coef);
  const long ngroups = (nstates + kSW - 1) / kSW;
  if (ngroups > 65535 || p.nat > 2147483647L) return set_err(c, FBSE_ERR_UNSUPPORTED, "projector grid too large");
  const int ch0 = c->so ? 0 : 1;
  const int nch = (c->so ? 1 : 0) + (c->nl ? 1 : 0);
  if (!c->so || !c->nl) {
    // zero the inactive channel so the scatter can skip it cheaply
    FBSE_CUDA(c, cudaMemsetAsync(coef, 0, need, c->stream));
  }
  dim3 gg((unsigned)p.nat, (unsigned)nch, (unsigned)ngroups);
  k_proj_gather<T><<<gg, kProjThreads, 0, c->stream>>>(in, coef, view<T>(c), p.nat, nstates, c->ngrid, c->nspin, ch0,
                                                       c->dv);
  FBSE_CHECK_LAUNCH(c);
  dim3 gs((unsigned)p.nat, (unsigned)ngroups);
  k_proj_scatter<T><<<gs, kProjThreads, 0, c->stream>>>(out, coef, view<T>(c), p.nat, nstates, c->ngrid, c->nspin,
                                                        c->so, c->nl, (T)scale);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

template <typename T>
int hpsi_apply(fbse_ctx *c, const C<T> *in, C<T> *out, long nstates, double a, double b)
{
  const size_t need = (size_t)nstates * c->nspin * c->ngrid * sizeof(C<T>);
  int rc = ensure(c, &c->wk, &c->wk_bytes, need);
  if (rc) return rc;
  if ((rc = kinetic_apply<T>(c, in, out, reinterpret_cast<C<T> *>(c->wk), nstates * c->nspin, a, b, 1))) return rc;
  return proj_apply<T>(c, in, out, nstates, a);
}

template int proj_apply<float>(fbse_ctx *, const C<float> *, C<float> *, long, double);
template int proj_apply<double>(fbse_ctx *, const C<double> *, C<double> *, long, double);
template int hpsi_apply<float>(fbse_ctx *, const C<float> *, C<float> *, long, double, double);
template int hpsi_apply<double>(fbse_ctx *, const C<double> *, C<double> *, long, double, double);

}  // namespace fbse
