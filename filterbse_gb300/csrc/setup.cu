// Local pseudopotential on the grid (build_local_pot, filter_mpi/init.c:481-703,
// short-ranged tables, no strain / interpolation / LSD / long range):
//   V(r) = sum_atoms v_type(|r - R_atom|),
// v linear-interpolated in the atom type's radial table exactly as
// interpolate() does (filter_mpi/interpolate.c:5-49): row i = (long)(r/dr),
// 0 beyond the table.  One thread per grid point, FP64; the O(N natoms)
// host loop of the reference becomes one short kernel.
#include <cmath>

#include "fbse_internal.cuh"

namespace fbse {

__global__ void k_local_pot(int nx, int ny, int nz, const double *__restrict__ gx, const double *__restrict__ gy,
                            const double *__restrict__ gz, int nat, const double *__restrict__ R,
                            const int *__restrict__ atype, const double *__restrict__ tr,
                            const double *__restrict__ tv, const long *__restrict__ toff,
                            const long *__restrict__ tlen, const double *__restrict__ tdr, double *__restrict__ pot)
{
  const long N = (long)nx * ny * nz;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int jx = (int)(g % nx), jy = (int)((g / nx) % ny), jz = (int)(g / ((long)nx * ny));
    const double x = gx[jx], y = gy[jy], z = gz[jz];
    double sum = 0.0;
    for (int a = 0; a < nat; a++) {
      const double dx = x - R[3 * a], dy = y - R[3 * a + 1], dz = z - R[3 * a + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      const int t = atype[a];
      const long i = (long)(r / tdr[t]);
      if (i > tlen[t] - 2) continue;
      const double *vr = tr + toff[t], *v = tv + toff[t];
      const double sl = 1.0 * (v[i + 1] - v[i]) / (vr[i + 1] - vr[i]);
      const double b = 1.0 * v[i] - vr[i] * sl;
      sum += sl * r + b;
    }
    pot[g] = sum;
  }
}

}  // namespace fbse

using namespace fbse;

extern "C" int fbse_build_local_pot(long nx, long ny, long nz, const double *gx, const double *gy, const double *gz,
                                    long natoms, const double *coords, const int *atype, int ntypes,
                                    const double *tab_r, const double *tab_v, const long *tab_off,
                                    const long *tab_len, double *pot)
{
  if (nx < 1 || ny < 1 || nz < 1 || natoms < 0 || ntypes < 1 || !gx || !gy || !gz || !pot || !tab_r || !tab_v ||
      !tab_off || !tab_len || (natoms > 0 && (!coords || !atype)))
    return FBSE_ERR_ARG;
  long ntab = 0;
  std::vector<double> dr(ntypes);
  for (int t = 0; t < ntypes; t++) {
    if (tab_len[t] < 2) return FBSE_ERR_ARG;
    ntab = std::max(ntab, tab_off[t] + tab_len[t]);
    dr[t] = tab_r[tab_off[t] + 1] - tab_r[tab_off[t]];
    if (!(dr[t] > 0)) return FBSE_ERR_ARG;
  }
  for (long a = 0; a < natoms; a++)
    if (atype[a] < 0 || atype[a] >= ntypes) return FBSE_ERR_ARG;
  const long N = nx * ny * nz;
  double *d_g = nullptr, *d_R = nullptr, *d_tr = nullptr, *d_tv = nullptr, *d_dr = nullptr, *d_pot = nullptr;
  long *d_off = nullptr, *d_len = nullptr;
  int *d_at = nullptr;
  int rc = FBSE_OK;
  auto A = [&](void **p, size_t b) { return cudaMalloc(p, b ? b : 8) == cudaSuccess; };
  if (!A((void **)&d_g, (nx + ny + nz) * sizeof(double)) || !A((void **)&d_R, 3 * natoms * sizeof(double)) ||
      !A((void **)&d_tr, ntab * sizeof(double)) || !A((void **)&d_tv, ntab * sizeof(double)) ||
      !A((void **)&d_dr, ntypes * sizeof(double)) || !A((void **)&d_pot, N * sizeof(double)) ||
      !A((void **)&d_off, ntypes * sizeof(long)) || !A((void **)&d_len, ntypes * sizeof(long)) ||
      !A((void **)&d_at, natoms * sizeof(int))) {
    rc = FBSE_ERR_OOM;
  } else {
    cudaMemcpy(d_g, gx, nx * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_g + nx, gy, ny * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_g + nx + ny, gz, nz * sizeof(double), cudaMemcpyHostToDevice);
    if (natoms) {
      cudaMemcpy(d_R, coords, 3 * natoms * sizeof(double), cudaMemcpyHostToDevice);
      cudaMemcpy(d_at, atype, natoms * sizeof(int), cudaMemcpyHostToDevice);
    }
    cudaMemcpy(d_tr, tab_r, ntab * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_tv, tab_v, ntab * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_dr, dr.data(), ntypes * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(d_off, tab_off, ntypes * sizeof(long), cudaMemcpyHostToDevice);
    cudaMemcpy(d_len, tab_len, ntypes * sizeof(long), cudaMemcpyHostToDevice);
    FBSE_COUNT(1); k_local_pot<<<152 * 16, 256>>>((int)nx, (int)ny, (int)nz, d_g, d_g + nx, d_g + nx + ny, (int)natoms, d_R, d_at,
                                   d_tr, d_tv, d_off, d_len, d_dr, d_pot);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(pot, d_pot, N * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = FBSE_ERR_CUDA;
  }
  void *bufs[] = {d_g, d_R, d_tr, d_tv, d_dr, d_pot, d_off, d_len, d_at};
  for (void *b : bufs)
    if (b) cudaFree(b);
  return rc;
}

// ---------------------------------------------------------------------------
// Projector table (init_NL_projectors, filter_mpi/init.c:848-1135, body
// 508-589): for every projector atom the grid points with r^2 < R_NLcut2 in
// jz, jy, jx order, Y_1m with the reference's EPSDX shifts (init.c:1002-1040)
// and the radial projectors interpolated at r (interpolate(), linear).  One
// CTA per atom: the sphere's bounding box comes from three axis scans (each
// axis' set of in-range points is an interval), a first kernel counts the
// points, a second writes them in order with a block-wide scan.  Every
// product, sum, quotient and root is rounded on its own (no fused
// multiply-add), so the table is bit-identical to a plain IEEE evaluation of
// the same expressions on the host.
// ---------------------------------------------------------------------------
namespace fbse {
namespace {

struct NlcArgs {
  int nx, ny, nz;
  const double *gx, *gy, *gz;  // grid coordinates
  const double *xyz;           // [nat][3]
  const double *sq;            // [nat] sqrt(SO_par), or null
  const double *so_tab;        // [nproj][PROJ_LEN], or null
  const double *nl_tab;        // [nat][nproj][PROJ_LEN], or null
  int nproj;
  long ntab;
  double rcut2, drp, tmp1, tmp2, eps;
  int *box;                    // [nat][6] lo/hi per axis (x, y, z)
  long *cnt;                   // [nat]
};

__device__ __forceinline__ double sq3(double a, double b, double c)
{
  return __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
}

// interpolate()'s linear rule on a radial table with spacing dr, 0 beyond it
__device__ __forceinline__ double interp_rn(double r, double dr, const double *__restrict__ tab, long n)
{
  const long i = (long)__ddiv_rn(r, dr);
  if (i > n - 2) return 0.0;
  const double x0 = __dmul_rn((double)i, dr), x1 = __dmul_rn((double)(i + 1), dr);
  const double a = __ddiv_rn(__dsub_rn(tab[i + 1], tab[i]), __dsub_rn(x1, x0));
  return __dadd_rn(__dmul_rn(a, r), __dsub_rn(tab[i], __dmul_rn(x0, a)));
}

// box and point count of atom blockIdx.x
__global__ void k_nlc_count(NlcArgs g)
{
  const int a = blockIdx.x;
  const double cx = g.xyz[3 * a], cy = g.xyz[3 * a + 1], cz = g.xyz[3 * a + 2];
  __shared__ int lo[3], hi[3];
  __shared__ unsigned long long tot;
  if (threadIdx.x < 3) {
    lo[threadIdx.x] = 0x7fffffff;
    hi[threadIdx.x] = -1;
  }
  if (threadIdx.x == 0) tot = 0;
  __syncthreads();
  const int n[3] = {g.nx, g.ny, g.nz};
  const double *ax[3] = {g.gx, g.gy, g.gz};
  const double c[3] = {cx, cy, cz};
  for (int d = 0; d < 3; d++)
    for (int j = threadIdx.x; j < n[d]; j += blockDim.x) {
      const double t = __dsub_rn(ax[d][j], c[d]);
      if (__dmul_rn(t, t) < g.rcut2) {
        atomicMin(&lo[d], j);
        atomicMax(&hi[d], j);
      }
    }
  __syncthreads();
  const long bx = hi[0] - lo[0] + 1, by = hi[1] - lo[1] + 1, bz = hi[2] - lo[2] + 1;
  const long nb = (bx > 0 && by > 0 && bz > 0) ? bx * by * bz : 0;
  unsigned long long my = 0;
  for (long q = threadIdx.x; q < nb; q += blockDim.x) {
    const int jx = lo[0] + (int)(q % bx), jy = lo[1] + (int)((q / bx) % by), jz = lo[2] + (int)(q / (bx * by));
    const double d2 = sq3(__dsub_rn(g.gx[jx], cx), __dsub_rn(g.gy[jy], cy), __dsub_rn(g.gz[jz], cz));
    my += d2 < g.rcut2;
  }
  atomicAdd(&tot, my);
  __syncthreads();
  if (threadIdx.x < 3) {
    g.box[6 * a + 2 * threadIdx.x] = lo[threadIdx.x];
    g.box[6 * a + 2 * threadIdx.x + 1] = hi[threadIdx.x];
  }
  if (threadIdx.x == 0) g.cnt[a] = (long)tot;
}

// the entries of atom blockIdx.x in jz, jy, jx order at rows a * npts + k
__global__ void __launch_bounds__(256) k_nlc_fill(NlcArgs g, long npts, int *__restrict__ jxyz,
                                                  double *__restrict__ y1, double *__restrict__ sop,
                                                  double *__restrict__ nlp)
{
  const int a = blockIdx.x;
  const double cx = g.xyz[3 * a], cy = g.xyz[3 * a + 1], cz = g.xyz[3 * a + 2];
  const int *b = g.box + 6 * a;
  const long bx = b[1] - b[0] + 1, by = b[3] - b[2] + 1, bz = b[5] - b[4] + 1;
  const long nb = (bx > 0 && by > 0 && bz > 0) ? bx * by * bz : 0;
  __shared__ int wsum[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  long base = (long)a * npts;
  for (long q0 = 0; q0 < nb; q0 += blockDim.x) {
    const long q = q0 + threadIdx.x;
    int jx = 0, jy = 0, jz = 0;
    double ddx = 0, dy = 0, dz = 0, d2 = 0;
    bool in = false;
    if (q < nb) {
      jx = b[0] + (int)(q % bx);
      jy = b[2] + (int)((q / bx) % by);
      jz = b[4] + (int)(q / (bx * by));
      ddx = __dsub_rn(g.gx[jx], cx);
      dy = __dsub_rn(g.gy[jy], cy);
      dz = __dsub_rn(g.gz[jz], cz);
      d2 = sq3(ddx, dy, dz);
      in = d2 < g.rcut2;
    }
    const unsigned bal = __ballot_sync(0xffffffffu, in);
    if (lane == 0) wsum[w] = __popc(bal);
    __syncthreads();
    int off = 0, tot = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
      off += i < w ? wsum[i] : 0;
      tot += wsum[i];
    }
    off += __popc(bal & ((1u << lane) - 1u));
    if (in && base + off < (long)(a + 1) * npts) {  // the count kernel sized the row with the same test
      const long e = base + off;
      jxyz[e] = g.nx * (g.ny * jz + jy) + jx;
      const double dzeps = __dadd_rn(dz, g.eps), dxeps = __dadd_rn(ddx, g.eps), dyeps = __dadd_rn(dy, g.eps);
      double r_1 = __ddiv_rn(1.0, __dsqrt_rn(sq3(ddx, dy, dzeps)));
      y1[e * 6 + 2] = __dmul_rn(__dmul_rn(g.tmp1, dzeps), r_1);
      y1[e * 6 + 3] = 0.0;
      r_1 = __ddiv_rn(1.0, __dsqrt_rn(sq3(dxeps, dy, dz)));
      y1[e * 6 + 4] = __dmul_rn(__dmul_rn(-g.tmp2, dxeps), r_1);
      y1[e * 6 + 0] = __dmul_rn(__dmul_rn(g.tmp2, dxeps), r_1);
      r_1 = __ddiv_rn(1.0, __dsqrt_rn(sq3(ddx, dyeps, dz)));
      y1[e * 6 + 5] = __dmul_rn(__dmul_rn(-g.tmp2, dyeps), r_1);
      y1[e * 6 + 1] = __dmul_rn(__dmul_rn(-g.tmp2, dyeps), r_1);
      const double r = __dsqrt_rn(d2);
      for (int p = 0; p < g.nproj; p++) {
        sop[e * g.nproj + p] =
            g.so_tab ? __dmul_rn(interp_rn(r, g.drp, g.so_tab + (long)p * g.ntab, g.ntab), g.sq[a]) : 0.0;
        nlp[e * g.nproj + p] =
            g.nl_tab ? interp_rn(r, g.drp, g.nl_tab + ((long)a * g.nproj + p) * g.ntab, g.ntab) : 0.0;
      }
    }
    base += tot;
    __syncthreads();  // wsum is rewritten by the next chunk
  }
}

}  // namespace
}  // namespace fbse

extern "C" int fbse_build_nlc(long nx, long ny, long nz, const double *gx, const double *gy, const double *gz, long nat,
                              const double *xyz, const double *so_par, const double *so_tab, const double *nl_tab,
                              int nproj, double rcut2, long *npts_out, long **nl_out, int **jxyz_out,
                              double **y1_out, double **so_out, double **nl_p_out)
{
  if (nx < 1 || ny < 1 || nz < 1 || nat < 0 || nproj < 1 || nproj > 5 || !(rcut2 > 0) || !gx || !gy || !gz ||
      !npts_out || !nl_out || !jxyz_out || !y1_out || !so_out || !nl_p_out || (nat > 0 && !xyz) ||
      (so_tab && nat > 0 && !so_par) || nx * ny * nz > 2147483647L)
    return FBSE_ERR_ARG;
  constexpr long kTab = 1024;  // PROJ_LEN, filter_mpi/fd.h
  const long na1 = nat > 0 ? nat : 1;
  long *nl = (long *)calloc(na1, sizeof(long));
  if (!nl) return FBSE_ERR_OOM;
  std::vector<double> sq(na1, 0.0);
  if (so_tab)
    for (long a = 0; a < nat; a++) sq[a] = sqrt(so_par[a]);
  NlcArgs g{};
  g.nx = (int)nx; g.ny = (int)ny; g.nz = (int)nz;
  g.nproj = nproj;
  g.ntab = kTab;
  g.rcut2 = rcut2;
  g.drp = sqrt(rcut2) / (double)kTab;
  g.tmp1 = 0.5 * sqrt(3.0 / 3.14159265358979323846);
  g.tmp2 = 0.5 * sqrt(3.0 / (2.0 * 3.14159265358979323846));
  g.eps = 1.0e-20;  // EPSDX, filter_mpi/fd.h
  double *d_g = nullptr, *d_xyz = nullptr, *d_sq = nullptr, *d_so = nullptr, *d_nlt = nullptr;
  double *d_y1 = nullptr, *d_sop = nullptr, *d_nlp = nullptr;
  int *d_box = nullptr, *d_jx = nullptr;
  long *d_cnt = nullptr;
  int *jx = nullptr;
  double *y1 = nullptr, *sop = nullptr, *nlp = nullptr;
  long npts = 1;
  int rc = FBSE_OK;
  auto A = [&](void **p, size_t b) { return cudaMalloc(p, b ? b : 8) == cudaSuccess; };
  do {
    if (!A((void **)&d_g, (nx + ny + nz) * sizeof(double)) || !A((void **)&d_xyz, 3 * na1 * sizeof(double)) ||
        !A((void **)&d_sq, na1 * sizeof(double)) || !A((void **)&d_box, 6 * na1 * sizeof(int)) ||
        !A((void **)&d_cnt, na1 * sizeof(long)) ||
        (so_tab && !A((void **)&d_so, (size_t)nproj * kTab * sizeof(double))) ||
        (nl_tab && !A((void **)&d_nlt, (size_t)na1 * nproj * kTab * sizeof(double)))) {
      rc = FBSE_ERR_OOM;
      break;
    }
    bool ok = cudaMemcpy(d_g, gx, nx * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(d_g + nx, gy, ny * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(d_g + nx + ny, gz, nz * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(d_sq, sq.data(), na1 * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok && nat > 0) ok = cudaMemcpy(d_xyz, xyz, 3 * nat * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok && so_tab)
      ok = cudaMemcpy(d_so, so_tab, (size_t)nproj * kTab * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok && nl_tab)
      ok = cudaMemcpy(d_nlt, nl_tab, (size_t)nat * nproj * kTab * sizeof(double), cudaMemcpyHostToDevice) ==
           cudaSuccess;
    if (!ok) {
      rc = FBSE_ERR_CUDA;
      break;
    }
    g.gx = d_g; g.gy = d_g + nx; g.gz = d_g + nx + ny;
    g.xyz = d_xyz; g.sq = d_sq; g.so_tab = so_tab ? d_so : nullptr; g.nl_tab = nl_tab ? d_nlt : nullptr;
    g.box = d_box; g.cnt = d_cnt;
    if (nat > 0) {
      FBSE_COUNT(1);
      k_nlc_count<<<(unsigned)nat, 256>>>(g);
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpy(nl, d_cnt, nat * sizeof(long), cudaMemcpyDeviceToHost) != cudaSuccess) {
        rc = FBSE_ERR_CUDA;
        break;
      }
      for (long a = 0; a < nat; a++) npts = std::max(npts, nl[a]);
    }
    const size_t ne = (size_t)na1 * npts;
    jx = (int *)calloc(ne, sizeof(int));
    y1 = (double *)calloc(ne * 6, sizeof(double));
    sop = (double *)calloc(ne * nproj, sizeof(double));
    nlp = (double *)calloc(ne * nproj, sizeof(double));
    if (!jx || !y1 || !sop || !nlp || !A((void **)&d_jx, ne * sizeof(int)) ||
        !A((void **)&d_y1, ne * 6 * sizeof(double)) || !A((void **)&d_sop, ne * nproj * sizeof(double)) ||
        !A((void **)&d_nlp, ne * nproj * sizeof(double))) {
      rc = FBSE_ERR_OOM;
      break;
    }
    // rows past an atom's count stay zero, as the host arrays are
    if (cudaMemset(d_jx, 0, ne * sizeof(int)) != cudaSuccess ||
        cudaMemset(d_y1, 0, ne * 6 * sizeof(double)) != cudaSuccess ||
        cudaMemset(d_sop, 0, ne * nproj * sizeof(double)) != cudaSuccess ||
        cudaMemset(d_nlp, 0, ne * nproj * sizeof(double)) != cudaSuccess) {
      rc = FBSE_ERR_CUDA;
      break;
    }
    if (nat > 0) {
      FBSE_COUNT(1);
      k_nlc_fill<<<(unsigned)nat, 256>>>(g, npts, d_jx, d_y1, d_sop, d_nlp);
      if (cudaGetLastError() != cudaSuccess) {
        rc = FBSE_ERR_CUDA;
        break;
      }
    }
    if (cudaMemcpy(jx, d_jx, ne * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(y1, d_y1, ne * 6 * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(sop, d_sop, ne * nproj * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(nlp, d_nlp, ne * nproj * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = FBSE_ERR_CUDA;
  } while (0);
  void *bufs[] = {d_g, d_xyz, d_sq, d_so, d_nlt, d_y1, d_sop, d_nlp, d_box, d_jx, d_cnt};
  for (void *p : bufs)
    if (p) cudaFree(p);
  if (rc) {
    free(nl);
    free(jx);
    free(y1);
    free(sop);
    free(nlp);
    return rc;
  }
  *npts_out = npts;
  *nl_out = nl;
  *jxyz_out = jx;
  *y1_out = y1;
  *so_out = sop;
  *nl_p_out = nlp;
  return FBSE_OK;
}
