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
