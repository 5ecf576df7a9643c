// Spin and angular-momentum statistics of the filter's eigenstates
// (calcSpinAngStat, filter_mpi/angular.c:4-165 via mod_optional_output.c:51-62).
//
// Per state: the reference's k-space low-pass, normalisation, p = -i grad by
// FFT for both spin blocks, J = r x p + sigma/2 and the eight sums of
// angular.dat.  The FFTs are the library's FP64 convolution passes
// (conv_apply: forward transform, k-space multiplier, inverse transform); the
// cross product, the spin part and the sums are one fused pass over the grid
// with per-block partials summed in a fixed order on the host, so the result
// does not depend on the launch or the device.
#include "fbse_internal.cuh"

#include <cmath>
#include <vector>

namespace fbse {
namespace {

constexpr int kAngBlocks = 456;  // 3 x 152 SMs; fixed so the partial sums have a fixed order
constexpr int kAngThreads = 256;

// the four k-space multipliers of one grid in the transform's (z, y, x) index
// order: [0] the low-pass mask (angular.c:419-453: kept where kx^2 + ky^2 +
// kz^2 < (3 dkz)^2 on the wave vectors that carry the transform's 1/N, so the
// cut keeps every wave vector of an ordinary grid; 1 where kept, leaving the
// round trip's factor N as FFTW does), [1..3] kx/N, ky/N, kz/N (apply_L_op,
// angular.c:256-262)
__global__ void k_ang_multipliers(long ngrid, int nx, int ny, const double *__restrict__ kx,
                                  const double *__restrict__ ky, const double *__restrict__ kz, double cut2,
                                  double2 *__restrict__ out)
{
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < ngrid; g += (long)gridDim.x * blockDim.x) {
    const double a = kx[g % nx], b = ky[(g / nx) % ny], c = kz[g / ((long)nx * ny)];
    out[g] = make_double2((a * a + b * b + c * c < cut2) ? 1.0 : 0.0, 0.0);
    out[ngrid + g] = make_double2(a, 0.0);
    out[2 * ngrid + g] = make_double2(b, 0.0);
    out[3 * ngrid + g] = make_double2(c, 0.0);
  }
}

// psi: the low-passed spinor (up block, down block); P: p_x psi, p_y psi,
// p_z psi (each two blocks).  Per grid point: L = r x p per spin block
// (angular.c:377-398, distribution centre at the origin), the spin part
// (apply_J_op, angular.c:189-212), and the sums of calc_angular_exp
// (angular.c:127-146): Re<psi|J_d psi>, |J_d psi|^2 (d = x, y, z), the sum
// of the three squares, |psi|^2.  part[block][8]
__global__ void __launch_bounds__(kAngThreads) k_ang_sums(const double2 *__restrict__ psi, const double2 *__restrict__ P,
                                                          long ngrid, int nx, int ny, const double *__restrict__ gx,
                                                          const double *__restrict__ gy, const double *__restrict__ gz,
                                                          double *__restrict__ part)
{
  double s[8];
#pragma unroll
  for (int k = 0; k < 8; k++) s[k] = 0.0;
  const long nsg = 2 * ngrid;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < ngrid; g += (long)gridDim.x * blockDim.x) {
    const double x = gx[g % nx], y = gy[(g / nx) % ny], z = gz[g / ((long)nx * ny)];
    double2 J[2][3], ps[2];
#pragma unroll
    for (int sp = 0; sp < 2; sp++) {
      const long q = sp * ngrid + g;
      const double2 px = P[q], py = P[nsg + q], pz = P[2 * nsg + q];
      J[sp][0] = make_double2(y * pz.x - z * py.x, y * pz.y - z * py.y);
      J[sp][1] = make_double2(z * px.x - x * pz.x, z * px.y - x * pz.y);
      J[sp][2] = make_double2(x * py.x - y * px.x, x * py.y - y * px.y);
      ps[sp] = psi[q];
    }
    const double2 u = ps[0], d = ps[1];
    // Jx: + 1/2 of the other block; Jy: -i/2 down into up, +i/2 up into down;
    // Jz: +1/2 up, -1/2 down
    J[0][0].x += 0.5 * d.x;
    J[0][0].y += 0.5 * d.y;
    J[1][0].x += 0.5 * u.x;
    J[1][0].y += 0.5 * u.y;
    J[0][1].x += 0.5 * d.y;
    J[0][1].y -= 0.5 * d.x;
    J[1][1].x -= 0.5 * u.y;
    J[1][1].y += 0.5 * u.x;
    J[0][2].x += 0.5 * u.x;
    J[0][2].y += 0.5 * u.y;
    J[1][2].x -= 0.5 * d.x;
    J[1][2].y -= 0.5 * d.y;
#pragma unroll
    for (int sp = 0; sp < 2; sp++) {
      const double2 p = ps[sp];
      double sq = 0.0;
#pragma unroll
      for (int a = 0; a < 3; a++) {
        const double2 j = J[sp][a];
        const double j2 = j.x * j.x + j.y * j.y;
        s[2 * a] += p.x * j.x + p.y * j.y;
        s[2 * a + 1] += j2;
        sq += j2;
      }
      s[6] += sq;
      s[7] += p.x * p.x + p.y * p.y;
    }
  }
  // fixed-order block reduction: warp shuffles, then the warps in order
  __shared__ double red[kAngThreads / 32][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    double v = 0.0;
    for (int i = 0; i < kAngThreads / 32; i++) v += red[i][threadIdx.x];
    part[(long)blockIdx.x * 8 + threadIdx.x] = v;
  }
}

// init_kvec (filter_mpi/init.c:1383-1394): k[j] = j dk norm, k[n - j] = -j dk
// norm for j = 1..n/2 (for even n the second write leaves k[n/2] negative)
void kvec(std::vector<double> &k, long n, double dk, double norm)
{
  k.assign(n, 0.0);
  const long npos = (n % 2 == 0) ? n / 2 : (n - 1) / 2;
  for (long j = 1; j <= npos; j++) {
    k[j] = j * dk * norm;
    k[n - j] = -(j * dk * norm);
  }
}

}  // namespace
}  // namespace fbse

using namespace fbse;

extern "C" int fbse_angular_stats(fbse_ctx *c, const double *psitot, long n, const double *gx, const double *gy,
                                  const double *gz, double *stats)
{
  if (!c || !psitot || !gx || !gy || !gz || !stats || n < 0)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_angular_stats: bad arguments") : FBSE_ERR_ARG;
  if (!c->is_complex || c->nspin != 2)
    return set_err(c, FBSE_ERR_UNSUPPORTED, "fbse_angular_stats: complex spinor states required "
                                            "(calcSpinAngStat is only available with spin-orbit coupling)");
  if (n == 0) return FBSE_OK;
  const long N = c->ngrid, nsg = 2 * N;
  const double norm = 1.0 / (double)N;
  std::vector<double> kx, ky, kz;
  kvec(kx, c->nx, c->dk[0], norm);
  kvec(ky, c->ny, c->dk[1], norm);
  kvec(kz, c->nz, c->dk[2], norm);
  const double cut = 3.0 * c->dk[2];
  double2 *kq = nullptr, *lp = nullptr, *P = nullptr, *work = nullptr;
  double *dk = nullptr, *dg = nullptr, *part = nullptr;
  const long naxes = c->nx + c->ny + c->nz;
  int rc = FBSE_OK;
  if (cudaMalloc(&kq, 4 * N * sizeof(double2)) != cudaSuccess || cudaMalloc(&lp, nsg * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&P, 3 * nsg * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&work, nsg * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&dk, naxes * sizeof(double)) != cudaSuccess || cudaMalloc(&dg, naxes * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&part, (size_t)kAngBlocks * 8 * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    rc = set_err(c, FBSE_ERR_OOM, "fbse_angular_stats");
  }
  std::vector<double> hp((size_t)kAngBlocks * 8);
  do {
    if (rc) break;
    if (h2d(c->stream, dk, kx.data(), c->nx * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dk + c->nx, ky.data(), c->ny * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dk + c->nx + c->ny, kz.data(), c->nz * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dg, gx, c->nx * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dg + c->nx, gy, c->ny * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dg + c->nx + c->ny, gz, c->nz * sizeof(double)) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_angular_stats upload");
      break;
    }
    k_ang_multipliers<<<(unsigned)std::min<long>((N + 255) / 256, 4096), 256, 0, c->stream>>>(
        N, (int)c->nx, (int)c->ny, dk, dk + c->nx, dk + c->nx + c->ny, cut * cut, kq);
    FBSE_LAUNCH_OR_BREAK(c, rc);
    for (long i = 0; i < n && !rc; i++) {
      const double2 *st = reinterpret_cast<const double2 *>(psitot) + i * nsg;
      // low_pass_filter on each spin block (angular.c:75-79)
      if ((rc = conv_apply<double>(c, st, lp, work, 2, kq))) break;
      // apply_L_op: p_d psi for both blocks (angular.c:264-363)
      for (int d = 0; d < 3 && !rc; d++) rc = conv_apply<double>(c, lp, P + d * nsg, work, 2, kq + (1 + d) * N);
      if (rc) break;
      k_ang_sums<<<kAngBlocks, kAngThreads, 0, c->stream>>>(lp, P, N, (int)c->nx, (int)c->ny, dg, dg + c->nx,
                                                           dg + c->nx + c->ny, part);
      FBSE_LAUNCH_OR_BREAK(c, rc);
      if (d2h(c->stream, hp.data(), part, hp.size() * sizeof(double)) != cudaSuccess) {
        rc = set_err(c, FBSE_ERR_CUDA, "fbse_angular_stats download");
        break;
      }
      double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int b = 0; b < kAngBlocks; b++)
        for (int k = 0; k < 8; k++) s[k] += hp[(size_t)b * 8 + k];
      // normalize (angular.c:81) folded into the sums: every sum is quadratic
      // in the state, so dividing by |psi|^2 equals summing the normalised state
      if (!(s[7] > 0.0)) {
        rc = set_err(c, FBSE_ERR_NAN, std::isnan(s[7]) ? "Norm is NAN! exiting!" : "Norm is 0! exiting!");
        break;
      }
      for (int k = 0; k < 7; k++) stats[i * 8 + k] = s[k] / s[7];
      stats[i * 8 + 7] = 1.0;
    }
  } while (0);
  cudaStreamSynchronize(c->stream);
  void *bufs[] = {kq, lp, P, work, dk, dg, part};
  for (void *b : bufs)
    if (b) cudaFree(b);
  return rc;
}
