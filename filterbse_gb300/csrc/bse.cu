// Bethe-Salpeter exciton stage on the GPU (bse_cplx/).
//
//   potentials  init_elec_hole_kernel (bse_cplx/init.c:8-268): bare v(k) and
//               screened W(k) from erf-regularised 1/r on the grid, FFT'd with
//               the same FFT engine as H psi, phase-shifted to the box centre,
//               plus the analytic long-range terms, times 1/N -- FP64.
//   kernels     calc_eh_kernel_cplx (bse_cplx/coulomb.c:20-738): the direct
//               kernel K^d[(a,i),(b,j)] = dv sum_r [W * rho_ab](r) rho_ji(r) and
//               the exchange kernel K^x[(a,i),(b,j)] = -dv sum_r [v * rho_ai](r)
//               rho_jb(r), rho_xy = sum_sigma conj(psi_x) psi_y.  The reference
//               loops over pairs with one FFT convolution and one length-N dot
//               per matrix element; here every pair density is formed and
//               convolved in batches (the FFT engine's hartree mode), and each
//               kernel becomes one complex GEMM over the grid,
//               [pairs x N] x [N x pairs], with FP64 split-K partial sums.
//   solve       build_h0_mat / build_BSE_mat (bse_cplx/mod_bse.c:54-148) and
//               bethe_salpeter (bse_cplx/bethe-salpeter.c:7-350):
//               H = diag(e_a - e_i) - (K^d + K^x), Hermitian FP64 eigensolve on
//               the GPU (the same Jacobi solver as the subspace step), and the
//               exciton expectation values <H>, <K^d>, <K^x>, <h0>.
//   dipoles     calc_elec_dipole (bse_cplx/dipole.c:7-158) and the exciton
//               transition dipoles / oscillator strengths of calc_optical_exc
//               (bse_cplx/optical.c:6-99).
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <vector>

#include "fbse_internal.cuh"

namespace fbse {

int jacobi_eig_dev(fbse_ctx *c, double2 *A, double2 *V, int n, std::vector<double> &w);
int zgemm_dev(fbse_ctx *c, int m, int p, int k, const double2 *A, int lda, bool ah, const double2 *B, int ldb, bool bh,
              double2 *C, int ldc);
int forward_fft64(fbse_ctx *c, double2 *data, double2 *work);

static unsigned gridn(long n, int t = 256)
{
  long g = (n + t - 1) / t;
  if (g > 152L * 32) g = 152L * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
// potentials
// ---------------------------------------------------------------------------
__device__ double coulomb_erf(double r, double gamma)
{  // calc_coulomb (bse_cplx/init.c:271-291)
  if (r < 1.0e-10) return 2.0 * gamma / 1.7724538509055160273;
  return erf(gamma * r) / r;
}

__global__ void k_pot_real(int nx, int ny, int nz, const double *gx, const double *gy, const double *gz, double boxl2,
                           double gamma, double gammaeps, double ex_1, double ey_1, double ez_1, double sqe_1,
                           double2 *potr, double2 *potrx)
{
  const long N = (long)nx * ny * nz;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int jx = (int)(g % nx), jy = (int)((g / nx) % ny), jz = (int)(g / ((long)nx * ny));
    const double x2 = gx[jx] * gx[jx], y2 = gy[jy] * gy[jy], z2 = gz[jz] * gz[jz];
    const double r2 = x2 + y2 + z2;
    double a = 0.0, b = 0.0;
    if (r2 < boxl2) {
      a = coulomb_erf(sqrt(x2 + y2 + z2), gamma);
      b = sqe_1 * coulomb_erf(sqrt(ex_1 * x2 + ey_1 * y2 + ez_1 * z2), gammaeps);
    }
    potr[g] = make_double2(a, 0.0);
    potrx[g] = make_double2(b, 0.0);
  }
}

__global__ void k_pot_kspace(int nx, int ny, int nz, double dkx, double dky, double dkz, double dv, double gamma2,
                             double epsx, double epsy, double epsz, double sqrk0, double ngrid_1, double2 *bare,
                             double2 *scr)
{
  const long N = (long)nx * ny * nz;
  for (long g = blockIdx.x * (long)blockDim.x + threadIdx.x; g < N; g += (long)gridDim.x * blockDim.x) {
    const int jx = (int)(g % nx), jy = (int)((g / nx) % ny), jz = (int)(g / ((long)nx * ny));
    // k^2 tables of init.c:160-165: index j and n - j share (j dk)^2
    const int mx = (jx <= nx / 2) ? jx : nx - jx, my = (jy <= ny / 2) ? jy : ny - jy,
              mz = (jz <= nz / 2) ? jz : nz - jz;
    const double x2 = (mx * dkx) * (mx * dkx), y2 = (my * dky) * (my * dky), z2 = (mz * dkz) * (mz * dkz);
    const double alpha = 3.14159265358979323846 * (double)(jx + jy + jz + N / 2);
    const double ca = cos(alpha), sa = sin(alpha);
    double2 t = bare[g];
    double2 v = make_double2((t.x * ca - t.y * sa) * dv, (t.x * sa + t.y * ca) * dv);
    v.x += 4.0 * 3.14159265358979323846 / (x2 + y2 + z2 + gamma2);
    bare[g] = make_double2(v.x * ngrid_1, v.y * ngrid_1);
    t = scr[g];
    v = make_double2((t.x * ca - t.y * sa) * dv, (t.x * sa + t.y * ca) * dv);
    const double ek = epsx * x2 + epsy * y2 + epsz * z2;
    v.x += 4.0 * 3.14159265358979323846 * (1.0 - exp(-0.25 * ek / sqrk0)) / (ek + 1.0e-10);
    scr[g] = make_double2(v.x * ngrid_1, v.y * ngrid_1);
  }
}

// ---------------------------------------------------------------------------
// pair densities rho[p][r] = sum_sigma conj(psi_x(r,sigma)) psi_y(r,sigma)
// for a list of (x, y) state pairs (indices into psi_qp)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_pair_density(const double2 *__restrict__ psi, long nsg, long ngrid, int nspin,
                               const int2 *__restrict__ pairs, int npairs, C<T> *__restrict__ rho)
{
  const long total = (long)npairs * ngrid;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int p = (int)(e / ngrid);
    const long r = e - (long)p * ngrid;
    const int2 xy = pairs[p];
    double sr = 0.0, si = 0.0;
    for (int s = 0; s < nspin; s++) {
      const double2 a = psi[(long)xy.x * nsg + s * ngrid + r], b = psi[(long)xy.y * nsg + s * ngrid + r];
      sr += a.x * b.x + a.y * b.y;  // conj(a) b
      si += a.x * b.y - a.y * b.x;
    }
    rho[e] = mk<T>((T)sr, (T)si);
  }
}

// ---------------------------------------------------------------------------
// C[m][n] = scale * sum_r A[m][r] B[n][r] (no conjugation), complex, A and B in
// the working precision; split-K partial sums in FP64, tile 64 x 64
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_cgemm_nt(const C<T> *__restrict__ A, int ma, const C<T> *__restrict__ B,
                                                  int nb, long L, long kchunk, double2 *__restrict__ part)
{
  constexpr int TM = 64, TK = 16;
  __shared__ T Ar[TK][TM], Ai[TK][TM], Br[TK][TM], Bi[TK][TM];
  const int i0 = blockIdx.x * TM, j0 = blockIdx.y * TM;
  const long k0 = blockIdx.z * kchunk;
  const long k1 = min(L, k0 + kchunk);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  T cr[4][4], ci[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) { cr[a][b] = 0; ci[a][b] = 0; }
  for (long kb = k0; kb < k1; kb += TK) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = ty + 16 * q;
      const long k = kb + tx;
      const C<T> va = (i0 + r < ma && k < k1) ? A[(long)(i0 + r) * L + k] : mk<T>(0, 0);
      const C<T> vb = (j0 + r < nb && k < k1) ? B[(long)(j0 + r) * L + k] : mk<T>(0, 0);
      Ar[tx][r] = va.x; Ai[tx][r] = va.y;
      Br[tx][r] = vb.x; Bi[tx][r] = vb.y;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++) {
      T ar[4], ai[4], br[4], bi[4];
#pragma unroll
      for (int a = 0; a < 4; a++) {
        ar[a] = Ar[kk][ty + 16 * a]; ai[a] = Ai[kk][ty + 16 * a];
        br[a] = Br[kk][tx + 16 * a]; bi[a] = Bi[kk][tx + 16 * a];
      }
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          cr[a][b] += ar[a] * br[b] - ai[a] * bi[b];
          ci[a][b] += ar[a] * bi[b] + ai[a] * br[b];
        }
    }
    __syncthreads();
  }
  double2 *P = part + (long)blockIdx.z * ma * nb;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      if (i < ma && j < nb) P[(long)i * nb + j] = make_double2((double)cr[a][b], (double)ci[a][b]);
    }
}

__global__ void k_sum_parts(const double2 *__restrict__ part, int nchunk, long nn, double scale,
                            double2 *__restrict__ out)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nn; e += (long)gridDim.x * blockDim.x) {
    double r = 0, im = 0;
    for (int c = 0; c < nchunk; c++) { r += part[(long)c * nn + e].x; im += part[(long)c * nn + e].y; }
    out[e] = make_double2(r * scale, im * scale);
  }
}

// the mixed path's contraction runs on the tensor cores (tcgemm.cu, split-TF32
// products, FP32 accumulation, FP64 split-K sums); fbse_tuning.bse_simt = 1
// keeps it on the SIMT kernel below
static bool bse_tensor_cores(fbse_ctx *c) { return c->tune.bse_simt == 0; }

template <typename T>
static int cgemm_nt(fbse_ctx *c, const C<T> *A, int ma, const C<T> *B, int nb, long L, double scale, double2 *out)
{
  if constexpr (sizeof(T) == 4) {
    if (bse_tensor_cores(c))
      return tc_complex_nt<float>(c, reinterpret_cast<const float *>(A), ma, reinterpret_cast<const float *>(B), nb,
                                  L, false, scale, out);
  }
  long nchunk = std::max<long>(1, std::min<long>(64, L / 8192));
  // keep the partials bounded (64 x ma x nb complex doubles)
  while (nchunk > 1 && (double)nchunk * ma * nb * 16.0 > 8.0e9) nchunk /= 2;
  const long kchunk = (L + nchunk - 1) / nchunk;
  double2 *part = nullptr;
  if (cudaMalloc(&part, (size_t)nchunk * ma * nb * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_OOM, "bse gemm partials");
  }
  dim3 g((ma + 63) / 64, (nb + 63) / 64, (unsigned)nchunk);
  k_cgemm_nt<T><<<g, 256, 0, c->stream>>>(A, ma, B, nb, L, kchunk, part);
  int rc = FBSE_OK;
  if (cudaGetLastError() != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "bse gemm launch");
  FBSE_COUNT(1);
  if (!rc) {
    k_sum_parts<<<gridn((long)ma * nb), 256, 0, c->stream>>>(part, (int)nchunk, (long)ma * nb, scale, out);
    FBSE_COUNT(1);
    if (cudaGetLastError() != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "bse gemm reduce");
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(part);
  return rc;
}

// scatter the (pair x pair) GEMM result into the n_xton x n_xton kernel:
// direct: Kd[ibs][jbs] = G[(a,b)][(j,i)], ibs = a*nh + i, jbs = b*nh + j
// exchange: Kx[ibs][jbs] = G[ibs][jbs]; only ibs >= jbs is kept
__global__ void k_scatter_direct(const double2 *__restrict__ G, int ne, int nh, double2 *__restrict__ K)
{
  const long nx = (long)ne * nh;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nx * nx; e += (long)gridDim.x * blockDim.x) {
    const long ibs = e / nx, jbs = e % nx;
    if (ibs < jbs) { K[e] = make_double2(0, 0); continue; }
    const long a = ibs / nh, i = ibs % nh, b = jbs / nh, j = jbs % nh;
    K[e] = G[(a * ne + b) * ((long)nh * nh) + (j * nh + i)];
  }
}

__global__ void k_lower_only(double2 *K, long n)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n * n; e += (long)gridDim.x * blockDim.x)
    if (e / n < e % n) K[e] = make_double2(0, 0);
}

// pair densities for a list of (x, y) pairs into dst[p][r]; with conv set, each
// density is convolved with that k-space potential (hartree, bse_cplx/hartree.c)
// in batches: wk holds 2 x batch grids (densities, FFT scratch)
template <typename T>
static int conv_batches(fbse_ctx *c, const double *psi_qp, const std::vector<int2> &pairs, C<T> *dst, C<T> *wk,
                        long batch, int2 *dpairs, const double2 *conv)
{
  const long N = c->ngrid;
  const long nsg = (long)c->nspin * N;
  FBSE_CUDA(c, cudaMemcpyAsync(dpairs, pairs.data(), pairs.size() * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
  for (long p0 = 0; p0 < (long)pairs.size(); p0 += batch) {
    const int np = (int)std::min<long>(batch, (long)pairs.size() - p0);
    C<T> *tgt = dst + p0 * N;
    k_pair_density<T><<<gridn((long)np * N), 256, 0, c->stream>>>((const double2 *)psi_qp, nsg, N, c->nspin,
                                                                     dpairs + p0, np, conv ? wk : tgt);
    FBSE_CHECK_LAUNCH(c);
    if (conv) {
      const int r2 = conv_apply<T>(c, wk, tgt, wk + batch * N, np, conv);
      if (r2) return r2;
    }
  }
  return FBSE_OK;
}

template <typename T>
static int eh_kernels_t(fbse_ctx *c, const double *psi_qp, long nh, long ne, long lumo, const double *pot_bare,
                        const double *pot_scr, double *direct, double *exchange)
{
  const long N = c->ngrid;
  const long nx = ne * nh;
  int rc = FBSE_OK;
  const long batch = std::max<long>(1, std::min<long>(64, (long)(2.0e9 / (N * sizeof(C<T>)))));
  C<T> *P = nullptr, *Q = nullptr, *wk = nullptr;
  int2 *dpairs = nullptr;
  double2 *G = nullptr;
  const long maxrows = std::max(ne * ne, std::max(nh * nh, nx));
  auto fail = [&](const char *m) { cudaGetLastError(); rc = set_err(c, FBSE_ERR_OOM, m); };
  if (cudaMalloc(&P, (size_t)maxrows * N * sizeof(C<T>)) != cudaSuccess) fail("bse pair densities");
  else if (cudaMalloc(&Q, (size_t)maxrows * N * sizeof(C<T>)) != cudaSuccess) fail("bse pair densities");
  else if (cudaMalloc(&wk, (size_t)2 * batch * N * sizeof(C<T>)) != cudaSuccess) fail("bse fft scratch");
  else if (cudaMalloc(&dpairs, (size_t)maxrows * sizeof(int2)) != cudaSuccess) fail("bse pairs");
  else if (cudaMalloc(&G, (size_t)(ne * ne) * (nh * nh) * sizeof(double2)) != cudaSuccess) fail("bse G");
  std::vector<int2> pr;
  do {
    if (rc) break;
    // ---- direct: P[(a,b)] = W * rho_ab, Q[(j,i)] = rho_ji
    pr.clear();
    for (long a = 0; a < ne; a++)
      for (long b = 0; b < ne; b++) pr.push_back(make_int2((int)(lumo + a), (int)(lumo + b)));
    if ((rc = conv_batches<T>(c, psi_qp, pr, P, wk, batch, dpairs, (const double2 *)pot_scr))) break;
    pr.clear();
    for (long j = 0; j < nh; j++)
      for (long i = 0; i < nh; i++) pr.push_back(make_int2((int)j, (int)i));
    if ((rc = conv_batches<T>(c, psi_qp, pr, Q, wk, batch, dpairs, nullptr))) break;
    if ((rc = cgemm_nt<T>(c, P, (int)(ne * ne), Q, (int)(nh * nh), N, c->dv, G))) break;
    k_scatter_direct<<<gridn(nx * nx), 256, 0, c->stream>>>(G, (int)ne, (int)nh, (double2 *)direct);
    FBSE_LAUNCH_OR_BREAK(c, rc);
    // ---- exchange: P[(a,i)] = v * rho_ai (ibs order), Q[(b,j)] = rho_jb (jbs order)
    pr.clear();
    for (long a = 0; a < ne; a++)
      for (long i = 0; i < nh; i++) pr.push_back(make_int2((int)(lumo + a), (int)i));
    if ((rc = conv_batches<T>(c, psi_qp, pr, P, wk, batch, dpairs, (const double2 *)pot_bare))) break;
    pr.clear();
    for (long b = 0; b < ne; b++)
      for (long j = 0; j < nh; j++) pr.push_back(make_int2((int)j, (int)(lumo + b)));
    if ((rc = conv_batches<T>(c, psi_qp, pr, Q, wk, batch, dpairs, nullptr))) break;
    if ((rc = cgemm_nt<T>(c, P, (int)nx, Q, (int)nx, N, -c->dv, (double2 *)exchange))) break;
    k_lower_only<<<gridn(nx * nx), 256, 0, c->stream>>>((double2 *)exchange, nx);
    FBSE_LAUNCH_OR_BREAK(c, rc);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "bse kernels");
  } while (0);
  cudaStreamSynchronize(c->stream);
  if (P) cudaFree(P);
  if (Q) cudaFree(Q);
  if (wk) cudaFree(wk);
  if (dpairs) cudaFree(dpairs);
  if (G) cudaFree(G);
  return rc;
}

}  // namespace fbse

namespace fbse {

// ---------------------------------------------------------------------------
// BSE matrix, eigensolve and expectation values
// ---------------------------------------------------------------------------
// H = h0 - (Kd + Kx) from the lower triangles (build_BSE_mat's Hermitian fill,
// mod_bse.c:104-128, diagonal made real); also fills Kd, Kx to full Hermitian
__global__ void k_bse_matrix(double2 *Kd, double2 *Kx, const double *__restrict__ eval, int nh, int ne, long lumo,
                             double2 *H)
{
  const long n = (long)nh * ne;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n * n; e += (long)gridDim.x * blockDim.x) {
    const long i = e / n, j = e % n;
    if (i < j) continue;
    double2 d = Kd[i * n + j], x = Kx[i * n + j];
    if (i == j) { d.y = 0; x.y = 0; }
    Kd[i * n + j] = d;
    Kx[i * n + j] = x;
    Kd[j * n + i] = make_double2(d.x, -d.y);
    Kx[j * n + i] = make_double2(x.x, -x.y);
    double2 b = make_double2(d.x + x.x, d.y + x.y);
    if (i == j) {
      const long a = i / nh, h = i % nh;
      const double h0 = eval[lumo + a] - eval[h];  // build_h0_mat (mod_bse.c:54-87)
      H[i * n + i] = make_double2(h0 - b.x, 0.0);
    } else {
      H[i * n + j] = make_double2(-b.x, -b.y);
      H[j * n + i] = make_double2(-b.x, b.y);
    }
  }
}

// out[s] = Re sum_l conj(C[l][s]) (M C)[l][s]
__global__ void k_coldots(const double2 *__restrict__ Cm, const double2 *__restrict__ MC, long n, double *out)
{
  for (long s = blockIdx.x * (long)blockDim.x + threadIdx.x; s < n; s += (long)gridDim.x * blockDim.x) {
    double r = 0;
    for (long l = 0; l < n; l++) {
      const double2 a = Cm[l * n + s], b = MC[l * n + s];
      r += a.x * b.x + a.y * b.y;
    }
    out[s] = r;
  }
}

__global__ void k_diag_h0(const double *__restrict__ eval, int nh, int ne, long lumo, double2 *D)
{
  const long n = (long)nh * ne;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n * n; e += (long)gridDim.x * blockDim.x) {
    const long i = e / n, j = e % n;
    D[e] = make_double2(i == j ? eval[lumo + i / nh] - eval[i % nh] : 0.0, 0.0);
  }
}

__global__ void k_permute_columns(const double2 *__restrict__ U, const int *__restrict__ perm, long n, double2 *out)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n * n; e += (long)gridDim.x * blockDim.x)
    out[e] = U[(e / n) * n + perm[e % n]];
}

// ---------------------------------------------------------------------------
// dipoles: mu[(i * ne + a) * 3 + d] = dv sum_{r,sigma} conj(psi_i) x_d psi_a
// ---------------------------------------------------------------------------
__global__ void k_dipoles(const double2 *__restrict__ psi, long nsg, long ngrid, int nspin, int nx, int ny,
                          const double *__restrict__ gx, const double *__restrict__ gy, const double *__restrict__ gz,
                          int nh, int ne, long lumo, double dv, double2 *__restrict__ mu)
{
  const int pair = blockIdx.x;
  const int i = pair / ne, a = pair % ne;
  const double2 *pi = psi + (long)i * nsg, *pa = psi + (long)(lumo + a) * nsg;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (long g = threadIdx.x; g < ngrid; g += blockDim.x) {
    const double x = gx[g % nx], y = gy[(g / nx) % ny], z = gz[g / ((long)nx * ny)];
    for (int sp = 0; sp < nspin; sp++) {
      const double2 u = pi[sp * ngrid + g], v = pa[sp * ngrid + g];
      const double tr = u.x * v.x + u.y * v.y, ti = u.x * v.y - u.y * v.x;
      s[0] += tr * x; s[1] += ti * x;
      s[2] += tr * y; s[3] += ti * y;
      s[4] += tr * z; s[5] += ti * z;
    }
  }
  __shared__ double red[32][6];
  for (int k = 0; k < 6; k++) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[w][threadIdx.x];
    red[0][threadIdx.x] = v;  // each thread reads only its own column above
  }
  __syncthreads();
  if (threadIdx.x < 3)
    mu[(long)(i * ne + a) * 3 + threadIdx.x] =
        make_double2(dv * red[0][2 * threadIdx.x], dv * red[0][2 * threadIdx.x + 1]);
}

// exciton transition dipoles mu_j = sum_ibs C[ibs][j] mu_(i,a) (calc_optical_exc,
// bse_cplx/optical.c:36-57); one thread per (exciton, component)
__global__ void k_xton_dipoles(const double2 *__restrict__ Cm, const double2 *__restrict__ mu, int nh, int ne,
                               double2 *__restrict__ out)
{
  const long n = (long)nh * ne;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < 3 * n; t += (long)gridDim.x * blockDim.x) {
    const long j = t / 3;
    const int d = (int)(t % 3);
    double re = 0, im = 0;
    for (long ibs = 0; ibs < n; ibs++) {
      const long a = ibs / nh, i = ibs % nh;
      const double2 cc = Cm[ibs * n + j], m = mu[(i * ne + a) * 3 + d];
      re += cc.x * m.x - cc.y * m.y;
      im += cc.x * m.y + cc.y * m.x;
    }
    out[j * 3 + d] = make_double2(re, im);
  }
}

// ---------------------------------------------------------------------------
// magnetic transition dipoles (calc_mag_dipole, bse_cplx/dipole.c:160-331):
// p_d psi_a = IFFT(k_d FFT psi_a) per spin block (p_operator,
// bse_cplx/ang_mom_operators.c:105-170, k_d from init_kvec with the 1/N of the
// two unnormalised transforms), L psi = -(r x p psi) (l_operator, :6-52), and
//   m[(i * ne + a) * 3 + d] = (dv / 2) sum_{r,sigma} conj(psi_i) (L psi_a)_d
// One CTA per hole i for the electron a whose p psi_a is in P[3][nspin][N].
// ---------------------------------------------------------------------------
__global__ void k_mag_dots(const double2 *__restrict__ psi, long nsg, long ngrid, int nspin, int nx, int ny,
                           const double *__restrict__ gx, const double *__restrict__ gy, const double *__restrict__ gz,
                           const double2 *__restrict__ P, int ne, int a, double dv, double2 *__restrict__ m)
{
  const int i = blockIdx.x;
  const double2 *pi = psi + (long)i * nsg;
  const double2 *Px = P, *Py = P + nsg, *Pz = P + 2 * nsg;
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (long g = threadIdx.x; g < ngrid; g += blockDim.x) {
    const double x = gx[g % nx], y = gy[(g / nx) % ny], z = gz[g / ((long)nx * ny)];
    for (int sp = 0; sp < nspin; sp++) {
      const long q = sp * ngrid + g;
      const double2 u = pi[q], px = Px[q], py = Py[q], pz = Pz[q];
      const double2 l[3] = {make_double2(-(y * pz.x - z * py.x), -(y * pz.y - z * py.y)),
                            make_double2(-(z * px.x - x * pz.x), -(z * px.y - x * pz.y)),
                            make_double2(-(x * py.x - y * px.x), -(x * py.y - y * px.y))};
#pragma unroll
      for (int d = 0; d < 3; d++) {
        s[2 * d] += u.x * l[d].x + u.y * l[d].y;  // conj(u) l
        s[2 * d + 1] += u.x * l[d].y - u.y * l[d].x;
      }
    }
  }
  __shared__ double red[32][6];
  for (int k = 0; k < 6; k++) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[w][threadIdx.x];
    red[0][threadIdx.x] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3)
    m[(long)(i * ne + a) * 3 + threadIdx.x] =
        make_double2(0.5 * dv * red[0][2 * threadIdx.x], 0.5 * dv * red[0][2 * threadIdx.x + 1]);
}

// real quasiparticle states as complex ones (imaginary part 0), and the real
// parts of complex kernels back, scaled
__global__ void k_real_to_cplx(const double *__restrict__ src, double2 *__restrict__ dst, long n)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    dst[e] = make_double2(src[e], 0.0);
}

__global__ void k_real_part(const double2 *__restrict__ src, double *__restrict__ dst, long n, double scale)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x)
    dst[e] = scale * src[e].x;
}

// ---------------------------------------------------------------------------
// quasiparticle spin and angular-momentum matrices (calc_qp_spin_mtrx,
// calc_qp_ang_mom_mtrx, bse_cplx/angular.c:7-690) for spinor states.
// l_operator's L'psi = -(r x p psi) (ang_mom_operators.c:6-52) per spin block:
// k_cross forms component d (or all three) of L' from P = (p_x, p_y, p_z) psi.
// ---------------------------------------------------------------------------
__global__ void k_cross(const double2 *__restrict__ P, long nsg, long ngrid, int nx, int ny,
                        const double *__restrict__ gx, const double *__restrict__ gy, const double *__restrict__ gz,
                        int only, double2 *__restrict__ out, int accumulate)
{
  // out[d][q] (d = 0..2, or only component `only` into out[0] when only >= 0)
  const double2 *Px = P, *Py = P + nsg, *Pz = P + 2 * nsg;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < nsg; q += (long)gridDim.x * blockDim.x) {
    const long g = q % ngrid;
    const double x = gx[g % nx], y = gy[(g / nx) % ny], z = gz[g / ((long)nx * ny)];
    const double2 px = Px[q], py = Py[q], pz = Pz[q];
    const double2 l[3] = {make_double2(-(y * pz.x - z * py.x), -(y * pz.y - z * py.y)),
                          make_double2(-(z * px.x - x * pz.x), -(z * px.y - x * pz.y)),
                          make_double2(-(x * py.x - y * px.x), -(x * py.y - y * px.y))};
    if (only < 0) {
      out[q] = l[0];
      out[nsg + q] = l[1];
      out[2 * nsg + q] = l[2];
    } else {
      const double2 v = l[only];
      out[q] = accumulate ? make_double2(out[q].x + v.x, out[q].y + v.y) : v;
    }
  }
}

// for the state i whose L'_d psi_i (Lp[3]) and sum_d L'_d L'_d psi_i (L2) are
// given, and every partner j of its block (CTA j, ncols partners from j0):
//   r[0..2] = sum conj(psi_j) L'_d psi_i, r[3] = sum conj(psi_j) L2,
//   r[4]    = sum [conj(psi_j,dn) L'x_up + conj(psi_j,up) L'x_dn
//                  + i conj(psi_j,dn) L'y_up - i conj(psi_j,up) L'y_dn
//                  + conj(psi_j,up) L'z_up - conj(psi_j,dn) L'z_dn]     (the L.S sum)
//   r[5..7] = the sx, sy, sz sums of calc_qp_spin_mtrx on psi_j, psi_i
// (complex, unscaled) into out[(j - j0) * 8 + k]
__global__ void k_ang_dots(const double2 *__restrict__ psi, long nsg, long ngrid, long i, long j0,
                           const double2 *__restrict__ Lp, const double2 *__restrict__ L2,
                           double2 *__restrict__ out)
{
  const long j = j0 + blockIdx.x;
  const double2 *pj = psi + j * nsg, *pi = psi + i * nsg;
  double s[16];
#pragma unroll
  for (int k = 0; k < 16; k++) s[k] = 0.0;
  auto acc = [&](int k, double2 a, double2 b, double sr, double si) {
    // s[k] += (sr + i si) conj(a) b
    const double tr = a.x * b.x + a.y * b.y, ti = a.x * b.y - a.y * b.x;
    s[2 * k] += sr * tr - si * ti;
    s[2 * k + 1] += sr * ti + si * tr;
  };
  for (long g = threadIdx.x; g < ngrid; g += blockDim.x) {
    const double2 ju = pj[g], jd = pj[ngrid + g], iu = pi[g], id = pi[ngrid + g];
    for (int sp = 0; sp < 2; sp++) {
      const double2 jv = sp ? jd : ju;
      const long q = sp * ngrid + g;
      acc(0, jv, Lp[q], 1, 0);
      acc(1, jv, Lp[nsg + q], 1, 0);
      acc(2, jv, Lp[2 * nsg + q], 1, 0);
      acc(3, jv, L2[q], 1, 0);
    }
    acc(4, jd, Lp[g], 1, 0);
    acc(4, ju, Lp[ngrid + g], 1, 0);
    acc(4, jd, Lp[nsg + g], 0, 1);
    acc(4, ju, Lp[nsg + ngrid + g], 0, -1);
    acc(4, ju, Lp[2 * nsg + g], 1, 0);
    acc(4, jd, Lp[2 * nsg + ngrid + g], -1, 0);
    acc(5, jd, iu, 1, 0);
    acc(5, ju, id, 1, 0);
    acc(6, jd, iu, 0, 1);
    acc(6, ju, id, 0, -1);
    acc(7, ju, iu, 1, 0);
    acc(7, jd, id, -1, 0);
  }
  __shared__ double red[32][16];
  for (int k = 0; k < 16; k++) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 16) {
    double v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[w][threadIdx.x];
    red[0][threadIdx.x] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8)
    out[(long)blockIdx.x * 8 + threadIdx.x] = make_double2(red[0][2 * threadIdx.x], red[0][2 * threadIdx.x + 1]);
}

// init_kvec (ang_mom_operators.c:90-103): k[j] = j dk norm, k[n-j] = -j dk norm
// for j = 1..n/2 in that order (for even n the second write leaves k[n/2] < 0)
static void init_kvec(std::vector<double> &k, long n, double dk, double norm)
{
  k.assign(n, 0.0);
  const long npos = (n % 2 == 0) ? n / 2 : (n - 1) / 2;
  for (long j = 1; j <= npos; j++) {
    k[j] = j * dk * norm;
    k[n - j] = -(j * dk * norm);
  }
}

}  // namespace fbse

using namespace fbse;

extern "C" {

int fbse_bse_potentials(fbse_ctx *c, const double *gx, const double *gy, const double *gz, double xmin, double ymin,
                        double zmin, double eps_x, double eps_y, double eps_z, double *pot_bare, double *pot_screened)
{
  if (!c || !gx || !gy || !gz || !pot_bare || !pot_screened || !(eps_x > 0) || !(eps_y > 0) || !(eps_z > 0))
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_bse_potentials: bad arguments") : FBSE_ERR_ARG;
  const long N = c->ngrid;
  // init_elec_hole_kernel (bse_cplx/init.c:79-103): gamma from the smallest half box
  const double xm = std::fabs(xmin), ym = std::fabs(ymin), zm = std::fabs(zmin);
  double minr, boxl;
  if (xm < ym && xm < zm) { minr = xm; boxl = (double)c->nx * c->dx; }
  else if (ym < zm && ym < xm) { minr = ym; boxl = (double)c->ny * c->dy; }
  else { minr = zm; boxl = (double)c->nz * c->dz; }
  const double gamma = 7.0 / (2.0 * minr), gamma2 = gamma * gamma;
  const double ex_1 = 1.0 / eps_x, ey_1 = 1.0 / eps_y, ez_1 = 1.0 / eps_z;
  const double sqe_1 = 1.0 / std::sqrt(eps_x * eps_y * eps_z);
  const double sqrtaveps = std::sqrt((eps_x + eps_y + eps_z) / 3.0);
  const double gammaeps = gamma * sqrtaveps;
  const double sqrk0 = gamma2 * (sqrtaveps * sqrtaveps);
  double *dg = nullptr;
  double2 *work = nullptr;
  int rc = FBSE_OK;
  if (cudaMalloc(&dg, (c->nx + c->ny + c->nz) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&work, (size_t)N * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    if (dg) cudaFree(dg);
    return set_err(c, FBSE_ERR_OOM, "fbse_bse_potentials");
  }
  do {
    h2d(c->stream, dg, gx, c->nx * sizeof(double));
    h2d(c->stream, dg + c->nx, gy, c->ny * sizeof(double));
    h2d(c->stream, dg + c->nx + c->ny, gz, c->nz * sizeof(double));
    k_pot_real<<<gridn(N), 256, 0, c->stream>>>((int)c->nx, (int)c->ny, (int)c->nz, dg, dg + c->nx,
                                                 dg + c->nx + c->ny, boxl * boxl, gamma, gammaeps, ex_1, ey_1, ez_1,
                                                 sqe_1, (double2 *)pot_bare, (double2 *)pot_screened);
    FBSE_COUNT(1);
    if ((rc = forward_fft64(c, (double2 *)pot_bare, work))) break;
    if ((rc = forward_fft64(c, (double2 *)pot_screened, work))) break;
    // reciprocal spacing 2 pi / (n d) on every axis (init.c:108-110)
    const double dkx = 6.28318530717958647692 / ((double)c->nx * c->dx);
    const double dky = 6.28318530717958647692 / ((double)c->ny * c->dy);
    const double dkz = 6.28318530717958647692 / ((double)c->nz * c->dz);
    k_pot_kspace<<<gridn(N), 256, 0, c->stream>>>((int)c->nx, (int)c->ny, (int)c->nz, dkx, dky, dkz, c->dv, gamma2,
                                                   eps_x, eps_y, eps_z, sqrk0, 1.0 / (double)N,
                                                   (double2 *)pot_bare, (double2 *)pot_screened);
    FBSE_COUNT(1);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_potentials");
  } while (0);
  cudaStreamSynchronize(c->stream);
  cudaFree(dg);
  cudaFree(work);
  return rc;
}

int fbse_bse_kernel(fbse_ctx *c, const double *psi_qp, long n_h, long n_e, long lumo_idx, const double *pot_bare,
                    const double *pot_screened, double *direct, double *exchange)
{
  if (!c || !psi_qp || !pot_bare || !pot_screened || !direct || !exchange || n_h < 1 || n_e < 1 || lumo_idx < n_h)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_bse_kernel: bad arguments") : FBSE_ERR_ARG;
  if (!c->is_complex) return set_err(c, FBSE_ERR_UNSUPPORTED, "fbse_bse_kernel: complex quasiparticle states required");
  if (c->precision == FBSE_MIXED)
    return eh_kernels_t<float>(c, psi_qp, n_h, n_e, lumo_idx, pot_bare, pot_screened, direct, exchange);
  return eh_kernels_t<double>(c, psi_qp, n_h, n_e, lumo_idx, pot_bare, pot_screened, direct, exchange);
}

int fbse_bse_kernel_real(fbse_ctx *c, const double *psi_qp, long n_h, long n_e, long lumo_idx, const double *pot_bare,
                         const double *pot_screened, double *direct, double *exchange)
{
  if (!c || !psi_qp || !pot_bare || !pot_screened || !direct || !exchange || n_h < 1 || n_e < 1 || lumo_idx < n_h)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_bse_kernel_real: bad arguments") : FBSE_ERR_ARG;
  if (c->nspin != 1) return set_err(c, FBSE_ERR_UNSUPPORTED, "fbse_bse_kernel_real: one spin component per state");
  const long N = c->ngrid, nq = lumo_idx + n_e, nx = n_h * n_e;
  double2 *pc = nullptr, *dc = nullptr, *xc = nullptr;
  if (cudaMalloc(&pc, nq * N * sizeof(double2)) != cudaSuccess || cudaMalloc(&dc, nx * nx * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&xc, nx * nx * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    if (pc) cudaFree(pc);
    if (dc) cudaFree(dc);
    return set_err(c, FBSE_ERR_OOM, "fbse_bse_kernel_real");
  }
  int rc = FBSE_OK;
  k_real_to_cplx<<<gridn(nq * N), 256, 0, c->stream>>>(psi_qp, pc, nq * N);
  FBSE_COUNT(1);
  if (cudaGetLastError() != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_kernel_real");
  if (!rc)
    rc = c->precision == FBSE_MIXED
             ? eh_kernels_t<float>(c, (const double *)pc, n_h, n_e, lumo_idx, pot_bare, pot_screened, (double *)dc,
                                   (double *)xc)
             : eh_kernels_t<double>(c, (const double *)pc, n_h, n_e, lumo_idx, pot_bare, pot_screened, (double *)dc,
                                    (double *)xc);
  if (!rc) {
    // bse_real/coulomb.c: K^d = dv sum Re(W * rho_ab) psi_j psi_i; K^x carries the
    // singlet factor 2 (exchange = -2 sum, coulomb.c:568; hartree keeps the real
    // part of the convolution, hartree.c:31)
    k_real_part<<<gridn(nx * nx), 256, 0, c->stream>>>(dc, direct, nx * nx, 1.0);
    k_real_part<<<gridn(nx * nx), 256, 0, c->stream>>>(xc, exchange, nx * nx, 2.0);
    FBSE_COUNT(2);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_kernel_real");
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(pc);
  cudaFree(dc);
  cudaFree(xc);
  return rc;
}

int fbse_bse_solve(fbse_ctx *c, const double *eval_qp_host, long n_qp, long n_h, long n_e, long lumo_idx,
                   double *direct, double *exchange, double *xton_ene, double *coeff, double *h_exp, double *d_exp,
                   double *x_exp, double *h0_exp)
{
  if (!c || !eval_qp_host || !direct || !exchange || !xton_ene || !coeff || n_h < 1 || n_e < 1 ||
      lumo_idx + n_e > n_qp)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_bse_solve: bad arguments") : FBSE_ERR_ARG;
  const long n = n_h * n_e;
  double *ev = nullptr, *dots = nullptr;
  double2 *H = nullptr, *V = nullptr, *T1 = nullptr, *Cm = nullptr;
  int *perm_d = nullptr;
  int rc = FBSE_OK;
  if (cudaMalloc(&ev, n_qp * sizeof(double)) != cudaSuccess || cudaMalloc(&dots, 4 * n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&H, n * n * sizeof(double2)) != cudaSuccess || cudaMalloc(&V, n * n * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&T1, n * n * sizeof(double2)) != cudaSuccess || cudaMalloc(&perm_d, n * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    rc = set_err(c, FBSE_ERR_OOM, "fbse_bse_solve");
  }
  Cm = (double2 *)coeff;
  do {
    if (rc) break;
    h2d(c->stream, ev, eval_qp_host, n_qp * sizeof(double));
    k_bse_matrix<<<gridn(n * n), 256, 0, c->stream>>>((double2 *)direct, (double2 *)exchange, ev, (int)n_h, (int)n_e,
                                                       lumo_idx, H);
    FBSE_COUNT(1);
    if (cudaMemcpyAsync(T1, H, n * n * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "copy");
      break;
    }
    std::vector<double> w;
    if ((rc = jacobi_eig_dev(c, T1, V, (int)n, w))) break;
    std::vector<int> perm(n);
    for (long i = 0; i < n; i++) perm[i] = (int)i;
    std::sort(perm.begin(), perm.end(), [&](int a, int b) { return w[a] < w[b]; });
    for (long i = 0; i < n; i++) xton_ene[i] = w[perm[i]];
    if (h2d(c->stream, perm_d, perm.data(), n * sizeof(int)) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_solve upload");
      break;
    }
    k_permute_columns<<<gridn(n * n), 256, 0, c->stream>>>(V, perm_d, n, Cm);
    FBSE_COUNT(1);
    // expectation values diag(C^H M C) for M = H, Kd, Kx, h0 (bethe-salpeter.c:159-330)
    double2 *mats[3] = {H, (double2 *)direct, (double2 *)exchange};
    for (int q = 0; q < 4 && !rc; q++) {
      double2 *M = mats[q < 3 ? q : 0];
      if (q == 3) {
        k_diag_h0<<<gridn(n * n), 256, 0, c->stream>>>(ev, (int)n_h, (int)n_e, lumo_idx, V);
        FBSE_COUNT(1);
        M = V;
      }
      if ((rc = zgemm_dev(c, (int)n, (int)n, (int)n, M, (int)n, false, Cm, (int)n, false, T1, (int)n))) break;
      k_coldots<<<gridn(n), 256, 0, c->stream>>>(Cm, T1, n, dots + q * n);
      FBSE_COUNT(1);
    }
    if (rc) break;
    std::vector<double> hd(4 * n);
    if (d2h(c->stream, hd.data(), dots, 4 * n * sizeof(double)) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_solve download");
      break;
    }
    for (long i = 0; i < n; i++) {
      if (h_exp) h_exp[i] = hd[i];
      if (d_exp) d_exp[i] = hd[n + i];
      if (x_exp) x_exp[i] = hd[2 * n + i];
      if (h0_exp) h0_exp[i] = hd[3 * n + i];
    }
  } while (0);
  cudaStreamSynchronize(c->stream);
  void *bufs[] = {ev, dots, H, V, T1, perm_d};
  for (void *b : bufs)
    if (b) cudaFree(b);
  return rc;
}

int fbse_bse_dipoles(fbse_ctx *c, const double *psi_qp, const double *gx, const double *gy, const double *gz,
                     long n_h, long n_e, long lumo_idx, double *mu_host)
{
  if (!c || !psi_qp || !gx || !gy || !gz || !mu_host || n_h < 1 || n_e < 1)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_bse_dipoles: bad arguments") : FBSE_ERR_ARG;
  if (!c->is_complex) return set_err(c, FBSE_ERR_UNSUPPORTED, "fbse_bse_dipoles: complex states required");
  double *dg = nullptr;
  double2 *mu = nullptr;
  int rc = FBSE_OK;
  if (cudaMalloc(&dg, (c->nx + c->ny + c->nz) * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&mu, n_h * n_e * 3 * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    if (dg) cudaFree(dg);
    return set_err(c, FBSE_ERR_OOM, "fbse_bse_dipoles");
  }
  h2d(c->stream, dg, gx, c->nx * sizeof(double));
  h2d(c->stream, dg + c->nx, gy, c->ny * sizeof(double));
  h2d(c->stream, dg + c->nx + c->ny, gz, c->nz * sizeof(double));
  k_dipoles<<<(unsigned)(n_h * n_e), 256, 0, c->stream>>>((const double2 *)psi_qp, (long)c->nspin * c->ngrid, c->ngrid,
                                                          c->nspin, (int)c->nx, (int)c->ny, dg, dg + c->nx,
                                                          dg + c->nx + c->ny, (int)n_h, (int)n_e, lumo_idx, c->dv, mu);
  FBSE_COUNT(1);
  if (cudaGetLastError() != cudaSuccess ||
      d2h(c->stream, mu_host, mu, n_h * n_e * 3 * sizeof(double2)) != cudaSuccess)
    rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_dipoles");
  cudaFree(dg);
  cudaFree(mu);
  return rc;
}

int fbse_bse_mag_dipoles(fbse_ctx *c, const double *psi_qp, const double *gx, const double *gy, const double *gz,
                         long n_h, long n_e, long lumo_idx, double *m_host)
{
  if (!c || !psi_qp || !gx || !gy || !gz || !m_host || n_h < 1 || n_e < 1 || lumo_idx < n_h)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_bse_mag_dipoles: bad arguments") : FBSE_ERR_ARG;
  if (!c->is_complex) return set_err(c, FBSE_ERR_UNSUPPORTED, "fbse_bse_mag_dipoles: complex states required");
  const long N = c->ngrid, nsg = (long)c->nspin * N;
  // k_d multipliers in the transform's (z, y, x) order, with 1/N
  std::vector<double> kx, ky, kz;
  const double norm = 1.0 / (double)N;
  auto dk = [](long n, double d) { return 2.0 * M_PI / (n * d); };  // bse_cplx/read.c:347-349
  init_kvec(kx, c->nx, dk(c->nx, c->dx), norm);
  init_kvec(ky, c->ny, dk(c->ny, c->dy), norm);
  init_kvec(kz, c->nz, dk(c->nz, c->dz), norm);
  std::vector<double2> kq((size_t)3 * N);
  for (long g = 0; g < N; g++) {
    kq[g] = make_double2(kx[g % c->nx], 0.0);
    kq[N + g] = make_double2(ky[(g / c->nx) % c->ny], 0.0);
    kq[2 * N + g] = make_double2(kz[g / (c->nx * c->ny)], 0.0);
  }
  double2 *dk3 = nullptr, *P = nullptr, *work = nullptr, *m = nullptr;
  double *dg = nullptr;
  int rc = FBSE_OK;
  if (cudaMalloc(&dk3, 3 * N * sizeof(double2)) != cudaSuccess || cudaMalloc(&P, 3 * nsg * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&work, nsg * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&m, n_h * n_e * 3 * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&dg, (c->nx + c->ny + c->nz) * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    rc = set_err(c, FBSE_ERR_OOM, "fbse_bse_mag_dipoles");
  }
  do {
    if (rc) break;
    if (h2d(c->stream, dk3, kq.data(), 3 * N * sizeof(double2)) != cudaSuccess ||
        h2d(c->stream, dg, gx, c->nx * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dg + c->nx, gy, c->ny * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dg + c->nx + c->ny, gz, c->nz * sizeof(double)) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_mag_dipoles upload");
      break;
    }
    for (long a = 0; a < n_e && !rc; a++) {
      const double2 *pa = (const double2 *)psi_qp + (lumo_idx + a) * nsg;
      for (int d = 0; d < 3 && !rc; d++) rc = conv_apply<double>(c, pa, P + d * nsg, work, c->nspin, dk3 + d * N);
      if (rc) break;
      k_mag_dots<<<(unsigned)n_h, 256, 0, c->stream>>>((const double2 *)psi_qp, nsg, N, c->nspin, (int)c->nx,
                                                        (int)c->ny, dg, dg + c->nx, dg + c->nx + c->ny, P, (int)n_e,
                                                        (int)a, c->dv, m);
      FBSE_COUNT(1);
      if (cudaGetLastError() != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_mag_dipoles launch");
    }
    if (rc) break;
    if (d2h(c->stream, m_host, m, n_h * n_e * 3 * sizeof(double2)) != cudaSuccess)
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_mag_dipoles download");
  } while (0);
  cudaStreamSynchronize(c->stream);
  void *bufs[] = {dk3, P, work, m, dg};
  for (void *b : bufs)
    if (b) cudaFree(b);
  return rc;
}

int fbse_bse_qp_ang_mom(fbse_ctx *c, const double *psi_qp, const double *gx, const double *gy, const double *gz,
                        long n_h, long n_e, long lumo_idx, double *s_mom, double *l_mom, double *l2_mom,
                        double *ldots)
{
  if (!c || !psi_qp || !gx || !gy || !gz || !s_mom || !l_mom || !l2_mom || !ldots || n_h < 1 || n_e < 1 ||
      lumo_idx < n_h)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_bse_qp_ang_mom: bad arguments") : FBSE_ERR_ARG;
  if (!c->is_complex || c->nspin != 2)
    return set_err(c, FBSE_ERR_UNSUPPORTED, "fbse_bse_qp_ang_mom: complex spinor states required");
  const long N = c->ngrid, nsg = 2 * N;
  std::vector<double> kx, ky, kz;
  const double norm = 1.0 / (double)N;
  auto dk = [](long n, double d) { return 2.0 * M_PI / (n * d); };  // bse_cplx/read.c:347-349
  init_kvec(kx, c->nx, dk(c->nx, c->dx), norm);
  init_kvec(ky, c->ny, dk(c->ny, c->dy), norm);
  init_kvec(kz, c->nz, dk(c->nz, c->dz), norm);
  std::vector<double2> kq((size_t)3 * N);
  for (long g = 0; g < N; g++) {
    kq[g] = make_double2(kx[g % c->nx], 0.0);
    kq[N + g] = make_double2(ky[(g / c->nx) % c->ny], 0.0);
    kq[2 * N + g] = make_double2(kz[g / (c->nx * c->ny)], 0.0);
  }
  const long nmax = n_h > n_e ? n_h : n_e;
  double2 *dk3 = nullptr, *P = nullptr, *Lp = nullptr, *L2 = nullptr, *work = nullptr, *dots = nullptr;
  double *dg = nullptr;
  int rc = FBSE_OK;
  if (cudaMalloc(&dk3, 3 * N * sizeof(double2)) != cudaSuccess || cudaMalloc(&P, 3 * nsg * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&Lp, 3 * nsg * sizeof(double2)) != cudaSuccess || cudaMalloc(&L2, nsg * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&work, nsg * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&dots, nmax * 8 * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&dg, (c->nx + c->ny + c->nz) * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    rc = set_err(c, FBSE_ERR_OOM, "fbse_bse_qp_ang_mom");
  }
  const double dv = c->dv;
  const unsigned gblk = (unsigned)std::min<long>((nsg + 255) / 256, 4096);
  std::vector<double2> hd((size_t)nmax * 8);
  double2 *S = reinterpret_cast<double2 *>(s_mom), *Lm = reinterpret_cast<double2 *>(l_mom);
  double2 *L2m = reinterpret_cast<double2 *>(l2_mom), *LS = reinterpret_cast<double2 *>(ldots);
  auto conjd = [](double2 v) { return make_double2(v.x, -v.y); };
  auto sc = [](double2 v, double f) { return make_double2(f * v.x, f * v.y); };
  do {
    if (rc) break;
    if (h2d(c->stream, dk3, kq.data(), 3 * N * sizeof(double2)) != cudaSuccess ||
        h2d(c->stream, dg, gx, c->nx * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dg + c->nx, gy, c->ny * sizeof(double)) != cudaSuccess ||
        h2d(c->stream, dg + c->nx + c->ny, gz, c->nz * sizeof(double)) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_qp_ang_mom upload");
      break;
    }
    // blocks: holes (states 0..n_h-1, matrix offset 0), electrons (lumo_idx.., offset n_h^2)
    for (int blk = 0; blk < 2 && !rc; blk++) {
      const long n = blk ? n_e : n_h, s0 = blk ? lumo_idx : 0, off = blk ? n_h * n_h : 0;
      for (long i = 0; i < n && !rc; i++) {
        const double2 *pi = (const double2 *)psi_qp + (s0 + i) * nsg;
        // L' psi_i (three components), then sum_d L'_d (L'_d psi_i)
        for (int d = 0; d < 3 && !rc; d++) rc = conv_apply<double>(c, pi, P + d * nsg, work, 2, dk3 + d * N);
        if (rc) break;
        k_cross<<<gblk, 256, 0, c->stream>>>(P, nsg, N, (int)c->nx, (int)c->ny, dg, dg + c->nx, dg + c->nx + c->ny,
                                             -1, Lp, 0);
        FBSE_COUNT(1);
        for (int d = 0; d < 3 && !rc; d++) {
          for (int e = 0; e < 3 && !rc; e++) rc = conv_apply<double>(c, Lp + d * nsg, P + e * nsg, work, 2, dk3 + e * N);
          if (rc) break;
          k_cross<<<gblk, 256, 0, c->stream>>>(P, nsg, N, (int)c->nx, (int)c->ny, dg, dg + c->nx,
                                               dg + c->nx + c->ny, d, L2, d > 0);
          FBSE_COUNT(1);
        }
        if (rc) break;
        // partners: all j for the spins, j >= i for the L quantities (the
        // reference fills the rest by Hermitian conjugation)
        k_ang_dots<<<(unsigned)n, 256, 0, c->stream>>>((const double2 *)psi_qp, nsg, N, s0 + i, s0, Lp, L2, dots);
        FBSE_COUNT(1);
        if (cudaGetLastError() != cudaSuccess || d2h(c->stream, hd.data(), dots, n * 8 * sizeof(double2)) != cudaSuccess) {
          rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_qp_ang_mom");
          break;
        }
        for (long j = 0; j < n; j++) {
          const double2 *r = hd.data() + j * 8;
          // spins (angular.c:89-103 holes: -1/2 conj(s) dv; :172-183 electrons: 1/2 s dv), all pairs
          for (int d = 0; d < 3; d++)
            S[(off + i * n + j) * 3 + d] = blk ? sc(r[5 + d], 0.5 * dv) : sc(conjd(r[5 + d]), -0.5 * dv);
          if (j < i) continue;
          // L' sums: holes accumulate -conj(psi_j) L' psi_i and store conj (angular.c:404-434),
          // electrons store the sums as they are (:530-558)
          double2 l[3], l2, ls;
          for (int d = 0; d < 3; d++) l[d] = blk ? sc(r[d], dv) : sc(conjd(r[d]), -dv);
          l2 = blk ? sc(r[3], dv) : sc(conjd(r[3]), dv);
          ls = blk ? sc(r[4], 0.5 * dv) : sc(conjd(r[4]), 0.5 * dv);
          const long ut = off + i * n + j, lt = off + j * n + i;
          for (int d = 0; d < 3; d++) {
            Lm[ut * 3 + d] = l[d];
            Lm[lt * 3 + d] = conjd(l[d]);
          }
          L2m[ut] = l2;
          L2m[lt] = conjd(l2);
          LS[ut] = ls;
          LS[lt] = conjd(ls);
        }
      }
    }
  } while (0);
  cudaStreamSynchronize(c->stream);
  void *bufs[] = {dk3, P, Lp, L2, work, dots, dg};
  for (void *b : bufs)
    if (b) cudaFree(b);
  return rc;
}

int fbse_bse_optical(fbse_ctx *c, const double *coeff, const double *mu_pairs_host, long n_h, long n_e,
                     double *mu_xton_host)
{
  if (!c || !coeff || !mu_pairs_host || !mu_xton_host || n_h < 1 || n_e < 1)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_bse_optical: bad arguments") : FBSE_ERR_ARG;
  const long n = n_h * n_e;
  double2 *mu = nullptr;
  if (cudaMalloc(&mu, 2 * n * 3 * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_OOM, "fbse_bse_optical");
  }
  int rc = FBSE_OK;
  if (h2d(c->stream, mu, mu_pairs_host, n * 3 * sizeof(double2)) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "upload");
  if (!rc) {
    k_xton_dipoles<<<gridn(3 * n), 256, 0, c->stream>>>((const double2 *)coeff, mu, (int)n_h, (int)n_e, mu + 3 * n);
    FBSE_COUNT(1);
    if (cudaGetLastError() != cudaSuccess || d2h(c->stream, mu_xton_host, mu + 3 * n, n * 3 * sizeof(double2)) != cudaSuccess)
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_bse_optical");
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(mu);
  return rc;
}

}  // extern "C"
