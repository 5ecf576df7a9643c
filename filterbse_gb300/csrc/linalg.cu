// Orthogonalisation, subspace diagonalisation and sigma_E on the GPU.
//
// Replaces mod_ortho (thin SVD, filter_mpi/ortho.c:5-187), mod_diag
// (diag_H: n H psi, H_ij = dv <psi_i|H|psi_j>, dsyev/zheev, rotation,
// filter_mpi/Hmat.c:5-297) and mod_sigma (calc_sigma_E, two more H psi per
// state, filter_mpi/energy.c:383-539) with one Rayleigh-Ritz pass:
//
//   1. HPsi = H Psi                       (batched H psi, all n states)
//   2. G = dv Psi^H Psi, M = dv Psi^H HPsi (split-K GEMMs, FP64 partial sums)
//   3. G = V diag(l) V^H                  (FP64 Jacobi on the GPU)
//   4. keep l_i >= l_max * cut (the span of the left singular vectors with
//      s_i / s_0 above the cutoff), X = V_k diag(l_k)^{-1/2}
//   5. H' = X^H M X,  H' = U diag(E) U^H  (FP64 Jacobi on the GPU)
//   6. C = X U;  Psi_f = Psi C and HPsi_f = HPsi C in one pass, whose epilogue
//      forms the residual r_i = HPsi_f,i - E_i Psi_f,i and the norms
//   7. sigma_i = ||r_i|| / ||Psi_f,i||, states normalised (normalize_all).
// H is applied n times in total instead of the reference's 3n, and the Ritz
// vectors' residuals come from the same two GEMMs that build the vectors.
#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <numeric>

#include <cstdlib>

#include <type_traits>

#include "fbse_internal.cuh"

namespace cg = cooperative_groups;

namespace fbse {

int pack_states(fbse_ctx *c, const double *src, void *dst, long nsrc);
int unpack_states(fbse_ctx *c, const void *src, double *dst, long ndst);

// ---------------------------------------------------------------------------
// C[i][j] (+)= sum_l conj(A[i][l]) B[j][l]  over a K-chunk, i < n, j < n.
// A, B: n vectors of length L (complex: interleaved FP64 pairs; real: FP64).
// Tile 64 x 64 outputs per CTA, 256 threads x (4 x 4) outputs, K step 16.
// Compute type T (float for the mixed path, double for the FP64 path);
// partials are written in FP64: part[chunk][i][j].  Both products this file
// forms (Psi^H Psi and Psi^H H Psi) are Hermitian, so only tiles with
// ti <= tj are computed (blockIdx.x enumerates them) and an off-diagonal
// tile is also stored conjugate-transposed.  Shared tiles hold complex values
// as C<T> with one element of padding per K row, so the transposing stores
// (consecutive threads: consecutive k) and the float2 / double2 reads of the
// product loop are free of bank conflicts.
// ---------------------------------------------------------------------------
// (hi, lo) += x with TwoSum: hi + lo keeps the exact sum to about twice the
// working precision (Knuth, The Art of Computer Programming vol. 2, 4.2.2)
template <typename T> __device__ __forceinline__ void two_sum_acc(T &hi, T &lo, T x)
{
  const T s = hi + x;
  const T bb = s - hi;
  const T err = (hi - (s - bb)) + (x - bb);
  hi = s;
  lo += err;
}

template <typename T, bool CPLX, int MINB>
__global__ void __launch_bounds__(256, MINB) k_gram(const double *__restrict__ A, const double *__restrict__ B, int n,
                                              long L, long kchunk, double2 *__restrict__ part)
{
  constexpr int TM = 64, TK = 16;
  using E = typename std::conditional<CPLX, C<T>, T>::type;
  __shared__ E As[TK][TM + 1];
  __shared__ E Bs[TK][TM + 1];
  // tile pair (ti, tj), ti <= tj, from the linear index
  const int nt = (n + TM - 1) / TM;
  int ti = 0, rem = blockIdx.x;
  while (rem >= nt - ti) { rem -= nt - ti; ti++; }
  const int tj = ti + rem;
  const int i0 = ti * TM, j0 = tj * TM;
  const long k0 = blockIdx.z * kchunk;
  const long k1 = min(L, k0 + kchunk);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  // FP32: the sums of each K step of 16 products are added into a
  // float-float pair (hi, lo) with TwoSum (Knuth), so the long sums over the
  // grid keep about 48 bits; FP64: plain accumulation
  T accr[4][4], acci[4][4];
  T hir[4][4], hii[4][4], lor[4][4], loi[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) { accr[a][b] = 0; acci[a][b] = 0; hir[a][b] = hii[a][b] = lor[a][b] = loi[a][b] = 0; }
  for (long kb = k0; kb < k1; kb += TK) {
    // load: 64 rows x 16 k for A and B; thread t loads rows (t / 16) + 16 q, k = t % 16
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = ty + 16 * q, kk = tx;
      const long k = kb + kk;
      const bool okA = (i0 + r < n) && (k < k1);
      const bool okB = (j0 + r < n) && (k < k1);
      if constexpr (CPLX) {
        const double2 va = okA ? reinterpret_cast<const double2 *>(A)[(long)(i0 + r) * L + k] : make_double2(0, 0);
        const double2 vb = okB ? reinterpret_cast<const double2 *>(B)[(long)(j0 + r) * L + k] : make_double2(0, 0);
        As[kk][r] = mk<T>((T)va.x, (T)va.y);
        Bs[kk][r] = mk<T>((T)vb.x, (T)vb.y);
      } else {
        As[kk][r] = okA ? (T)A[(long)(i0 + r) * L + k] : T(0);
        Bs[kk][r] = okB ? (T)B[(long)(j0 + r) * L + k] : T(0);
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++) {
      T ar[4], ai[4], br[4], bi[4];
#pragma unroll
      for (int a = 0; a < 4; a++) {
        if constexpr (CPLX) {
          const C<T> u = As[kk][ty + 16 * a], v = Bs[kk][tx + 16 * a];
          ar[a] = u.x; ai[a] = u.y; br[a] = v.x; bi[a] = v.y;
        } else {
          ar[a] = As[kk][ty + 16 * a]; br[a] = Bs[kk][tx + 16 * a];
          ai[a] = bi[a] = T(0);
        }
      }
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          // conj(a) * b
          accr[a][b] += ar[a] * br[b] + (CPLX ? ai[a] * bi[b] : T(0));
          if (CPLX) acci[a][b] += ar[a] * bi[b] - ai[a] * br[b];
        }
    }
    if constexpr (sizeof(T) == 4) {
#pragma unroll
      for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) {
          two_sum_acc(hir[a][b], lor[a][b], accr[a][b]);
          accr[a][b] = 0;
          if (CPLX) {
            two_sum_acc(hii[a][b], loi[a][b], acci[a][b]);
            acci[a][b] = 0;
          }
        }
    }
    __syncthreads();
  }
  double2 *P = part + (long)blockIdx.z * n * n;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      double vr = (double)accr[a][b], vi = (double)acci[a][b];
      if constexpr (sizeof(T) == 4) {
        vr = (double)hir[a][b] + (double)lor[a][b];
        vi = (double)hii[a][b] + (double)loi[a][b];
      }
      if (i < n && j < n) {
        P[(long)i * n + j] = make_double2(vr, vi);
        if (ti != tj) P[(long)j * n + i] = make_double2(vr, -vi);
      }
    }
}

__global__ void k_sum_partials(const double2 *__restrict__ part, int nchunk, long nn, double scale,
                               double2 *__restrict__ out)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < nn; e += (long)gridDim.x * blockDim.x) {
    double r = 0, im = 0;
    for (int c = 0; c < nchunk; c++) { r += part[(long)c * nn + e].x; im += part[(long)c * nn + e].y; }
    out[e] = make_double2(r * scale, im * scale);
  }
}

// ---------------------------------------------------------------------------
// small dense FP64 complex GEMM: C[m][p] = op(A) op(B), row-major,
// opA = 'N' (A is m x k) or 'H' (A is k x m, conjugate-transposed)
// ---------------------------------------------------------------------------
__global__ void k_zgemm(int m, int p, int k, const double2 *__restrict__ A, int lda, bool ah,
                        const double2 *__restrict__ B, int ldb, bool bh, double2 *__restrict__ Cm, int ldc)
{
  const int i = blockIdx.y * 16 + threadIdx.y, j = blockIdx.x * 16 + threadIdx.x;
  if (i >= m || j >= p) return;
  double r = 0, im = 0;
  for (int l = 0; l < k; l++) {
    double2 a = ah ? A[(long)l * lda + i] : A[(long)i * lda + l];
    if (ah) a.y = -a.y;
    double2 b = bh ? B[(long)j * ldb + l] : B[(long)l * ldb + j];
    if (bh) b.y = -b.y;
    r += a.x * b.x - a.y * b.y;
    im += a.x * b.y + a.y * b.x;
  }
  Cm[(long)i * ldc + j] = make_double2(r, im);
}

int zgemm_dev(fbse_ctx *c, int m, int p, int k, const double2 *A, int lda, bool ah, const double2 *B, int ldb, bool bh,
              double2 *C, int ldc)
{
  dim3 b(16, 16), g((p + 15) / 16, (m + 15) / 16);
  k_zgemm<<<g, b, 0, c->stream>>>(m, p, k, A, lda, ah, B, ldb, bh, C, ldc);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

// ---------------------------------------------------------------------------
// Hermitian eigensolver: cyclic two-sided Jacobi with the round-robin pairing
// (n/2 disjoint rotations per round, n-1 rounds per sweep), one cooperative
// launch per sweep with two grid-wide barriers per round (rotation
// parameters, then the two-sided update of A and V).
// A (n x n, row-major, Hermitian) is diagonalised in place; V accumulates the
// unitary so that A_in = V diag(A_out) V^H.
// ---------------------------------------------------------------------------
struct Rot {
  double cs, sn, pr, pi;  // U = D J:  U_pp = cs, U_pq = sn, U_qp = -sn e^{-i phi}, U_qq = cs e^{-i phi}
  int p, q;
};

__device__ __forceinline__ void rr_pair(int r, int slot, int m, int &p, int &q)
{  // round-robin tournament: player m-1 fixed, the others rotate
  int a, b;
  if (slot == 0) { a = m - 1; b = r % (m - 1); }
  else { a = (r + slot) % (m - 1); b = (r - slot + (m - 1)) % (m - 1); }
  p = min(a, b);
  q = max(a, b);
}

__global__ void k_jacobi_sweep(double2 *__restrict__ A, double2 *__restrict__ V, int n, int m, Rot *__restrict__ rot,
                               double *__restrict__ off)
{
  cg::grid_group grid = cg::this_grid();
  const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long nth = (long)gridDim.x * blockDim.x;
  const int half = m / 2;
  const long nblk = (long)half * half;  // 2 x 2 blocks of A, one per (row pair, column pair)
  for (int r = 0; r < m - 1; r++) {
    // phase 1: rotation parameters for the n/2 pairs of this round
    for (long s = tid; s < half; s += nth) {
      int p, q;
      rr_pair(r, (int)s, m, p, q);
      Rot R{1.0, 0.0, 1.0, 0.0, p, q};
      if (q < n) {
        const double app = A[(long)p * n + p].x, aqq = A[(long)q * n + q].x;
        const double2 apq = A[(long)p * n + q];
        const double mag = hypot(apq.x, apq.y);
        if (mag > 1e-300 && mag > 1e-18 * sqrt(fabs(app * aqq))) {
          const double tau = (aqq - app) / (2.0 * mag);
          const double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
          R.cs = 1.0 / sqrt(1.0 + t * t);
          R.sn = t * R.cs;
          R.pr = apq.x / mag;  // e^{i phi}
          R.pi = apq.y / mag;
        }
      }
      rot[s] = R;
    }
    grid.sync();
    // phase 2: the pairs of a round cover every index once, so every element
    // of A lies in one 2 x 2 block (row pair a, column pair b) and every
    // element of V in one 1 x 2 block (row i, column pair b).  A block is
    // rotated from both sides at once, A_blk <- U_a^H A_blk U_b:
    //   rows:    new p = cs a_p - sn e^{i phi} a_q,   new q = sn a_p + cs e^{i phi} a_q
    //   columns: new p = cs a_p - sn e^{-i phi} a_q,  new q = sn a_p + cs e^{-i phi} a_q
    // and the rotated pair's off-diagonal element, zero in exact arithmetic,
    // is set to zero.  A dummy index (q = n for odd n) carries the identity.
    for (long w = tid; w < nblk + (long)n * half; w += nth) {
      if (w < nblk) {
        const Rot Ra = rot[w / half], Rb = rot[w % half];
        const bool qa = Ra.q < n, qb = Rb.q < n;
        double2 x[2][2];
        x[0][0] = A[(long)Ra.p * n + Rb.p];
        x[0][1] = qb ? A[(long)Ra.p * n + Rb.q] : make_double2(0, 0);
        x[1][0] = qa ? A[(long)Ra.q * n + Rb.p] : make_double2(0, 0);
        x[1][1] = qa && qb ? A[(long)Ra.q * n + Rb.q] : make_double2(0, 0);
        const double2 ea = make_double2(Ra.pr, Ra.pi);
#pragma unroll
        for (int c = 0; c < 2; c++) {
          const double2 ap = x[0][c], aq = x[1][c];
          const double2 eaq = make_double2(ea.x * aq.x - ea.y * aq.y, ea.x * aq.y + ea.y * aq.x);
          x[0][c] = make_double2(Ra.cs * ap.x - Ra.sn * eaq.x, Ra.cs * ap.y - Ra.sn * eaq.y);
          x[1][c] = make_double2(Ra.sn * ap.x + Ra.cs * eaq.x, Ra.sn * ap.y + Ra.cs * eaq.y);
        }
        const double2 eb = make_double2(Rb.pr, -Rb.pi);
#pragma unroll
        for (int rw = 0; rw < 2; rw++) {
          const double2 ap = x[rw][0], aq = x[rw][1];
          const double2 eaq = make_double2(eb.x * aq.x - eb.y * aq.y, eb.x * aq.y + eb.y * aq.x);
          x[rw][0] = make_double2(Rb.cs * ap.x - Rb.sn * eaq.x, Rb.cs * ap.y - Rb.sn * eaq.y);
          x[rw][1] = make_double2(Rb.sn * ap.x + Rb.cs * eaq.x, Rb.sn * ap.y + Rb.cs * eaq.y);
        }
        if (w / half == w % half && !(Ra.cs == 1.0 && Ra.sn == 0.0)) {
          x[0][1] = make_double2(0, 0);
          x[1][0] = make_double2(0, 0);
        }
        A[(long)Ra.p * n + Rb.p] = x[0][0];
        if (qb) A[(long)Ra.p * n + Rb.q] = x[0][1];
        if (qa) A[(long)Ra.q * n + Rb.p] = x[1][0];
        if (qa && qb) A[(long)Ra.q * n + Rb.q] = x[1][1];
      } else {
        const long w2 = w - nblk;
        const Rot R = rot[w2 / n];
        const int row = (int)(w2 % n);
        if (R.q >= n) continue;
        const double2 ap = V[(long)row * n + R.p], aq = V[(long)row * n + R.q];
        const double2 e = make_double2(R.pr, -R.pi);
        const double2 eaq = make_double2(e.x * aq.x - e.y * aq.y, e.x * aq.y + e.y * aq.x);
        V[(long)row * n + R.p] = make_double2(R.cs * ap.x - R.sn * eaq.x, R.cs * ap.y - R.sn * eaq.y);
        V[(long)row * n + R.q] = make_double2(R.sn * ap.x + R.cs * eaq.x, R.sn * ap.y + R.cs * eaq.y);
      }
    }
    grid.sync();
  }
  // off-diagonal Frobenius norm and diagonal norm: per-warp partials
  // (off[2 + 2 w], off[3 + 2 w]) summed by warp 0 of block 0 in a fixed order,
  // so that the sweep count is the same on every run
  double so = 0, sd = 0;
  for (long e = tid; e < (long)n * n; e += nth) {
    const double2 a = A[e];
    const double v = a.x * a.x + a.y * a.y;
    if (e / n == e % n) sd += v;
    else so += v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    so += __shfl_xor_sync(0xffffffffu, so, o);
    sd += __shfl_xor_sync(0xffffffffu, sd, o);
  }
  const long nw = nth / 32, w = tid / 32;
  if ((threadIdx.x & 31) == 0) {
    off[2 + 2 * w] = so;
    off[3 + 2 * w] = sd;
  }
  grid.sync();
  if (blockIdx.x == 0 && threadIdx.x < 32) {
    double to = 0, td = 0;
    for (long i = threadIdx.x; i < nw; i += 32) {
      to += off[2 + 2 * i];
      td += off[3 + 2 * i];
    }
    for (int o = 16; o > 0; o >>= 1) {
      to += __shfl_xor_sync(0xffffffffu, to, o);
      td += __shfl_xor_sync(0xffffffffu, td, o);
    }
    if (threadIdx.x == 0) {
      off[0] = to;
      off[1] = td;
    }
  }
}

__global__ void k_identity(double2 *V, int n)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)n * n; e += (long)gridDim.x * blockDim.x)
    V[e] = make_double2(e / n == e % n ? 1.0 : 0.0, 0.0);
}

// eigen-decomposition of the Hermitian n x n matrix A (device, overwritten);
// V (device, n x n) receives the eigenvectors as columns, w (host) the
// eigenvalues in the order of V's columns
int jacobi_eig_dev(fbse_ctx *c, double2 *A, double2 *V, int n, std::vector<double> &w)
{
  const int m = n + (n & 1);
  int dev = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_jacobi_sweep, 256, 0);
  const long work = (long)(m / 2) * (m / 2) + (long)n * (m / 2);
  long want = (work + 255) / 256;
  int blocks = (int)std::min<long>(std::max<long>(1, want), (long)nsm * std::max(1, per_sm));
  // rotation table, the two norms and their per-warp partials, kept in the
  // context between calls
  const size_t rot_bytes = (sizeof(Rot) * (m / 2 + 1) + 15) / 16 * 16;
  void *scratch = nullptr;
  int rc = cached(c, kSlotJacobi, rot_bytes + (2 + 2 * (size_t)blocks * 8) * sizeof(double), &scratch);
  if (rc) return rc;
  Rot *rot = static_cast<Rot *>(scratch);
  double *off = reinterpret_cast<double *>(static_cast<char *>(scratch) + rot_bytes);
  FBSE_COUNT(1); k_identity<<<256, 256, 0, c->stream>>>(V, n);
  double h[2] = {0, 0};
  bool conv = (n < 2);
  for (int sweep = 0; sweep < 60 && !conv; sweep++) {
    void *args[] = {&A, &V, &n, (void *)&m, &rot, &off};
    int mm = m;
    args[3] = &mm;
    FBSE_COUNT(1); if (cudaLaunchCooperativeKernel((void *)k_jacobi_sweep, blocks, 256, args, 0, c->stream) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, std::string("jacobi launch: ") + cudaGetErrorString(cudaGetLastError()));
      break;
    }
    if (cudaMemcpyAsync(h, off, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "jacobi sweep");
      break;
    }
    if (!(h[0] == h[0])) { rc = set_err(c, FBSE_ERR_NAN, "jacobi: NaN in matrix"); break; }
    if (h[0] <= 1e-30 * h[1] || h[0] < 1e-300) conv = true;
  }
  if (!rc && !conv) rc = set_err(c, FBSE_ERR_NOCONV, "jacobi eigensolver did not converge in 60 sweeps");
  if (!rc) {
    // only the diagonal is needed on the host: one strided copy (pitch n + 1)
    std::vector<double2> d((size_t)n);
    if (cudaMemcpy2DAsync(d.data(), sizeof(double2), A, (size_t)(n + 1) * sizeof(double2), sizeof(double2), (size_t)n,
                          cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      rc = set_err(c, FBSE_ERR_CUDA, "jacobi download");
    w.resize(n);
    for (int i = 0; i < n && !rc; i++) w[i] = d[i].x;
  }
  return rc;
}

// ---------------------------------------------------------------------------
// rotation with residual epilogue
//   P[i][l] = sum_j Psi[j][l] C[j][i],  Q[i][l] = sum_j HPsi[j][l] C[j][i]
//   out[i][l] = P;  part[blk][i] += |Q - E_i P|^2, |P|^2, Re(conj(P) Q)
// tile: 128 grid elements x 32 output states per CTA, 256 threads; the state
// tiles of one grid tile are consecutive blocks (they share the grid tile's
// Psi / H Psi through L2, so the states stream from DRAM once), and the next
// j block is loaded into registers while the current one is multiplied
// ---------------------------------------------------------------------------
// PART 2: rotate Psi and H Psi together; PART 0: Psi only (writes out);
// PART 1: H Psi only, reading the rotated Psi back from out for the residual
// sums (two launches of half the accumulators each: two CTAs per SM instead
// of one for the FP32 path).
template <typename T, bool CPLX, int PART>
__global__ void __launch_bounds__(256, PART == 2 ? 1 : 2) k_rotate(const double *__restrict__ Psi, const double *__restrict__ HPsi, int n,
                                                long L, const double2 *__restrict__ Cm, int k,
                                                const double *__restrict__ E, double *__restrict__ out,
                                                double *__restrict__ part)
{
  constexpr int TL = 128, TS = 32, TJ = 8;
  constexpr int NU = TJ * TL / 256;  // Psi / H Psi tile values per thread
  static_assert(TJ * TS == 256, "one coefficient per thread and j block");
  const int nsb = (k + TS - 1) / TS;
  const long bx = blockIdx.x / nsb;
  const long l0 = bx * TL;
  const int s0 = (int)(blockIdx.x % nsb) * TS;
  // complex values as C<T>: one float2 / double2 access per value
  using Elt = typename std::conditional<CPLX, C<T>, T>::type;
  using Raw = typename std::conditional<CPLX, double2, double>::type;
  __shared__ Elt Ps[TJ][TL];
  __shared__ Elt Hs[TJ][TL];
  __shared__ C<T> Cs[TJ][TS];
  __shared__ double red[TS][3];
  const int tl = threadIdx.x % 32;  // 4 grid elements per thread: tl + 32 q
  const int ts = threadIdx.x / 32;  // 4 output states per thread: ts + 8 r
  T pr[4][4], pim[4][4], qr[4][4], qim[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) { pr[a][b] = pim[a][b] = qr[a][b] = qim[a][b] = 0; }
  if (threadIdx.x < TS * 3) red[threadIdx.x / 3][threadIdx.x % 3] = 0;
  Raw rp[NU], rh[NU];
  double2 rc;
  auto fetch = [&](int jb) {
#pragma unroll
    for (int u = 0; u < NU; u++) {
      const int t = threadIdx.x + 256 * u;
      const int j = jb + t / TL;
      const long l = l0 + t % TL;
      const bool ok = (j < n) && (l < L);
      if constexpr (CPLX) {
        if constexpr (PART != 1) rp[u] = ok ? reinterpret_cast<const double2 *>(Psi)[(long)j * L + l] : make_double2(0, 0);
        if constexpr (PART != 0) rh[u] = ok ? reinterpret_cast<const double2 *>(HPsi)[(long)j * L + l] : make_double2(0, 0);
      } else {
        if constexpr (PART != 1) rp[u] = ok ? Psi[(long)j * L + l] : 0.0;
        if constexpr (PART != 0) rh[u] = ok ? HPsi[(long)j * L + l] : 0.0;
      }
    }
    const int j = jb + threadIdx.x / TS, sc = s0 + threadIdx.x % TS;
    rc = (j < n && sc < k) ? Cm[(long)j * k + sc] : make_double2(0, 0);
  };
  fetch(0);
  for (int jb = 0; jb < n; jb += TJ) {
#pragma unroll
    for (int u = 0; u < NU; u++) {
      const int t = threadIdx.x + 256 * u;
      const int jj = t / TL, ll = t % TL;
      if constexpr (CPLX) {
        if constexpr (PART != 1) Ps[jj][ll] = mk<T>((T)rp[u].x, (T)rp[u].y);
        if constexpr (PART != 0) Hs[jj][ll] = mk<T>((T)rh[u].x, (T)rh[u].y);
      } else {
        if constexpr (PART != 1) Ps[jj][ll] = (T)rp[u];
        if constexpr (PART != 0) Hs[jj][ll] = (T)rh[u];
      }
    }
    Cs[threadIdx.x / TS][threadIdx.x % TS] = mk<T>((T)rc.x, (T)rc.y);
    __syncthreads();
    if (jb + TJ < n) fetch(jb + TJ);
#pragma unroll
    for (int jj = 0; jj < TJ; jj++) {
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const int ll = tl + 32 * a;
        T xr = T(0), xi = T(0), yr = T(0), yi = T(0);
        if constexpr (CPLX) {
          if constexpr (PART != 1) { const C<T> x = Ps[jj][ll]; xr = x.x; xi = x.y; }
          if constexpr (PART != 0) { const C<T> y = Hs[jj][ll]; yr = y.x; yi = y.y; }
        } else {
          if constexpr (PART != 1) xr = Ps[jj][ll];
          if constexpr (PART != 0) yr = Hs[jj][ll];
        }
#pragma unroll
        for (int b = 0; b < 4; b++) {
          const int ss = ts + 8 * b;
          const C<T> cv = Cs[jj][ss];
          const T cr = cv.x, ci = cv.y;
          if constexpr (PART != 1) {
            pr[a][b] += xr * cr - xi * ci;
            pim[a][b] += xr * ci + xi * cr;
          }
          if constexpr (PART != 0) {
            qr[a][b] += yr * cr - yi * ci;
            qim[a][b] += yr * ci + yi * cr;
          }
        }
      }
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int b = 0; b < 4; b++) {
    const int s = s0 + ts + 8 * b;
    double rr = 0, pp = 0, pq = 0;
    if (s < k) {
      const double e = E[s];
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const long l = l0 + tl + 32 * a;
        if (l < L) {
          double Pr, Pi;
          if constexpr (PART != 1) {
            Pr = pr[a][b];
            Pi = CPLX ? (double)pim[a][b] : 0.0;
            if (CPLX) {
              out[((long)s * L + l) * 2] = Pr;
              out[((long)s * L + l) * 2 + 1] = Pi;
            } else {
              out[(long)s * L + l] = Pr;
            }
            if constexpr (PART == 0) continue;
          } else {
            Pr = CPLX ? out[((long)s * L + l) * 2] : out[(long)s * L + l];
            Pi = CPLX ? out[((long)s * L + l) * 2 + 1] : 0.0;
          }
          const double Qr = qr[a][b], Qi = CPLX ? (double)qim[a][b] : 0.0;
          const double dr = Qr - e * Pr, di = Qi - e * Pi;
          rr += dr * dr + di * di;
          pp += Pr * Pr + Pi * Pi;
          pq += Pr * Qr + Pi * Qi;
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      rr += __shfl_xor_sync(0xffffffffu, rr, o);
      pp += __shfl_xor_sync(0xffffffffu, pp, o);
      pq += __shfl_xor_sync(0xffffffffu, pq, o);
    }
    if (tl == 0) {
      red[ts + 8 * b][0] = rr;
      red[ts + 8 * b][1] = pp;
      red[ts + 8 * b][2] = pq;
    }
  }
  __syncthreads();
  if (PART != 0 && threadIdx.x < TS) {
    const int s = s0 + threadIdx.x;
    if (s < k) {
      double *P = part + (bx * k + s) * 3;
      P[0] = red[threadIdx.x][0];
      P[1] = red[threadIdx.x][1];
      P[2] = red[threadIdx.x][2];
    }
  }
}

__global__ void k_sum_rot(const double *__restrict__ part, int nblk, int k, double *__restrict__ out)
{
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < k; s += gridDim.x * blockDim.x) {
    double a = 0, b = 0, d = 0;
    for (int q = 0; q < nblk; q++) {
      a += part[((long)q * k + s) * 3];
      b += part[((long)q * k + s) * 3 + 1];
      d += part[((long)q * k + s) * 3 + 2];
    }
    out[3 * s] = a;
    out[3 * s + 1] = b;
    out[3 * s + 2] = d;
  }
}

__global__ void k_scale_copy(const double *__restrict__ src, double *__restrict__ dst, long stlen, long k,
                             const double *__restrict__ f)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < k * stlen; i += (long)gridDim.x * blockDim.x)
    dst[i] = src[i] * f[i / stlen];
}

// X[j][s] = V[j][keep[s]] / sqrt(l[keep[s]])
__global__ void k_build_x(const double2 *__restrict__ V, int n, const int *__restrict__ keep,
                          const double *__restrict__ lam, int k, double2 *__restrict__ X)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)n * k; e += (long)gridDim.x * blockDim.x) {
    const int j = (int)(e / k), s = (int)(e % k);
    const double f = 1.0 / sqrt(lam[s]);
    const double2 v = V[(long)j * n + keep[s]];
    X[e] = make_double2(v.x * f, v.y * f);
  }
}

__global__ void k_hermitize(double2 *A, int n)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)n * n; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e % n);
    if (i > j) continue;
    const double2 a = A[(long)i * n + j], b = A[(long)j * n + i];
    const double2 h = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
    A[(long)i * n + j] = h;
    A[(long)j * n + i] = make_double2(h.x, -h.y);
  }
}

// permute the columns of U (k x k): U2[:, s] = U[:, perm[s]]
__global__ void k_permute_cols(const double2 *__restrict__ U, const int *__restrict__ perm, int k,
                               double2 *__restrict__ U2)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)k * k; e += (long)gridDim.x * blockDim.x) {
    const int i = (int)(e / k), s = (int)(e % k);
    U2[e] = U[(long)i * k + perm[s]];
  }
}

// q[s] = sum_i conj(C[i][s]) T[i][s] (real part): the quadratic forms
// C_s^H A C_s from T = A C, for the k columns of the n x k matrix C
__global__ void k_quad_diag(const double2 *__restrict__ Cm, const double2 *__restrict__ Tm, int n, int k,
                            double *__restrict__ q)
{
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < k; s += gridDim.x * blockDim.x) {
    double v = 0;
    for (int i = 0; i < n; i++) {
      const double2 a = Cm[(long)i * k + s], b = Tm[(long)i * k + s];
      v += a.x * b.x + a.y * b.y;
    }
    q[s] = v;
  }
}

template <typename T>
static int gram_t(fbse_ctx *c, const double *A, const double *B, int n, long L, double2 *out, double scale,
                  double2 *part, int nchunk, long kchunk)
{
  const int nt = (n + 63) / 64;
  dim3 g(nt * (nt + 1) / 2, 1, nchunk);
  // resident CTAs per SM: one (no register cap) or two (a cap of 128
  // registers, which spills the FP32 path's float-float accumulators a
  // little); the same sums either way, so the autotuner picks by time
  auto launch = [&](long v) -> int {
    if (c->is_complex) {
      if (v == 2) k_gram<T, true, 2><<<g, 256, 0, c->stream>>>(A, B, n, L, kchunk, part);
      else k_gram<T, true, 1><<<g, 256, 0, c->stream>>>(A, B, n, L, kchunk, part);
    } else {
      if (v == 2) k_gram<T, false, 2><<<g, 256, 0, c->stream>>>(A, B, n, L, kchunk, part);
      else k_gram<T, false, 1><<<g, 256, 0, c->stream>>>(A, B, n, L, kchunk, part);
    }
    return launch_status(c);
  };
  long minb = 1;
  const std::string prob = std::string(sizeof(T) == 4 ? "fp32" : "fp64") + (c->is_complex ? " complex" : " real") +
                           " n=" + std::to_string(n) + " L=" + std::to_string(L);
  int rc = autotune(c, "gram CTAs per SM", prob, {1, 2}, launch, &minb);
  if (rc) return rc;
  if ((rc = launch(minb))) return rc;
  FBSE_COUNT(1);
  k_sum_partials<<<256, 256, 0, c->stream>>>(part, nchunk, (long)n * n, scale, out);
  FBSE_CHECK_LAUNCH(c);
  return FBSE_OK;
}

// default overlap cut of the mixed path, relative to the largest eigenvalue.
// Measured on the 3 nm CdSe spinor dot (256 filtered states): a cut of 1e-10
// keeps 250 pairs and matches 148 levels of the FP64 pipeline against 228 and
// 142 at 1e-6, but the extra directions are noise of the FP32 recursion and
// they leave the converged vectors less accurate (on the CsPbI3 cube the
// smallest singular value of the mixed / FP64 cluster overlaps drops from
// 1 - 4e-8 to 1 - 9e-6), so the default keeps 1e-6
constexpr double kMixedRitzCut = 1e-6;

template <typename T>
static int ortho_diag_sigma_t(fbse_ctx *c, double *psitot, long n_, long *n_kept, double *eval, double *sigma)
{
  const int n = (int)n_;
  const long len = (long)c->nspin * c->ngrid;     // points per state
  const long stlen = (long)(c->is_complex + 1) * len;
  const long L = len;                              // vector length in (complex or real) elements
  int rc = FBSE_OK;
  // scratch: HPsi (n states FP64), rotated states (n states FP64), working states
  double *hpsi = nullptr, *rot = nullptr;
  void *work = nullptr;
  double2 *G = nullptr, *M = nullptr, *V = nullptr, *X = nullptr, *Hp = nullptr, *Tm = nullptr, *U = nullptr,
          *Cm = nullptr, *part = nullptr, *G0 = nullptr;
  double *lam = nullptr, *Ed = nullptr, *rpart = nullptr, *rsum = nullptr, *fac = nullptr, *quad = nullptr;
  constexpr bool kMixed = sizeof(T) == 4;
  int *keepd = nullptr, *permd = nullptr;
  const long chunk_states = 16;
  const long nw_chunk = c->is_complex ? chunk_states : chunk_states / 2;
  const int nchunk = (int)std::min<long>(std::max<long>(1, L / 4096), 1024);
  const long kchunk = (L + nchunk - 1) / nchunk;
  const int nrb = (int)((L + 127) / 128);
  auto alloc = [&](void **p, size_t b) -> bool {
    if (cudaMalloc(p, b) != cudaSuccess) { cudaGetLastError(); rc = set_err(c, FBSE_ERR_OOM, "ortho/diag scratch"); return false; }
    return true;
  };
  do {
    {
      void *a = nullptr, *b = nullptr;
      if (cached(c, kSlotHpsi, (size_t)n * stlen * sizeof(double), &a) ||
          cached(c, kSlotRot, (size_t)n * stlen * sizeof(double), &b)) { rc = FBSE_ERR_OOM; break; }
      hpsi = (double *)a;
      rot = (double *)b;
    }
    // the mixed path applies H in FP32 here unless told otherwise (FP64 H psi
    // measured no better on the 3 nm dot: the FP32 recursion's noise in the
    // filtered states, not the operator, limits the projected problem)
    const bool h64 = kMixed && c->tune.ritz_hpsi == 2;
    if (!alloc(&work, (size_t)2 * nw_chunk * len * (h64 ? sizeof(double2) : sizeof(C<T>)))) break;
    const size_t nn = (size_t)n * n;
    if (!alloc((void **)&G, nn * sizeof(double2)) || !alloc((void **)&M, nn * sizeof(double2)) ||
        !alloc((void **)&V, nn * sizeof(double2)) || !alloc((void **)&X, nn * sizeof(double2)) ||
        !alloc((void **)&Hp, nn * sizeof(double2)) || !alloc((void **)&Tm, nn * sizeof(double2)) ||
        !alloc((void **)&U, nn * sizeof(double2)) || !alloc((void **)&Cm, nn * sizeof(double2)) ||
        !alloc((void **)&part, (size_t)nchunk * nn * sizeof(double2)) || !alloc((void **)&lam, n * sizeof(double)) ||
        !alloc((void **)&Ed, n * sizeof(double)) || !alloc((void **)&rpart, (size_t)nrb * n * 3 * sizeof(double)) ||
        !alloc((void **)&rsum, (size_t)n * 3 * sizeof(double)) || !alloc((void **)&fac, n * sizeof(double)) ||
        !alloc((void **)&keepd, n * sizeof(int)) || !alloc((void **)&permd, n * sizeof(int)) ||
        !alloc((void **)&G0, nn * sizeof(double2)) || !alloc((void **)&quad, 2 * (size_t)n * sizeof(double)))
      break;
    // 1. HPsi in chunks of working states
    for (long s0 = 0; s0 < n && !rc; s0 += chunk_states) {
      const long ns = std::min<long>(chunk_states, n - s0);
      const long nw = c->is_complex ? ns : (ns + 1) / 2;
      if (h64) {
        double2 *w0 = reinterpret_cast<double2 *>(work), *w1 = w0 + nw_chunk * len;
        if ((rc = pack<double>(c, psitot + s0 * stlen, w0, ns))) break;
        if ((rc = hpsi_apply<double>(c, w0, w1, nw, 1.0, 0.0))) break;
        if ((rc = unpack<double>(c, w1, hpsi + s0 * stlen, ns))) break;
      } else {
        C<T> *w0 = reinterpret_cast<C<T> *>(work), *w1 = w0 + nw_chunk * len;
        if ((rc = pack<T>(c, psitot + s0 * stlen, w0, ns))) break;
        if ((rc = hpsi_apply<T>(c, w0, w1, nw, 1.0, 0.0))) break;
        if ((rc = unpack<T>(c, w1, hpsi + s0 * stlen, ns))) break;
      }
    }
    if (rc) break;
    // 2. Gram and projected H (dv-weighted)
    if ((rc = gram_t<T>(c, psitot, psitot, n, L, G, c->dv, part, nchunk, kchunk))) break;
    if ((rc = gram_t<T>(c, psitot, hpsi, n, L, M, c->dv, part, nchunk, kchunk))) break;
    FBSE_COUNT(2); k_hermitize<<<64, 256, 0, c->stream>>>(G, n);
    k_hermitize<<<64, 256, 0, c->stream>>>(M, n);
    if (cudaMemcpyAsync(G0, G, nn * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "overlap copy");
      break;
    }
    // 3. overlap eigen-decomposition
    std::vector<double> w;
    if ((rc = jacobi_eig_dev(c, G, V, n, w))) break;
    // 4. rank cutoff (ortho.c:68-75 keeps s_i/s_0 >= 1e-10); the overlap
    //    resolves l_i / l_max to the precision of its products and of the
    //    states (fbse_tuning.ritz_cut overrides the default)
    double lmax = 0;
    for (double v : w) lmax = std::max(lmax, v);
    const double cut = lmax * (c->tune.ritz_cut > 0 ? c->tune.ritz_cut : (kMixed ? kMixedRitzCut : 1e-12));
    std::vector<int> keep;
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
    for (int i : order)
      if (w[i] > cut && w[i] >= lmax * 1e-20) keep.push_back(i);
    const int k = (int)keep.size();
    *n_kept = k;
    if (k == 0) { rc = set_err(c, FBSE_ERR_NAN, "orthogonalisation kept no states"); break; }
    std::vector<double> lk(k);
    for (int s = 0; s < k; s++) lk[s] = w[keep[s]];
    if (h2d(c->stream, keepd, keep.data(), k * sizeof(int)) != cudaSuccess ||
        h2d(c->stream, lam, lk.data(), k * sizeof(double)) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "orthogonalisation: basis upload");
      break;
    }
    FBSE_COUNT(1); k_build_x<<<64, 256, 0, c->stream>>>(V, n, keepd, lam, k, X);
    // 5. H' = X^H M X  (k x k), Hermitian eigen-decomposition
    if ((rc = zgemm_dev(c, n, k, n, M, n, false, X, k, false, Tm, k))) break;   // Tm = M X   (n x k)
    if ((rc = zgemm_dev(c, k, k, n, X, k, true, Tm, k, false, Hp, k))) break;  // Hp = X^H Tm (k x k)
    FBSE_COUNT(1); k_hermitize<<<64, 256, 0, c->stream>>>(Hp, k);
    std::vector<double> e;
    if ((rc = jacobi_eig_dev(c, Hp, U, k, e))) break;
    std::vector<int> perm(k);
    std::iota(perm.begin(), perm.end(), 0);
    std::sort(perm.begin(), perm.end(), [&](int a, int b) { return e[a] < e[b]; });
    std::vector<double> es(k);
    for (int s = 0; s < k; s++) es[s] = e[perm[s]];
    if (h2d(c->stream, permd, perm.data(), k * sizeof(int)) != cudaSuccess ||
        h2d(c->stream, Ed, es.data(), k * sizeof(double)) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "diagonalisation: eigenvalue upload");
      break;
    }
    FBSE_COUNT(1); k_permute_cols<<<64, 256, 0, c->stream>>>(U, permd, k, Tm);
    // 6. C = X U  (n x k); rotate Psi and HPsi with the residual epilogue
    if ((rc = zgemm_dev(c, n, k, k, X, k, false, Tm, k, false, Cm, k))) break;
    if constexpr (kMixed) {
      // the Rayleigh quotients of the exact combinations Psi C from the FP64
      // small matrices: (C^H M C)_ss / (C^H G C)_ss (X and Hp are free now)
      if ((rc = zgemm_dev(c, n, k, n, M, n, false, Cm, k, false, X, k))) break;
      if ((rc = zgemm_dev(c, n, k, n, G0, n, false, Cm, k, false, Hp, k))) break;
      FBSE_COUNT(2);
      k_quad_diag<<<(k + 127) / 128, 128, 0, c->stream>>>(Cm, X, n, k, quad);
      k_quad_diag<<<(k + 127) / 128, 128, 0, c->stream>>>(Cm, Hp, n, k, quad + n);
    }
    const dim3 gr((unsigned)(nrb * ((k + 31) / 32)));
    if constexpr (sizeof(T) == 4) {  // FP32: two half-register launches (Psi, then H Psi + residuals)
      if (c->is_complex) {
        k_rotate<T, true, 0><<<gr, 256, 0, c->stream>>>(psitot, hpsi, n, L, Cm, k, Ed, rot, rpart);
        k_rotate<T, true, 1><<<gr, 256, 0, c->stream>>>(psitot, hpsi, n, L, Cm, k, Ed, rot, rpart);
      } else {
        k_rotate<T, false, 0><<<gr, 256, 0, c->stream>>>(psitot, hpsi, n, L, Cm, k, Ed, rot, rpart);
        k_rotate<T, false, 1><<<gr, 256, 0, c->stream>>>(psitot, hpsi, n, L, Cm, k, Ed, rot, rpart);
      }
      FBSE_COUNT(1);
    } else {
      if (c->is_complex) k_rotate<T, true, 2><<<gr, 256, 0, c->stream>>>(psitot, hpsi, n, L, Cm, k, Ed, rot, rpart);
      else k_rotate<T, false, 2><<<gr, 256, 0, c->stream>>>(psitot, hpsi, n, L, Cm, k, Ed, rot, rpart);
    }
    FBSE_LAUNCH_OR_BREAK(c, rc);
    FBSE_COUNT(1); k_sum_rot<<<(k + 127) / 128, 128, 0, c->stream>>>(rpart, nrb, k, rsum);
    std::vector<double> hs(3 * k), hq(2 * (size_t)n);
    if (cudaMemcpyAsync(hs.data(), rsum, 3 * k * sizeof(double), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        (kMixed && cudaMemcpyAsync(hq.data(), quad, 2 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                                   c->stream) != cudaSuccess) ||
        cudaStreamSynchronize(c->stream) != cudaSuccess) { rc = set_err(c, FBSE_ERR_CUDA, "rotation"); break; }
    // 7. normalise; report the Rayleigh quotient rho = <psi|H psi>/<psi|psi> of
    //    the returned state and sigma = ||(H - rho) psi|| / ||psi||.  rho differs
    //    from the Ritz value E by the basis' departure from orthonormality
    //    (X^H G X = I up to eps * cond(G)); for the reference's SVD basis the
    //    two agree, so rho is the closer match to its eig_vals and is what
    //    calc_sigma_E reports for the state.  With r = ||(H - E) psi||^2:
    //    ||(H - rho) psi||^2 = r - (rho - E)^2 ||psi||^2.  The mixed path
    //    takes rho from the FP64 small matrices (the FP32 rotation loses
    //    digits where C is large, on near-dependent filtered states) and
    //    sigma from the rotated states.
    std::vector<double> f(k);
    for (int s = 0; s < k; s++) {
      const double pp = hs[3 * s + 1];
      const double nrm = pp * c->dv;
      if (!(nrm > 0)) { rc = set_err(c, FBSE_ERR_NAN, "Norm is 0/NAN after diagonalisation"); break; }
      f[s] = 1.0 / std::sqrt(nrm);
      const double rho = kMixed ? hq[s] / hq[n + s] : hs[3 * s + 2] / pp;
      const double d = rho - es[s];
      eval[s] = rho;
      sigma[s] = std::sqrt(std::fabs(hs[3 * s] / pp - d * d));
    }
    if (rc) break;
    if (h2d(c->stream, fac, f.data(), k * sizeof(double)) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "normalisation: factor upload");
      break;
    }
    k_scale_copy<<<4096, 256, 0, c->stream>>>(rot, psitot, stlen, k, fac);
    FBSE_LAUNCH_OR_BREAK(c, rc);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "ortho/diag/sigma");
  } while (0);
  cudaStreamSynchronize(c->stream);
  void *bufs[] = {work, G, M, V, X, Hp, Tm, U, Cm, part, lam, Ed, rpart, rsum, fac, keepd, permd, G0, quad};
  for (void *b : bufs)
    if (b) cudaFree(b);
  return rc;
}

// ---------------------------------------------------------------------------
// general FP64 products over a slab of points [off, off + len) of each state:
//   gram:   out[i][j] = dv sum_l conj(A_i[l]) B_j[l]          (na x nb)
//   rotate: out_j[l] = sum_i C[i][j] A_i[l]                   (k states)
// A, B, out: psitot rows (stlen doubles; complex states are (re, im) pairs,
// l counts complex values then).  64 x 64 output tile per CTA for the Gram,
// FP64 split-K partials summed in order.
// ---------------------------------------------------------------------------
template <bool CPLX>
__global__ void __launch_bounds__(256) k_gram_slab(const double *__restrict__ A, long na, const double *__restrict__ B,
                                                   long nb, long stride, long off, long len, long kchunk,
                                                   double2 *__restrict__ part)
{
  constexpr int TM = 64, TK = 16;
  __shared__ double2 As[TK][TM + 1], Bs[TK][TM + 1];
  const long i0 = (long)blockIdx.x * TM, j0 = (long)blockIdx.y * TM;
  const long k0 = off + blockIdx.z * kchunk, k1 = min(off + len, k0 + kchunk);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double ar_[4][4] = {}, ai_[4][4] = {};
  for (long kb = k0; kb < k1; kb += TK) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int r = ty + 16 * q;
      const long k = kb + tx;
      double2 va = make_double2(0, 0), vb = make_double2(0, 0);
      if (i0 + r < na && k < k1) va = CPLX ? reinterpret_cast<const double2 *>(A + (i0 + r) * stride)[k]
                                           : make_double2(A[(i0 + r) * stride + k], 0.0);
      if (j0 + r < nb && k < k1) vb = CPLX ? reinterpret_cast<const double2 *>(B + (j0 + r) * stride)[k]
                                           : make_double2(B[(j0 + r) * stride + k], 0.0);
      As[tx][r] = va;
      Bs[tx][r] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++)
#pragma unroll
      for (int a = 0; a < 4; a++) {
        const double2 u = As[kk][ty + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; b++) {
          const double2 v = Bs[kk][tx + 16 * b];
          ar_[a][b] += u.x * v.x + u.y * v.y;
          ai_[a][b] += u.x * v.y - u.y * v.x;
        }
      }
    __syncthreads();
  }
  double2 *P = part + (long)blockIdx.z * na * nb;
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) {
      const long i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      if (i < na && j < nb) P[i * nb + j] = make_double2(ar_[a][b], ai_[a][b]);
    }
}

template <bool CPLX>
__global__ void k_rotate_slab(const double *__restrict__ A, long na, const double2 *__restrict__ Cm, long k,
                              long stride, long off, long len, double *__restrict__ out)
{
  const long total = k * len;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long j = e / len, l = off + e % len;
    double re = 0, im = 0;
    for (long i = 0; i < na; i++) {
      const double2 cc = Cm[i * k + j];
      if (CPLX) {
        const double2 a = reinterpret_cast<const double2 *>(A + i * stride)[l];
        re += cc.x * a.x - cc.y * a.y;
        im += cc.x * a.y + cc.y * a.x;
      } else {
        re += cc.x * A[i * stride + l];
      }
    }
    if (CPLX) reinterpret_cast<double2 *>(out + j * stride)[l] = make_double2(re, im);
    else out[j * stride + l] = re;
  }
}

int gram_slab(fbse_ctx *c, const double *A, long na, const double *B, long nb, long off, long len, double *out_host)
{
  const long L = (long)c->nspin * c->ngrid;
  const long stride = (long)(c->is_complex + 1) * L;
  if (na < 1 || nb < 1 || off < 0 || len < 1 || off + len > L || na > 65535 * 64L || nb > 65535 * 64L)
    return set_err(c, FBSE_ERR_ARG, "fbse_gram: sizes");
  const int nchunk = (int)std::min<long>(std::max<long>(1, len / 8192), 256);
  const long kchunk = (len + nchunk - 1) / nchunk;
  double2 *part = nullptr, *sum = nullptr;
  if (cudaMalloc(&part, (size_t)nchunk * na * nb * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&sum, (size_t)na * nb * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    if (part) cudaFree(part);
    return set_err(c, FBSE_ERR_OOM, "fbse_gram: scratch");
  }
  int rc = FBSE_OK;
  do {
    dim3 g((unsigned)((na + 63) / 64), (unsigned)((nb + 63) / 64), (unsigned)nchunk);
    if (c->is_complex) k_gram_slab<true><<<g, 256, 0, c->stream>>>(A, na, B, nb, stride, off, len, kchunk, part);
    else k_gram_slab<false><<<g, 256, 0, c->stream>>>(A, na, B, nb, stride, off, len, kchunk, part);
    FBSE_LAUNCH_OR_BREAK(c, rc);
    k_sum_partials<<<256, 256, 0, c->stream>>>(part, nchunk, na * nb, c->dv, sum);
    FBSE_LAUNCH_OR_BREAK(c, rc);
    if (d2h(c->stream, out_host, sum, (size_t)na * nb * sizeof(double2)) != cudaSuccess)
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_gram: download");
  } while (0);
  cudaStreamSynchronize(c->stream);
  cudaFree(part);
  cudaFree(sum);
  return rc;
}

int rotate_slab(fbse_ctx *c, const double *A, long na, const double *C_host, long k, long off, long len, double *out)
{
  const long L = (long)c->nspin * c->ngrid;
  const long stride = (long)(c->is_complex + 1) * L;
  if (na < 1 || k < 1 || off < 0 || len < 1 || off + len > L) return set_err(c, FBSE_ERR_ARG, "fbse_rotate: sizes");
  double2 *Cd = nullptr;
  if (cudaMalloc(&Cd, (size_t)na * k * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_OOM, "fbse_rotate: coefficients");
  }
  int rc = FBSE_OK;
  do {
    if (h2d(c->stream, Cd, C_host, (size_t)na * k * sizeof(double2)) != cudaSuccess) {
      rc = set_err(c, FBSE_ERR_CUDA, "fbse_rotate: upload");
      break;
    }
    const long total = k * len;
    const unsigned g = (unsigned)std::min<long>((total + 255) / 256, 152L * 64);
    if (c->is_complex) k_rotate_slab<true><<<g, 256, 0, c->stream>>>(A, na, Cd, k, stride, off, len, out);
    else k_rotate_slab<false><<<g, 256, 0, c->stream>>>(A, na, Cd, k, stride, off, len, out);
    FBSE_LAUNCH_OR_BREAK(c, rc);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = set_err(c, FBSE_ERR_CUDA, "fbse_rotate");
  } while (0);
  cudaFree(Cd);
  return rc;
}

int ortho_diag_sigma(fbse_ctx *c, double *psitot, long n, long *n_kept, double *eval, double *sigma)
{
  if (n > 8192) return set_err(c, FBSE_ERR_UNSUPPORTED, "more than 8192 states in one subspace");
  return c->precision == FBSE_MIXED ? ortho_diag_sigma_t<float>(c, psitot, n, n_kept, eval, sigma)
                                    : ortho_diag_sigma_t<double>(c, psitot, n, n_kept, eval, sigma);
}

}  // namespace fbse
