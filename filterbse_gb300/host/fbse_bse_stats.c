/* Exciton spin and angular-momentum statistics of the BSE stage
 * (calc_xton_spin_mtrx and calc_xton_ang_mom_mtrx, bse_cplx/angular.c:692-1043),
 * on the host from the quasiparticle matrices of fbse_bse_qp_ang_mom and the
 * exciton coefficients.  The reference's double sums over (b, j) inside the
 * sums over (a, i) are reordered through partial sums T(a, j) = sum_b
 * conj(c_bj) M(a, b), so an exciton costs O(n_e^2 n_h + n_e n_h^2) instead of
 * O(n_e^2 n_h^2). */
#include <complex.h>
#include <stdlib.h>

#include "fbse_dropin.h"

typedef double complex zc;

/* C[ibs][n] (row-major n_xton x n_xton, ibs = a * n_h + i); pair matrices as
 * fbse_bse_qp_ang_mom returns them.  Outputs per exciton n (complex,
 * interleaved): spin[n][3], spintot[n], orbit[n][3], orbittot[n], lstot[n]. */
int fbse_xton_ang_stats(long nh, long ne, const double *coeff, const double *s_mom, const double *l_mom,
                        const double *l2_mom, const double *ldots, double *spin, double *spintot, double *orbit,
                        double *orbittot, double *lstot)
{
  const long nx = nh * ne, hh = nh * nh;
  const zc *C = (const zc *)coeff, *S = (const zc *)s_mom, *L = (const zc *)l_mom;
  const zc *L2 = (const zc *)l2_mom, *LS = (const zc *)ldots;
  zc *osp = (zc *)spin, *ost = (zc *)spintot, *oor = (zc *)orbit, *oot = (zc *)orbittot, *ols = (zc *)lstot;
  /* two-body sums: sum_{a,i,b,j} c_ai conj(c_bj) Me_d(a, b) Mh_d(i, j)
   *   = sum_{a,i,j} c_ai Mh_d(i, j) T_d(a, j),  T_d(a, j) = sum_b conj(c_bj) Me_d(a, b) */
  zc *T = malloc(sizeof(zc) * (size_t)ne * nh * 6), *Tl2 = malloc(sizeof(zc) * (size_t)ne * nh);
  if (!T || !Tl2) { free(T); free(Tl2); return -1; }
  for (long n = 0; n < nx; n++) {
    zc sp[3] = {0, 0, 0}, orb[3] = {0, 0, 0}, stot = 0, otot = 0, lst = 0;
    /* T[k][a][j] = sum_b conj(c_bj) E_k(a, b) for E = S_d (k 0..2), L_d (3..5) */
    for (long a = 0; a < ne; a++)
      for (long j = 0; j < nh; j++) {
        zc t[6] = {0, 0, 0, 0, 0, 0}, tl2 = 0;
        for (long b = 0; b < ne; b++) {
          const zc cb = conj(C[(b * nh + j) * nx + n]);
          const long e = hh + a * ne + b;
          for (int d = 0; d < 3; d++) {
            t[d] += cb * S[e * 3 + d];
            t[3 + d] += cb * L[e * 3 + d];
          }
          if (b == a) tl2 = cb; /* the a == b terms: conj(c_aj) */
        }
        for (int k = 0; k < 6; k++) T[(k * ne + a) * nh + j] = t[k];
        Tl2[a * nh + j] = tl2; /* = conj(c_aj) */
      }
    for (long a = 0; a < ne; a++)
      for (long i = 0; i < nh; i++) {
        const zc cai = C[(a * nh + i) * nx + n];
        /* one-body parts: <S>, <L> (angular.c:737-764, 890-917) */
        for (int d = 0; d < 3; d++) {
          zc st = 0, lt = 0;
          for (long b = 0; b < ne; b++) {
            const zc cb = conj(C[(b * nh + i) * nx + n]);
            st += cb * S[(hh + a * ne + b) * 3 + d];
            lt += cb * L[(hh + a * ne + b) * 3 + d];
          }
          for (long j = 0; j < nh; j++) {
            const zc cj = conj(C[(a * nh + j) * nx + n]);
            st += cj * S[(i * nh + j) * 3 + d];
            lt += cj * L[(i * nh + j) * 3 + d];
          }
          sp[d] += cai * st;
          orb[d] += cai * lt;
        }
        /* two-body parts over (b, j) (angular.c:766-787, 919-947, 980-1032) */
        for (long j = 0; j < nh; j++) {
          const long h = i * nh + j;
          zc s2 = 0, o2 = 0, x2 = 0;
          for (int d = 0; d < 3; d++) {
            const zc Ts = T[(d * ne + a) * nh + j], Tl = T[((3 + d) * ne + a) * nh + j];
            s2 += Ts * S[h * 3 + d];
            o2 += 2.0 * Tl * L[h * 3 + d];
            x2 += Tl * S[h * 3 + d] + Ts * L[h * 3 + d];
          }
          /* a == b: + L2_h(i, j), + LS_h(i, j) with weight conj(c_aj) */
          o2 += Tl2[a * nh + j] * L2[h];
          x2 += Tl2[a * nh + j] * LS[h];
          stot += cai * s2;
          otot += cai * o2;
          lst += cai * x2;
        }
        /* i == j: + L2_e(a, b), + LS_e(a, b) with weight conj(c_bi) */
        for (long b = 0; b < ne; b++) {
          const zc cb = conj(C[(b * nh + i) * nx + n]);
          const long e = hh + a * ne + b;
          otot += cai * cb * L2[e];
          lst += cai * cb * LS[e];
        }
      }
    for (int d = 0; d < 3; d++) {
      osp[n * 3 + d] = sp[d];
      oor[n * 3 + d] = orb[d];
    }
    ost[n] = stot;
    oot[n] = otot;
    ols[n] = lst;
  }
  free(T);
  free(Tl2);
  return 0;
}
