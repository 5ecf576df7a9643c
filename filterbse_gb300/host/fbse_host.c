/*
 * fbse_host.c -- host-side pieces of the filter path that stay C (tiny,
 * FP64, bit-exact requirements): the reference's random generator and
 * random starts, and the Newton interpolation nodes and coefficients.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/fbse.h"

/* ran_nrc (filter_mpi/rand.c:22-62): L'Ecuyer's combination of two
 * multiplicative congruential generators (moduli 2147483563 and 2147483399,
 * Schrage's method) with a 32-entry Bays-Durham shuffle.  Like the reference,
 * the second generator, the shuffle table and its last output are
 * process-wide; a non-positive seed re-initialises them. */
static struct {
  long s2;
  long last;
  long table[32];
} g_rng = {123456789, 0, {0}};

static long lcg_step(long s, long a, long q, long r, long m)
{
  long k = s / q;
  s = a * (s - k * q) - k * r;
  return (s < 0) ? s + m : s;
}

double fbse_ran(long *seed)
{
  enum { M1 = 2147483563, M2 = 2147483399, TAB = 32 };
  if (*seed <= 0) {
    *seed = (-(*seed) < 1) ? 1 : -(*seed);
    g_rng.s2 = *seed;
    for (int j = TAB + 7; j >= 0; j--) { /* 8 warm-up steps, then fill */
      *seed = lcg_step(*seed, 40014, 53668, 12211, M1);
      if (j < TAB) g_rng.table[j] = *seed;
    }
    g_rng.last = g_rng.table[0];
  }
  *seed = lcg_step(*seed, 40014, 53668, 12211, M1);
  g_rng.s2 = lcg_step(g_rng.s2, 40692, 52774, 3791, M2);
  long slot = g_rng.last / (1 + (M1 - 1) / TAB);
  g_rng.last = g_rng.table[slot] - g_rng.s2;
  g_rng.table[slot] = *seed;
  if (g_rng.last < 1) g_rng.last += M1 - 1;
  double u = g_rng.last * (1.0 / (double)M1);
  return (u > 1.0 - 1.2e-7) ? 1.0 - 1.2e-7 : u;
}

/* init_psi (filter_mpi/init.c:1256-1307): one spin block of U[-1, 1] values in
 * grid order (re then im per point for complex jobs), normalised to 1 with dv
 * (normalize, filter_mpi/norm.c:42-79).  psi is interleaved complex.
 * Returns the advanced seed. */
long fbse_host_init_psi(double *psi, long seed, long ngrid, int is_complex, double dv)
{
  for (long j = 0; j < ngrid; j++) {
    psi[2 * j] = -1.0 + 2.0 * fbse_ran(&seed);
    psi[2 * j + 1] = is_complex ? -1.0 + 2.0 * fbse_ran(&seed) : 0.0;
  }
  double s = 0.0;
  for (long j = 0; j < ngrid; j++) s += psi[2 * j] * psi[2 * j] + psi[2 * j + 1] * psi[2 * j + 1];
  double nrm = sqrt(s * dv);
  for (long j = 0; j < 2 * ngrid; j++) psi[j] /= nrm;
  return seed;
}

long fbse_init_filter_states(double *psitot, long n_filters, long ngrid, int nspin, int is_complex, double dv,
                             long seed, long *seeds_out)
{
  double *blk = (double *)malloc(2 * ngrid * sizeof(double));
  long cidx = is_complex ? 2 : 1;
  long stlen = cidx * nspin * ngrid;
  for (long jns = 0; jns < n_filters; jns++) {
    for (int s = 0; s < nspin; s++) {
      if (seeds_out) seeds_out[jns * nspin + s] = seed;
      seed = fbse_host_init_psi(blk, seed, ngrid, is_complex, dv);
      double *dst = psitot + jns * stlen + (long)s * ngrid * cidx;
      for (long j = 0; j < ngrid; j++) {
        if (is_complex) {
          dst[2 * j] = blk[2 * j];
          dst[2 * j + 1] = blk[2 * j + 1];
        } else {
          dst[j] = blk[2 * j];
        }
      }
    }
  }
  free(blk);
  return seed;
}

/* samp_points_ashkenazy (filter_mpi/coeff.c:227-293) on [-2, 2]: 32*ncheby
 * candidates, the last eighth on the (zero-length) imaginary segment; each new
 * node maximises the running sum of log squared distances to the chosen ones
 * (candidates closer than 1e-5 to a chosen node are excluded).  The nodes are
 * real, so only their real parts are returned. */
double fbse_samp_points(long ncheby, double *zn)
{
  const long nc = 32 * ncheby, nim = nc / 8;
  const double lo = -2.0, hi = 2.0, step = (hi - lo) / (double)(nc - 1 - nim);
  double *cand = (double *)calloc(nc, sizeof(double));
  double *score = (double *)malloc(nc * sizeof(double));
  double *zim = (double *)calloc(ncheby, sizeof(double));
  for (long j = 0; j < nc - nim; j++) cand[j] = lo + (double)j * step;
  /* the imaginary segment of zero width maps to the point 0 (coeff.c:237-246) */
  zn[0] = cand[0];
  for (long k = 0; k < nc; k++) {
    double d = (cand[k] - zn[0]) * (cand[k] - zn[0]);
    score[k] = (d < 1.0e-10) ? -1.0e30 : log(d);
  }
  for (long j = 1; j < ncheby; j++) {
    long arg = 0;
    double best = -2.0e30;
    for (long k = 0; k < nc; k++)
      if (score[k] > best) { best = score[k]; arg = k; }
    zn[j] = cand[arg];
    for (long k = 0; k < nc; k++) {
      double d = (cand[k] - zn[j]) * (cand[k] - zn[j]);
      if (d < 1.0e-10) score[k] = -1.0e30;
      else score[k] += log(d);
    }
  }
  double prod = 1.0;
  for (long j = 0; j < ncheby; j++) prod *= zn[j] * zn[j] + zim[j] * zim[j];
  free(cand);
  free(score);
  free(zim);
  return pow(sqrt(prod), 1.0 / (double)ncheby);
}

/* gen_newton_coeff (filter_mpi/coeff.c:8-118): Newton divided differences
 * of the Gaussian filter sqrt(dt/pi) exp(-dt (x - E_t)^2) at the nodes mapped
 * back to energy, x = (z + 2) dE/4 + Vmin.  an is [m][ncheby] complex
 * (interleaved), imaginary parts 0. */
int fbse_newton_coeff(long ncheby, long m, const double *zn, const double *targets, double vmin, double de,
                      double dt, double *an)
{
  if (ncheby < 2 || m < 1 || !(de > 0)) return FBSE_ERR_ARG;
  const double scale = 4.0 / de, pref = sqrt(dt / 3.14159265358979323846);
  for (long t = 0; t < m; t++) {
    double *a = an + 2 * ncheby * t;
    double x = (zn[0] + 2.0) / scale + vmin;
    a[0] = pref * exp(-(x - targets[t]) * (x - targets[t]) * dt);
    a[1] = 0.0;
    x = (zn[1] + 2.0) / scale + vmin;
    a[2] = (pref * exp(-(x - targets[t]) * (x - targets[t]) * dt) - a[0]) / (zn[1] - zn[0]);
    a[3] = (-a[1]) / (zn[1] - zn[0]);
    for (long j = 2; j < ncheby; j++) {
      double w = 1.0, sr = 0.0, si = 0.0;
      for (long i = 1; i < j; i++) {
        w *= (zn[j] - zn[i - 1]);
        sr += a[2 * i] * w;
        si += a[2 * i + 1] * w;
      }
      w *= (zn[j] - zn[j - 1]);
      x = (zn[j] + 2.0) / scale + vmin;
      a[2 * j] = (pref * exp(-(x - targets[t]) * (x - targets[t]) * dt) - a[0] - sr) / w;
      a[2 * j + 1] = (-a[1] - si) / w;
    }
  }
  return FBSE_OK;
}
