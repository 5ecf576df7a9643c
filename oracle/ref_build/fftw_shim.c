/* Test-only FFTW subset for oracle/_ref/libfbse_ref_fft.so: the reference's
 * FFT-dependent files (hamiltonian.c's kinetic(), angular.c) are compiled from
 * where they lie against the type-only fftw3.h stand-in and linked with these
 * definitions.  Transforms are unnormalised 3D DFTs with FFTW's conventions
 * (fftw_plan_dft_3d(n0, n1, n2): n2 fastest; FFTW_FORWARD = e^{-2 pi i jk/n},
 * FFTW_BACKWARD = e^{+2 pi i jk/n}, no 1/N), computed as direct
 * one-dimensional DFTs along each axis with long-double twiddles and sums, so
 * they are exact to the FP64 rounding of the data for the small grids the pin
 * tests use.  Plans keep their arrays as FFTW's do. */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fftw3.h"

struct fbse_ref_fftw_plan_s {
  int n[3];
  fftw_complex *in, *out;
  int sign;
};

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign, unsigned flags)
{
  (void)flags;
  fftw_plan p = malloc(sizeof *p);
  if (!p) return NULL;
  p->n[0] = n0;
  p->n[1] = n1;
  p->n[2] = n2;
  p->in = in;
  p->out = out;
  p->sign = sign;
  return p;
}

/* DFT of every line along axis ax of the row-major [n0][n1][n2] array a */
static void dft_axis(fftw_complex *a, const int *n, int ax, int sign)
{
  const long len = n[ax];
  const long stride = ax == 2 ? 1 : (ax == 1 ? n[2] : (long)n[1] * n[2]);
  const long total = (long)n[0] * n[1] * n[2];
  long double *wr = malloc(len * sizeof *wr), *wi = malloc(len * sizeof *wi);
  long double *xr = malloc(len * sizeof *xr), *xi = malloc(len * sizeof *xi);
  const long double two_pi = 6.283185307179586476925286766559005768L;
  for (long m = 0; m < len; m++) {
    const long double t = two_pi * (long double)m / (long double)len;
    wr[m] = cosl(t);
    wi[m] = sign < 0 ? -sinl(t) : sinl(t);
  }
  for (long base = 0; base < total; base++) {
    /* a line starts at every index whose coordinate along ax is 0 */
    if ((base / stride) % len != 0) continue;
    for (long j = 0; j < len; j++) {
      xr[j] = a[base + j * stride][0];
      xi[j] = a[base + j * stride][1];
    }
    for (long k = 0; k < len; k++) {
      long double sr = 0.0L, si = 0.0L;
      for (long j = 0; j < len; j++) {
        const long m = (j * k) % len;
        sr += xr[j] * wr[m] - xi[j] * wi[m];
        si += xr[j] * wi[m] + xi[j] * wr[m];
      }
      a[base + k * stride][0] = (double)sr;
      a[base + k * stride][1] = (double)si;
    }
  }
  free(wr);
  free(wi);
  free(xr);
  free(xi);
}

void fftw_execute(const fftw_plan p)
{
  const long total = (long)p->n[0] * p->n[1] * p->n[2];
  if (p->out != p->in) memcpy(p->out, p->in, total * sizeof(fftw_complex));
  for (int ax = 2; ax >= 0; ax--) dft_axis(p->out, p->n, ax, p->sign);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
void *fftw_malloc(unsigned long n) { return malloc(n); }
void fftw_free(void *p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void)n; }
void fftw_cleanup_threads(void) {}
