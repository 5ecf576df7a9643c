/* Test-only LAPACK entry points for oracle/_ref/libfbse_ref_fft.so: the
 * reference calls MKL's ILP64 LAPACK (zgesvd_, dgesvd_, zheev_, dsyev_ with
 * long long integers, ortho.c:54,150, Hmat.c:201,211, aux.c:122).  These
 * forward to the ILP64 LAPACK that numpy ships (OpenBLAS, symbols with the
 * scipy_ prefix and 64_ suffix), opened at run time from the path the test
 * passes to ref_set_lapack, with the hidden lengths of the one-character
 * arguments that the Fortran routines take. */
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>

typedef long long ll;
static void *g_lapack;

int ref_set_lapack(const char *path)
{
  g_lapack = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  return g_lapack != NULL;
}

static void *sym(const char *name)
{
  void *f = g_lapack ? dlsym(g_lapack, name) : NULL;
  if (!f) {
    fprintf(stderr, "oracle/_ref: %s is not available (call ref_set_lapack first)\n", name);
    abort();
  }
  return f;
}

typedef void (*gesvd_z)(const char *, const char *, const ll *, const ll *, void *, const ll *, double *, void *,
                        const ll *, void *, const ll *, void *, const ll *, double *, ll *, size_t, size_t);
typedef void (*gesvd_d)(const char *, const char *, const ll *, const ll *, double *, const ll *, double *,
                        double *, const ll *, double *, const ll *, double *, const ll *, ll *, size_t, size_t);
typedef void (*heev_z)(const char *, const char *, const ll *, void *, const ll *, double *, void *, const ll *,
                       double *, ll *, size_t, size_t);
typedef void (*syev_d)(const char *, const char *, const ll *, double *, const ll *, double *, double *, const ll *,
                       ll *, size_t, size_t);

void zgesvd_(const char *jobu, const char *jobvt, const ll *m, const ll *n, void *a, const ll *lda, double *s,
             void *u, const ll *ldu, void *vt, const ll *ldvt, void *work, const ll *lwork, double *rwork, ll *info)
{
  ((gesvd_z)sym("scipy_zgesvd_64_"))(jobu, jobvt, m, n, a, lda, s, u, ldu, vt, ldvt, work, lwork, rwork, info, 1, 1);
}

void dgesvd_(const char *jobu, const char *jobvt, const ll *m, const ll *n, double *a, const ll *lda, double *s,
             double *u, const ll *ldu, double *vt, const ll *ldvt, double *work, const ll *lwork, ll *info)
{
  ((gesvd_d)sym("scipy_dgesvd_64_"))(jobu, jobvt, m, n, a, lda, s, u, ldu, vt, ldvt, work, lwork, info, 1, 1);
}

void zheev_(const char *jobz, const char *uplo, const ll *n, void *a, const ll *lda, double *w, void *work,
            const ll *lwork, double *rwork, ll *info)
{
  ((heev_z)sym("scipy_zheev_64_"))(jobz, uplo, n, a, lda, w, work, lwork, rwork, info, 1, 1);
}

void dsyev_(const char *jobz, const char *uplo, const ll *n, double *a, const ll *lda, double *w, double *work,
            const ll *lwork, ll *info)
{
  ((syev_d)sym("scipy_dsyev_64_"))(jobz, uplo, n, a, lda, w, work, lwork, info, 1, 1);
}

/* LAPACKE_zheev (row-major, bse_cplx/diag.c:38): the row-major matrix is
 * copied to column-major storage of the same logical matrix, zheev_ runs on
 * it, and the eigenvectors (columns) are copied back, as LAPACKE does */
typedef struct { double re, im; } zc;
ll LAPACKE_zheev(int layout, char jobz, char uplo, ll n, void *a, ll lda, double *w)
{
  zc *m = (zc *)a;
  zc *t = malloc((size_t)(n > 0 ? n * n : 1) * sizeof(zc));
  double *rwork = malloc((size_t)(3 * n > 1 ? 3 * n : 1) * sizeof(double));
  ll info = 0, lwork = -1;
  zc q;
  if (!t || !rwork) abort();
  for (ll i = 0; i < n; i++)
    for (ll j = 0; j < n; j++) t[i + j * n] = layout == 101 ? m[i * lda + j] : m[i + j * lda];
  const ll ldt = n > 0 ? n : 1;
  zheev_(&jobz, &uplo, &n, t, &ldt, w, &q, &lwork, rwork, &info);  /* workspace query */
  lwork = (ll)q.re;
  zc *work = malloc((size_t)(lwork > 0 ? lwork : 1) * sizeof(zc));
  if (!work) abort();
  zheev_(&jobz, &uplo, &n, t, &ldt, w, work, &lwork, rwork, &info);
  for (ll i = 0; i < n; i++)
    for (ll j = 0; j < n; j++) {
      if (layout == 101) m[i * lda + j] = t[i + j * n];
      else m[i + j * lda] = t[i + j * n];
    }
  free(work);
  free(rwork);
  free(t);
  return info;
}
