/* Type-only stand-in for <mkl.h> (MKL ILP64 types) used only to compile the
 * reference's pure-C hot-path files into the test-only oracle/_ref library. */
#pragma once
#include <stdlib.h>
typedef struct { double real; double imag; } MKL_Complex16;
static inline void mkl_set_num_threads(int n) { (void)n; }
static inline void mkl_set_dynamic(int n) { (void)n; }
/* the LAPACKE row-major interface the BSE solve uses (bse_cplx/diag.c:38),
 * ILP64 as the reference builds it; defined in lapack_shim.c */
typedef long long lapack_int;
typedef MKL_Complex16 lapack_complex_double;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int LAPACKE_zheev(int matrix_layout, char jobz, char uplo, lapack_int n, lapack_complex_double *a,
                         lapack_int lda, double *w);
