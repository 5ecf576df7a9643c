/* Stand-in for <fftw3.h>, used only to compile the reference's hot-path C
 * files into the test-only oracle/_ref libraries.  In libfbse_ref.so the
 * transform resolves to an aborting stub (ref_harness.c); in
 * libfbse_ref_fft.so / libfbse_ref_bse.so to the project-written FFTW subset
 * (fftw_shim.c). */
#pragma once
/* as FFTW's own header: a C99 complex type when <complex.h> came first */
#if defined(_Complex_I) && defined(complex) && defined(I)
typedef double _Complex fftw_complex;
#else
typedef double fftw_complex[2];
#endif
typedef struct fbse_ref_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
void fftw_execute(const fftw_plan p);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(unsigned long n);
void fftw_free(void *p);
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int n);
void fftw_cleanup_threads(void);
