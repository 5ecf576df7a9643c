/* Type-only stand-in for <mkl.h> (MKL ILP64 types) used only to compile the
 * reference's pure-C hot-path files into the test-only oracle/_ref library. */
#pragma once
#include <stdlib.h>
typedef struct { double real; double imag; } MKL_Complex16;
static inline void mkl_set_num_threads(int n) { (void)n; }
