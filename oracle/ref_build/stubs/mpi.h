/* Type-only stand-in for <mpi.h> used only to compile the reference's
 * pure-C hot-path files into the test-only oracle/_ref library.  None of the
 * compiled functions communicates. */
#pragma once
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
#define MPI_COMM_NULL (-1)
