/* Type-only stand-in for <mpi.h> used only to compile the reference's
 * pure-C hot-path files into the test-only oracle/_ref library.  None of the
 * compiled functions communicates. */
#pragma once
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int source, tag, error; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_COMM_NULL (-1)
#define MPI_DOUBLE 1
typedef int MPI_Op;
#define MPI_SUM 1
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
/* declared so that filter.c and the BSE files compile; libfbse_ref_fft.so
 * defines them as aborting stubs (ref_fft_stubs.c: the pinned filter paths
 * never communicate), libfbse_ref_bse.so with one-rank semantics
 * (mpi_single.c: the reference's BSE kernel calls its collectives at one rank too) */
int MPI_Barrier(MPI_Comm comm);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *newcomm);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Gather(const void *s, int sc, MPI_Datatype st, void *r, int rc, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Send(const void *b, int c, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *b, int c, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status *st);
int MPI_Abort(MPI_Comm comm, int code);
