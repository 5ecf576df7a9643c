/* Test-only: one-rank MPI for oracle/_ref/libfbse_ref_bse.so.  The
 * reference's BSE kernel (bse_cplx/coulomb.c:125-150, 650-725) splits
 * communicators and reduces its matrices even when it runs on one rank; with
 * one rank a split returns a usable communicator, rank 0 of size 1, an
 * in-place reduction leaves the data as it is and a barrier returns. */
#include <stdlib.h>
#include <string.h>

#include "mpi.h"

int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *newcomm)
{
  (void)comm;
  (void)key;
  *newcomm = 100 + color;
  return 0;
}
int MPI_Comm_free(MPI_Comm *comm)
{
  *comm = MPI_COMM_NULL;
  return 0;
}
int MPI_Comm_rank(MPI_Comm comm, int *rank)
{
  (void)comm;
  *rank = 0;
  return 0;
}
int MPI_Comm_size(MPI_Comm comm, int *size)
{
  (void)comm;
  *size = 1;
  return 0;
}
int MPI_Barrier(MPI_Comm comm)
{
  (void)comm;
  return 0;
}
int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm)
{
  (void)op;
  (void)root;
  (void)comm;
  if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)count * (t == MPI_DOUBLE ? sizeof(double) : 1));
  return 0;
}
int MPI_Send(const void *b, int c, MPI_Datatype t, int dest, int tag, MPI_Comm comm)
{
  (void)b; (void)c; (void)t; (void)dest; (void)tag; (void)comm;
  abort(); /* no partner at one rank */
}
int MPI_Recv(void *b, int c, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status *st)
{
  (void)b; (void)c; (void)t; (void)src; (void)tag; (void)comm; (void)st;
  abort();
}
