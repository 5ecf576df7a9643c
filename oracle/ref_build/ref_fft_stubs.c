/* Test-only: the functions that the reference's init.c and filter.c call
 * into files not compiled into oracle/_ref/libfbse_ref_fft.so (file readers,
 * strain, LAPACK-based projector generation, cube writer, MPI, the k-point
 * path).  The pinned paths (init_kvec, kinetic, p_hamiltonian, filter_cycle,
 * calc_angular_exp) never reach them; these definitions only satisfy the
 * linker and stop the process loudly if one is ever called. */
#include <stdio.h>
#include <stdlib.h>

static void unreachable(const char *name)
{
  fprintf(stderr, "oracle/_ref: %s is not part of the pinned reference subset\n", name);
  abort();
}

void allocate_memory(void) { unreachable("allocate_memory"); }
void calc_strain_scale(void) { unreachable("calc_strain_scale"); }
void gen_SO_projectors(void) { unreachable("gen_SO_projectors"); }
void gen_nlc_projectors(void) { unreachable("gen_nlc_projectors"); }
void read_nearest_neighbors(void) { unreachable("read_nearest_neighbors"); }
void read_pot(void) { unreachable("read_pot"); }
void read_psi_dat(void) { unreachable("read_psi_dat"); }
void write_cube_file(void) { unreachable("write_cube_file"); }
/* filter.c: the MPI gathers of psi_rank, the periodic (k-point) path, energy
 * and timing helpers, and the progress bar (rank 0 only; the harness runs as
 * rank 1) */
void MPI_Abort(void) { unreachable("MPI_Abort"); }
void MPI_Comm_rank(void) { unreachable("MPI_Comm_rank"); }
void MPI_Comm_size(void) { unreachable("MPI_Comm_size"); }
void MPI_Gather(void) { unreachable("MPI_Gather"); }
void MPI_Recv(void) { unreachable("MPI_Recv"); }
void MPI_Send(void) { unreachable("MPI_Send"); }
void create_fft_plans(void) { unreachable("create_fft_plans"); }
void destroy_fft_plans(void) { unreachable("destroy_fft_plans"); }
void e_ikr(void) { unreachable("e_ikr"); }
void energy_all(void) { unreachable("energy_all"); }
void energy_all_k(void) { unreachable("energy_all_k"); }
void get_time(void) { unreachable("get_time"); }
void kinetic_k(void) { unreachable("kinetic_k"); }
void p_hamiltonian_k(void) { unreachable("p_hamiltonian_k"); }
void print_progress_bar(void) { unreachable("print_progress_bar"); }
