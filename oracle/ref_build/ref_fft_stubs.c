/* Test-only: the functions that the reference files compiled into
 * oracle/_ref/libfbse_ref_fft.so call in files that are not compiled (file
 * readers, strain, MPI, the periodic k-point path).  The pinned single-rank,
 * non-periodic paths (kinetic, p_hamiltonian, filter_cycle, ortho_cplx,
 * diag_H, calc_sigma_E, calc_angular_exp, get_energy_range,
 * init_NL_projectors, read_conf, init_grid_params, build_grid_ksqr,
 * build_local_pot) never reach them; these definitions only satisfy the
 * linker and stop the process loudly if one is ever called. */
#include <stdio.h>
#include <stdlib.h>

static void unreachable(const char *name)
{
  fprintf(stderr, "oracle/_ref: %s is not part of the pinned reference subset\n", name);
  abort();
}

void MPI_Abort(void) { unreachable("MPI_Abort"); }
void MPI_Comm_rank(void) { unreachable("MPI_Comm_rank"); }
void MPI_Comm_size(void) { unreachable("MPI_Comm_size"); }
void MPI_Gather(void) { unreachable("MPI_Gather"); }
void MPI_Recv(void) { unreachable("MPI_Recv"); }
void MPI_Send(void) { unreachable("MPI_Send"); }
void calc_strain_scale(void) { unreachable("calc_strain_scale"); }
void e_ikr(void) { unreachable("e_ikr"); }
void hamiltonian_k(void) { unreachable("hamiltonian_k"); }
void kinetic_k(void) { unreachable("kinetic_k"); }
void p_hamiltonian_k(void) { unreachable("p_hamiltonian_k"); }
void read_nearest_neighbors(void) { unreachable("read_nearest_neighbors"); }
void retScaledVector(void) { unreachable("retScaledVector"); }
