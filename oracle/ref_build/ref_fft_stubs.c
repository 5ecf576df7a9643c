/* Test-only: the functions of the reference's init.c that call into files
 * not compiled into oracle/_ref/libfbse_ref_fft.so (file readers, strain,
 * LAPACK-based projector generation, cube writer).  The pinned paths (init_kvec,
 * kinetic, calc_angular_exp) never reach them; these definitions only satisfy
 * the linker and stop the process loudly if one is ever called. */
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
