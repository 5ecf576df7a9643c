/* Test-only: print_input_state (bse_cplx/save.c, not compiled) for the BSE
 * read_input compiled into oracle/_ref/libfbse_ref_bse.so.  read_input calls
 * it only at rank 0; the harness runs it at a non-zero rank, so this
 * definition only satisfies the linker and stops the process loudly if it is
 * ever called. */
#include <stdio.h>
#include <stdlib.h>

void print_input_state(void)
{
  fprintf(stderr, "oracle/_ref: print_input_state is not part of the pinned reference subset\n");
  abort();
}
