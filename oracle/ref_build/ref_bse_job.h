/* Test-only: the job description (grid, indices, parameters, flags, one-rank
 * parallel record) shared by the wrappers around the reference's BSE stages
 * (bse_cplx/, bse_real/: the same struct layouts).  Include after "fd.h". */
#pragma once
#include <string.h>

struct bjob {
  grid_st grid;
  index_st ist;
  par_st par;
  flag_st flag;
  parallel_st pl;
};

/* the grid of the BSE stage (x_j = xmin + j dx as bse_cplx/read.c:398-409
 * builds it, coordinates passed in) and the spinor job of n_h holes and
 * n_e electrons at lumo_idx */
static void bjob_init(struct bjob *j, long nx, long ny, long nz, double dx, double dy, double dz, double xmin,
                      double ymin, double zmin, double *gx, double *gy, double *gz, long nh, long ne, long lumo)
{
  memset(j, 0, sizeof *j);
  j->grid.nx = nx;
  j->grid.ny = ny;
  j->grid.nz = nz;
  j->grid.ngrid = nx * ny * nz;
  j->grid.dx = dx;
  j->grid.dy = dy;
  j->grid.dz = dz;
  j->grid.dv = dx * dy * dz;
  /* set by read_input (read.c:353) and init_elec_hole_kernel (init.c:132) */
  j->grid.nx_1 = 1.0 / (double)nx;
  j->grid.ny_1 = 1.0 / (double)ny;
  j->grid.nz_1 = 1.0 / (double)nz;
  j->grid.dkx = 2.0 * 3.14159265358979323846 / ((double)nx * dx);
  j->grid.dky = 2.0 * 3.14159265358979323846 / ((double)ny * dy);
  j->grid.dkz = 2.0 * 3.14159265358979323846 / ((double)nz * dz);
  j->grid.xmin = xmin;
  j->grid.ymin = ymin;
  j->grid.zmin = zmin;
  j->grid.x = gx;
  j->grid.y = gy;
  j->grid.z = gz;
  j->ist.nx = nx;
  j->ist.ny = ny;
  j->ist.nz = nz;
  j->ist.ngrid = nx * ny * nz;
  j->ist.ngrid_1 = 1.0 / (double)j->ist.ngrid;
  j->ist.nspin = 2;
  j->ist.nspinngrid = 2 * j->ist.ngrid;
  j->ist.complex_idx = 2;
  j->ist.nthreads = 1;
  j->ist.n_holes = nh;
  j->ist.n_elecs = ne;
  j->ist.lumo_idx = lumo;
  j->ist.n_xton = nh * ne;
  j->par.dv = j->grid.dv;
  j->par.dx = dx;
  j->par.dy = dy;
  j->par.dz = dz;
  j->flag.SO = 1;
  j->flag.useSpinors = 1;
  j->flag.isComplex = 1;
  j->pl.nthreads = 1;
  j->pl.mpi_rank = 0;
  j->pl.mpi_size = 1;
}
