/* Test-only harness of oracle/_ref/libfbse_ref_fft.so: plain-argument
 * wrappers around the reference's FFT-dependent functions, compiled from the
 * reference tree with the FFTW subset of fftw_shim.c, so the tests can pin
 * the oracle's kinetic term and angular statistics against the reference's
 * own code. */
#include <string.h>

#include "fd.h"
#include "angular.h"

/* kinetic() (hamiltonian.c:62-99) on one block of ngrid complex values:
 * out = FFTW_BACKWARD(ksqr * FFTW_FORWARD(psi)), ksqr as build_grid_ksqr
 * leaves it (1/N and the KE cap included); plans as create_fft_plans makes
 * them (aux.c:259-270: nz, ny, nx, in place) */
void ref_kinetic(double *out, const double *psi, long nx, long ny, long nz, double *ksqr)
{
  index_st ist;
  memset(&ist, 0, sizeof ist);
  ist.nx = nx;
  ist.ny = ny;
  ist.nz = nz;
  ist.ngrid = nx * ny * nz;
  fftw_complex *buf = fftw_malloc(ist.ngrid * sizeof(fftw_complex));
  fftw_plan fw = fftw_plan_dft_3d((int)nz, (int)ny, (int)nx, buf, buf, FFTW_FORWARD, FFTW_MEASURE);
  fftw_plan bw = fftw_plan_dft_3d((int)nz, (int)ny, (int)nx, buf, buf, FFTW_BACKWARD, FFTW_MEASURE);
  memcpy(out, psi, ist.ngrid * 2 * sizeof(double));
  kinetic((zomplex *)out, ksqr, fw, bw, buf, &ist);
  fftw_destroy_plan(fw);
  fftw_destroy_plan(bw);
  fftw_free(buf);
}

/* calc_angular_exp (angular.c:4-165) for complex spinor states start..stop-1
 * of psitot; writes angular.dat into the working directory */
void ref_angular(double *psitot, long n_states, long nx, long ny, long nz, double dx, double dy, double dz, double *gx,
                 double *gy, double *gz, double dkx, double dky, double dkz, int start, int stop)
{
  grid_st grid;
  index_st ist;
  par_st par;
  flag_st flag;
  parallel_st pl;
  memset(&grid, 0, sizeof grid);
  memset(&ist, 0, sizeof ist);
  memset(&par, 0, sizeof par);
  memset(&flag, 0, sizeof flag);
  memset(&pl, 0, sizeof pl);
  grid.nx = nx;
  grid.ny = ny;
  grid.nz = nz;
  grid.ngrid = nx * ny * nz;
  grid.ngrid_1 = 1.0 / (double)grid.ngrid;
  grid.nx_1 = 1.0 / (double)nx;
  grid.ny_1 = 1.0 / (double)ny;
  grid.nz_1 = 1.0 / (double)nz;
  grid.dx = dx;
  grid.dy = dy;
  grid.dz = dz;
  grid.x = gx;
  grid.y = gy;
  grid.z = gz;
  grid.dkx = dkx;
  grid.dky = dky;
  grid.dkz = dkz;
  grid.dv = dx * dy * dz;
  ist.nx = nx;
  ist.ny = ny;
  ist.nz = nz;
  ist.ngrid = nx * ny * nz;
  ist.nspin = 2;
  ist.nspinngrid = 2 * ist.ngrid;
  ist.complex_idx = 2;
  ist.mn_states_tot = n_states;
  par.dv = dx * dy * dz;
  flag.isComplex = 1;
  flag.useSpinors = 1;
  flag.SO = 1;
  pl.nthreads = 1;
  calc_angular_exp(psitot, &grid, start, stop, &ist, &par, &flag, &pl);
}
