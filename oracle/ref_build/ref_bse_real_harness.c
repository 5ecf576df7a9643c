/* Test-only harness of oracle/_ref/libfbse_ref_bse_real.so: the reference's
 * real-valued BSE stage (bse_real/: one-component real states) compiled from
 * where it lies with the FFTW subset (fftw_shim.c), the LAPACK forwarders
 * (lapack_shim.c: its diag calls dsyev_) and one-rank MPI (mpi_single.c),
 * behind plain-argument wrappers for the pin tests. */
#include <string.h>

#include "fd.h"
#include "ref_bse_job.h"

void init_elec_hole_kernel(double complex *pot_bare, double complex *pot_screened, grid_st *grid, index_st *ist,
                           par_st *par, flag_st *flag, parallel_st *parallel);
void calc_eh_kernel_cplx(double *psi_qp, double complex *pot_bare, double complex *pot_screened, double *direct,
                         double *exchange, index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);
void build_h0_mat(double *h0mat, double *eval, index_st *ist);
void build_BSE_mat(double *bsmat, double *direct, double *exchange, index_st *ist);
void bethe_salpeter(double *direct, double *exchange, double *bsmat, double *bs_coeff, double *h0mat,
                    double *xton_ene, grid_st *grid, index_st *ist, par_st *par, flag_st *flag,
                    parallel_st *parallel);
void calc_elec_dipole(xyz_st *elec_dip, double *psi_qp, double *eig_vals, grid_st *grid, index_st *ist, par_st *par,
                      flag_st *flag);
void calc_mag_dipole(xyz_st *mag_dip, double *psi_qp, double *eig_vals, grid_st *grid, index_st *ist, par_st *par,
                     flag_st *flag);
void calc_optical_exc(double *bs_coeff, double *xton_ene, double *eig_vals, xyz_st *mu, xyz_st *m, index_st *ist,
                      par_st *par);

/* the spinor job made a one-component real one */
static void real_job(struct bjob *j)
{
  j->ist.nspin = 1;
  j->ist.nspinngrid = j->ist.ngrid;
  j->ist.complex_idx = 1;
  j->flag.SO = 0;
  j->flag.useSpinors = 0;
  j->flag.isComplex = 0;
}

/* init_elec_hole_kernel (bse_real/init.c:8-283) */
void ref_bser_potentials(long nx, long ny, long nz, double dx, double dy, double dz, double xmin, double ymin,
                         double zmin, double *gx, double *gy, double *gz, double epsx, double epsy, double epsz,
                         double *bare, double *scr)
{
  struct bjob j;
  bjob_init(&j, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, gx, gy, gz, 1, 1, 1);
  real_job(&j);
  j.par.epsX = epsx;
  j.par.epsY = epsy;
  j.par.epsZ = epsz;
  j.pl.mpi_rank = 1; /* quiet */
  init_elec_hole_kernel((double complex *)bare, (double complex *)scr, &j.grid, &j.ist, &j.par, &j.flag, &j.pl);
}

/* calc_eh_kernel_cplx of bse_real (coulomb.c:20-705) at one rank: direct and
 * exchange [n_xton][n_xton] real; writes its kernel files into the working
 * directory */
void ref_bser_kernel(double *psi_qp, long nh, long ne, long lumo, long nx, long ny, long nz, double dx, double dy,
                     double dz, double xmin, double ymin, double zmin, double *gx, double *gy, double *gz,
                     double *bare, double *scr, double *direct, double *exchange)
{
  struct bjob j;
  bjob_init(&j, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, gx, gy, gz, nh, ne, lumo);
  real_job(&j);
  calc_eh_kernel_cplx(psi_qp, (double complex *)bare, (double complex *)scr, direct, exchange, &j.ist, &j.par,
                      &j.flag, &j.pl);
}

/* build_h0_mat + build_BSE_mat + bethe_salpeter (bse_real/mod_bse.c:59-130,
 * bethe-salpeter.c:7-250): exciton energies and coefficients (row n of the
 * [n_xton][n_xton] matrix is exciton n, as dsyev leaves them); writes h0.dat,
 * bs.dat, HBSmat.dat, BSEcoeff.dat and exciton.dat into the working directory */
void ref_bser_solve(double *direct, double *exchange, double *eval_qp, long nh, long ne, long lumo, double *xton_ene,
                    double *coeff)
{
  struct bjob j;
  double g0 = 0;
  bjob_init(&j, 1, 1, 1, 1, 1, 1, 0, 0, 0, &g0, &g0, &g0, nh, ne, lumo);
  real_job(&j);
  const long n = nh * ne;
  double *h0 = calloc(n * n, sizeof(double));
  double *bs = calloc(n * n, sizeof(double));
  build_h0_mat(h0, eval_qp, &j.ist);
  build_BSE_mat(bs, direct, exchange, &j.ist);
  bethe_salpeter(direct, exchange, bs, coeff, h0, xton_ene, &j.grid, &j.ist, &j.par, &j.flag, &j.pl);
  free(h0);
  free(bs);
}

/* calc_elec_dipole and calc_mag_dipole (bse_real/dipole.c:7-331): mu and m
 * [n_h * n_e][3] complex; writes OS0.dat and M0.dat into the working
 * directory */
void ref_bser_dipoles(double *psi_qp, double *eval_qp, long nh, long ne, long lumo, long nx, long ny, long nz,
                      double dx, double dy, double dz, double xmin, double ymin, double zmin, double *gx, double *gy,
                      double *gz, double *mu, double *m)
{
  struct bjob j;
  bjob_init(&j, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, gx, gy, gz, nh, ne, lumo);
  real_job(&j);
  calc_elec_dipole((xyz_st *)mu, psi_qp, eval_qp, &j.grid, &j.ist, &j.par, &j.flag);
  calc_mag_dipole((xyz_st *)m, psi_qp, eval_qp, &j.grid, &j.ist, &j.par, &j.flag);
}

/* calc_optical_exc (bse_real/optical.c:6-100): writes OS.dat, M.dat, rs.dat
 * and bs-coeff-<j>.dat into the working directory */
void ref_bser_optical(double *coeff, double *xton_ene, double *eval_qp, double *mu, double *m, long nh, long ne,
                      long lumo)
{
  struct bjob j;
  double g0 = 0;
  bjob_init(&j, 1, 1, 1, 1, 1, 1, 0, 0, 0, &g0, &g0, &g0, nh, ne, lumo);
  real_job(&j);
  calc_optical_exc(coeff, xton_ene, eval_qp, (xyz_st *)mu, (xyz_st *)m, &j.ist, &j.par);
}
