/* Test-only harness of oracle/_ref/libfbse_ref_bse.so: the reference's BSE
 * stage (bse_cplx/) compiled from where it lies with the FFTW subset
 * (fftw_shim.c), the LAPACKE / LAPACK forwarders (lapack_shim.c) and one-rank
 * MPI (mpi_single.c), behind plain-argument wrappers for the pin tests. */
#include <string.h>

#include "fd.h"
#include "ref_bse_job.h"

void init_elec_hole_kernel(double complex *pot_bare, double complex *pot_screened, grid_st *grid, index_st *ist,
                           par_st *par, flag_st *flag, parallel_st *parallel);
void calc_eh_kernel_cplx(double complex *psi_qp, double complex *pot_bare, double complex *pot_screened,
                         double complex *direct, double complex *exchange, index_st *ist, par_st *par, flag_st *flag,
                         parallel_st *parallel);
void build_h0_mat(double *h0mat, double *eval, index_st *ist);
void build_BSE_mat(double complex *bsmat, double complex *direct, double complex *exchange, index_st *ist);
void bethe_salpeter(double complex *direct, double complex *exchange, double complex *bsmat, double complex *bs_coeff,
                    double *h0mat, double *xton_ene, grid_st *grid, index_st *ist, par_st *par, flag_st *flag,
                    parallel_st *parallel);
void calc_elec_dipole(xyz_st *elec_dip, double complex *psi_qp, double *eig_vals, grid_st *grid, index_st *ist,
                      par_st *par, flag_st *flag);

/* init_elec_hole_kernel (bse_cplx/init.c:8-268): bare and screened
 * interactions in k space (ngrid complex each) */
void ref_bse_potentials(long nx, long ny, long nz, double dx, double dy, double dz, double xmin, double ymin,
                        double zmin, double *gx, double *gy, double *gz, double epsx, double epsy, double epsz,
                        double *bare, double *scr)
{
  struct bjob j;
  bjob_init(&j, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, gx, gy, gz, 1, 1, 1);
  j.par.epsX = epsx;
  j.par.epsY = epsy;
  j.par.epsZ = epsz;
  j.pl.mpi_rank = 1; /* quiet */
  init_elec_hole_kernel((double complex *)bare, (double complex *)scr, &j.grid, &j.ist, &j.par, &j.flag, &j.pl);
}

/* calc_eh_kernel_cplx (bse_cplx/coulomb.c:20-738) at one rank: direct and
 * exchange [n_xton][n_xton] complex (the triangles the reference fills);
 * writes its kernel files into the working directory */
void ref_bse_kernel(double *psi_qp, long nh, long ne, long lumo, long nx, long ny, long nz, double dx, double dy,
                    double dz, double xmin, double ymin, double zmin, double *gx, double *gy, double *gz,
                    double *bare, double *scr, double *direct, double *exchange)
{
  struct bjob j;
  bjob_init(&j, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, gx, gy, gz, nh, ne, lumo);
  calc_eh_kernel_cplx((double complex *)psi_qp, (double complex *)bare, (double complex *)scr,
                      (double complex *)direct, (double complex *)exchange, &j.ist, &j.par, &j.flag, &j.pl);
}

/* build_h0_mat + build_BSE_mat + bethe_salpeter (bse_cplx/mod_bse.c:54-148,
 * bethe-salpeter.c:7-350): exciton energies and coefficients (column j of the
 * row-major [n_xton][n_xton] matrix); writes h0.dat, bs*.dat, HBSmat*.dat,
 * BSEcoeff*.dat and exciton.dat into the working directory */
void ref_bse_solve(double *direct, double *exchange, double *eval_qp, long nh, long ne, long lumo, double *xton_ene,
                   double *coeff)
{
  struct bjob j;
  double gx = 0, gy = 0, gz = 0;
  bjob_init(&j, 1, 1, 1, 1, 1, 1, 0, 0, 0, &gx, &gy, &gz, nh, ne, lumo);
  const long n = nh * ne;
  double *h0 = calloc(n * n, sizeof(double));
  double complex *bs = calloc(n * n, sizeof(double complex));
  build_h0_mat(h0, eval_qp, &j.ist);
  build_BSE_mat(bs, (double complex *)direct, (double complex *)exchange, &j.ist);
  bethe_salpeter((double complex *)direct, (double complex *)exchange, bs, (double complex *)coeff, h0, xton_ene,
                 &j.grid, &j.ist, &j.par, &j.flag, &j.pl);
  free(h0);
  free(bs);
}

/* calc_elec_dipole (bse_cplx/dipole.c:7-158): mu [n_h * n_e][3] complex;
 * writes OS0.dat into the working directory */
void ref_bse_dipoles(double *psi_qp, double *eval_qp, long nh, long ne, long lumo, long nx, long ny, long nz,
                     double dx, double dy, double dz, double xmin, double ymin, double zmin, double *gx, double *gy,
                     double *gz, double *mu)
{
  struct bjob j;
  bjob_init(&j, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, gx, gy, gz, nh, ne, lumo);
  calc_elec_dipole((xyz_st *)mu, (double complex *)psi_qp, eval_qp, &j.grid, &j.ist, &j.par, &j.flag);
}

void calc_mag_dipole(xyz_st *mag_dip, double complex *psi_qp, double *eig_vals, grid_st *grid, index_st *ist,
                     par_st *par, flag_st *flag);
void calc_optical_exc(double complex *bs_coeff, double *xton_ene, double *eig_vals, xyz_st *mu, xyz_st *m,
                      index_st *ist, par_st *par);

/* calc_mag_dipole (bse_cplx/dipole.c:160-331): m [n_h * n_e][3] complex;
 * writes M0.dat into the working directory */
void ref_bse_mag_dipoles(double *psi_qp, double *eval_qp, long nh, long ne, long lumo, long nx, long ny, long nz,
                         double dx, double dy, double dz, double xmin, double ymin, double zmin, double *gx,
                         double *gy, double *gz, double *m)
{
  struct bjob j;
  bjob_init(&j, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, gx, gy, gz, nh, ne, lumo);
  calc_mag_dipole((xyz_st *)m, (double complex *)psi_qp, eval_qp, &j.grid, &j.ist, &j.par, &j.flag);
}

/* calc_optical_exc (bse_cplx/optical.c:6-99): writes OS.dat, M.dat, rs.dat
 * and bs-coeff-<j>.dat into the working directory */
void ref_bse_optical(double *coeff, double *xton_ene, double *eval_qp, double *mu, double *m, long nh, long ne,
                     long lumo)
{
  struct bjob j;
  double g0 = 0;
  bjob_init(&j, 1, 1, 1, 1, 1, 1, 0, 0, 0, &g0, &g0, &g0, nh, ne, lumo);
  calc_optical_exc((double complex *)coeff, xton_ene, eval_qp, (xyz_st *)mu, (xyz_st *)m, &j.ist, &j.par);
}

void calc_qp_spin_mtrx(double complex *psi_qp, xyz_st *s_mom, grid_st *grid, index_st *ist, par_st *par);
void calc_qp_ang_mom_mtrx(double complex *psi_qp, xyz_st *l_mom, double complex *l2_mom, double complex *ldots,
                          grid_st *grid, index_st *ist, par_st *par);
void calc_xton_spin_mtrx(double complex *bs_coeff, xyz_st *s_mom, index_st *ist, par_st *par, flag_st *flag,
                         parallel_st *parallel);
void calc_xton_ang_mom_mtrx(double complex *bs_coeff, xyz_st *s_mom, xyz_st *l_mom, double complex *l2_mom,
                            double complex *ldots, index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);

/* calc_qp_spin_mtrx + calc_qp_ang_mom_mtrx (bse_cplx/angular.c:7-690): the
 * hole-hole then electron-electron blocks, s and l [nh^2 + ne^2][3] complex,
 * l2 and ls [nh^2 + ne^2] complex; writes sx/sy/sz, lx/ly/lz, lsqr and ls
 * .dat files into the working directory */
void ref_bse_qp_ang_mom(double *psi_qp, long nh, long ne, long lumo, long nx, long ny, long nz, double dx, double dy,
                        double dz, double xmin, double ymin, double zmin, double *gx, double *gy, double *gz,
                        double *s, double *l, double *l2, double *ls)
{
  struct bjob j;
  bjob_init(&j, nx, ny, nz, dx, dy, dz, xmin, ymin, zmin, gx, gy, gz, nh, ne, lumo);
  calc_qp_spin_mtrx((double complex *)psi_qp, (xyz_st *)s, &j.grid, &j.ist, &j.par);
  calc_qp_ang_mom_mtrx((double complex *)psi_qp, (xyz_st *)l, (double complex *)l2, (double complex *)ls, &j.grid,
                       &j.ist, &j.par);
}

/* calc_xton_spin_mtrx + calc_xton_ang_mom_mtrx (bse_cplx/angular.c:692-1043)
 * on exciton coefficients [n_xton][n_xton] (column n = exciton n); writes
 * spins.dat, orbital.dat and couple.dat into the working directory */
void ref_bse_xton_ang(double *coeff, double *s, double *l, double *l2, double *ls, long nh, long ne, long lumo)
{
  struct bjob j;
  double g0 = 0;
  bjob_init(&j, 1, 1, 1, 1, 1, 1, 0, 0, 0, &g0, &g0, &g0, nh, ne, lumo);
  calc_xton_spin_mtrx((double complex *)coeff, (xyz_st *)s, &j.ist, &j.par, &j.flag, &j.pl);
  calc_xton_ang_mom_mtrx((double complex *)coeff, (xyz_st *)s, (xyz_st *)l, (double complex *)l2,
                         (double complex *)ls, &j.ist, &j.par, &j.flag, &j.pl);
}

void get_qp_basis_indices(double *eig_vals, double *sigma_E, long **eval_hole_idxs, long **eval_elec_idxs,
                          index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);

/* get_qp_basis_indices (bse_cplx/basis.c:7-254) at rank 0 over n eval.dat
 * entries (eval and sigma are reordered in place, as the reference does):
 * the eval.dat indices of the kept holes then electrons into sel, the counts
 * and homo / lumo positions into info[4]; writes BSEeval.par into the working
 * directory */
void ref_bse_qp_basis(double *eval, double *sigma, long n, double sigma_cut, double fermi_e, long max_holes,
                      long max_elecs, long *sel, long *info)
{
  struct bjob j;
  double g0 = 0;
  bjob_init(&j, 1, 1, 1, 1, 1, 1, 0, 0, 0, &g0, &g0, &g0, 0, 0, 0);
  j.ist.mn_states_tot = n;
  j.ist.max_hole_states = max_holes;
  j.ist.max_elec_states = max_elecs;
  j.par.sigma_E_cut = sigma_cut;
  j.par.fermi_E = fermi_e;
  long *hole = NULL, *elec = NULL;
  get_qp_basis_indices(eval, sigma, &hole, &elec, &j.ist, &j.par, &j.flag, &j.pl);
  for (long i = 0; i < j.ist.n_holes; i++) sel[i] = hole[i];
  for (long i = 0; i < j.ist.n_elecs; i++) sel[j.ist.n_holes + i] = elec[i];
  info[0] = j.ist.n_holes;
  info[1] = j.ist.n_elecs;
  info[2] = j.ist.homo_idx;
  info[3] = j.ist.lumo_idx;
  free(hole);
  free(elec);
}

void read_input(flag_st *flag, grid_st *grid, index_st *ist, par_st *par, parallel_st *parallel);

/* read_input of the BSE stage (bse_cplx/read.c:7-220) at a non-zero rank on
 * input.par in the working directory.  d[8]: sigma_E_cut, epsX, epsY, epsZ,
 * fermi_E, delta_E_hole, delta_E_elec, KE_max.  l[9]: max_hole_states,
 * max_elec_states, coulombDone, restartCoulomb, calcCoulombOnly,
 * calcSpinAngStat, SO, NL, useSpinors. */
void ref_bse_read_input(double *d, long *l)
{
  struct bjob j;
  double g0 = 0;
  bjob_init(&j, 1, 1, 1, 1, 1, 1, 0, 0, 0, &g0, &g0, &g0, 0, 0, 0);
  memset(&j.flag, 0, sizeof j.flag);
  j.pl.mpi_rank = 1;
  read_input(&j.flag, &j.grid, &j.ist, &j.par, &j.pl);
  const double dv[8] = {j.par.sigma_E_cut, j.par.epsX, j.par.epsY, j.par.epsZ,
                        j.par.fermi_E, j.par.delta_E_hole, j.par.delta_E_elec, j.par.KE_max};
  const long lv[9] = {j.ist.max_hole_states, j.ist.max_elec_states, j.flag.coulombDone, j.flag.restartCoulomb,
                      j.flag.calcCoulombOnly, j.flag.calcSpinAngStat, j.flag.SO, j.flag.NL, j.flag.useSpinors};
  memcpy(d, dv, sizeof dv);
  memcpy(l, lv, sizeof lv);
}

void qp_spin_frac(double complex *psi_qp, double *eig_vals, grid_st *grid, index_st *ist, par_st *par,
                  flag_st *flag, parallel_st *parallel);

/* qp_spin_frac (bse_cplx/spin.c:3-60): qp_spins.dat for n_qp complex spinors
 * of ngrid points per spin block, into the working directory */
void ref_bse_qp_spins(double *psi_qp, double *eval, long n_qp, long nx, long ny, long nz, double dv)
{
  struct bjob j;
  double g0 = 0;
  bjob_init(&j, nx, ny, nz, 1, 1, dv, 0, 0, 0, &g0, &g0, &g0, 0, 0, 0);
  j.ist.n_qp = n_qp;
  j.par.dv = dv;
  qp_spin_frac((double complex *)psi_qp, eval, &j.grid, &j.ist, &j.par, &j.flag, &j.pl);
}
