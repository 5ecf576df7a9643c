/* Host-side setup of the drop-in executables: the reference's input files
 * (input.par, conf.par, pot<Atm>.par, SO_<Atm>.par), its grid rule, the
 * spin-orbit / nonlocal projector table, and its output files (eval.dat,
 * psi.dat, output.dat).  Plain C; the compute runs through libfbse_gpu. */
#ifndef FBSE_DROPIN_H
#define FBSE_DROPIN_H

#include <stdio.h>

#define FBSE_PROJ_LEN 1024 /* PROJ_LEN, filter_mpi/fd.h */
#define FBSE_NPROJ 5       /* ist->nproj default, filter_mpi/read.c:75 */
#define FBSE_MAX_TYPES 32

/* the subset of filter_mpi/input.par this library runs (read.c:23-112 defaults) */
typedef struct {
  long nx, ny, nz;            /* requested minimum grid (0: from the atoms) */
  double dx, dy, dz;
  long m_states_per_filter, n_filter_cycles, ncheby;
  double vbmin, vbmax, cbmin, cbmax;
  double ke_max, fermi_e, sigma_e_cut;
  int set_targets;
  long n_targets_vb, n_targets_cb;
  int set_seed;
  long seed;
  int use_spinors, so, nl, get_all_states, approx_energy_range, precision;
  /* restart / state files (read.c:34-35, 87-93, 762-787, 954-967) */
  int print_psi_filt, print_psi_diag, calc_filter_only, restart_from_ortho, restart_from_sigma;
  long n_states_for_ortho, n_states_for_sigma;
  int print_cubes; /* printCubes = 1 <ncubes> (read.c:691-715) */
  long ncubes;
  int read_coeffs; /* readCoeffs = 1: zn.dat and coeff-<t>.dat are read (mod_filter.c:116-126) */
  int input_psi_filt; /* inputPsiFilt = 1 <start> <end>: starts from psi-init.dat (init.c:1166-1203) */
  long init_psi_start, init_psi_end;
  int calc_spin_ang_stat; /* calcSpinAngStat = 1: angular.dat (mod_optional_output.c:51-62) */
} fbse_filter_params;

/* the subset of bse_cplx/input.par (bse_cplx/read.c) */
typedef struct {
  long max_hole_states, max_elec_states;
  double sigma_e_cut, eps_x, eps_y, eps_z, fermi_e, delta_e_hole, delta_e_elec;
  int precision;
  /* kernel files (bse_cplx/read.c:58-60, 127-129; mod_kernel.c:31-96) */
  int coulomb_done, restart_coulomb, calc_coulomb_only;
  int calc_spin_ang_stat; /* main.c:160-195 */
} fbse_bse_params;

/* input.par parsing: returns 0, or -1 with a message in err */
int fbse_read_filter_params(const char *path, fbse_filter_params *p, char *err, size_t errlen);
int fbse_read_bse_params(const char *path, fbse_bse_params *p, char *err, size_t errlen);

/* conf.par: natoms, then "Atm x y z" (bohr); centred (centerConf).  types[i]
 * indexes names[]; returns 0 or -1. */
int fbse_read_conf(const char *path, long *natoms, double **xyz, int **types, char names[][8], int *ntypes,
                   char *err, size_t errlen);

/* energy targets of one filter (set_ene_targets, init.c:401-478): n_vb in
 * the valence window, m - n_vb in the conduction window; targets [m] */
void fbse_ene_targets(long m, long n_vb, double vbmin, double vbmax, double cbmin, double cbmax, double *targets);

/* quasiparticle basis of the BSE stage (get_qp_basis_indices,
 * bse_cplx/basis.c:7-254): sel [n] receives the eval.dat indices of the kept
 * holes then electrons; returns their number */
long fbse_qp_basis(const double *eval, const double *sigma, long n, double sigma_cut, double fermi_e,
                   long max_holes, long max_elecs, long *sel, long *n_holes, long *n_elecs);

/* 1 for the ligand labels (P1-P4, PC5, PC6, PR1-3, PA1-3, C1-3), which carry
 * no SO / NL projectors */
int fbse_is_ligand(const char *atyp);

/* SO_<atyp>.par from the working directory: SO_par and NL_par[2]; 0 or -1 */
int fbse_read_so_params(const char *atyp, double *so_par, double *nl_par, char *err, size_t errlen);

/* two-column table (r, V): returns the number of rows (or -1) */
long fbse_read_table(const char *path, double **r, double **v);

/* init_grid_params (filter_mpi/init.c:5-255, non-periodic) */
void fbse_grid_rule(const double *xyz, long natoms, double d, long n_in, int axis, long *n, double *xmin);

/* cumulative-sum coordinates of build_grid_ksqr (init.c:284-290) */
void fbse_grid_axis(long n, double lo, double d, double *out);

/* R_NLcut2 (read.c:908) */
double fbse_r_nlcut2(double dx);

/* radial projectors (filter_mpi/projectors.c): SO (kind 0) or NL (kind 1,
 * lam1 exp(-r^2) + lam2 exp(-(r-1.5)^2)); out [nproj][PROJ_LEN]; sgn (NL)
 * gets the eigenvalue signs.  Returns 0 or -1. */
int fbse_radial_projectors(double dx, double rcut, int kind, double lam1, double lam2, int nproj, double *out,
                           int *sgn);

/* the init_NL_projectors table: fbse_build_nlc (on the GPU, declared in
 * include/fbse.h) */

/* NL spectral bounds of the table (init.c:1095-1130) */
void fbse_nl_bounds(long nat, long npts, int nproj, const long *nl, const double *y1, const double *nlp,
                    const int *sgn, double dv, double *lam_min, double *lam_max);

/* spectrum range rule of get_energy_range (energy.c:302-369): approx = 1
 * builds [Emin, Emax] from Vmax_local, KE_max and the projector pads; both
 * then get the inflation.  emin / emax in (approx = 0: the iterated
 * extremes) and out. */
void fbse_energy_range_rule(int approx, int so, int nl, double vmin_loc, double vmax_loc, double ke_max,
                            double lam_min, double lam_max, double *emin, double *emax);

/* outputs (filter_mpi/write.c:263-299, save.c:446-503) */
int fbse_write_eval(const char *path, const double *eval, const double *sigma, long n);
int fbse_write_psi(const char *path, const double *psi, long n_doubles);

/* direct-0.dat / exchange-0.dat in the working directory (bse_cplx/coulomb.c:
 * 289-371, 534-602; bse_real/coulomb.c:352, 583): dir / exc [n_xton][n_xton]
 * as (re, im) pairs; 0 or -1 */
int fbse_write_kernel_files(const double *dir, const double *exc, long nh, long ne, long lumo, int real);

/* h0.dat, bs*.dat, HBSmat*.dat, BSEcoeff*.dat of the solve (bse_cplx/mod_bse.c,
 * bethe-salpeter.c; bse_real's single-part files when real = 1) from the full
 * kernels and the eigenvectors ([n_xton][n_xton] (re, im) pairs); 0 or -1 */
int fbse_write_bse_matrices(const double *dir, const double *exc, const double *coef, const double *eqp, long nh,
                            long ne, long lumo, int real);

/* qp_spins.dat (qp_spin_frac, bse_cplx/spin.c:3-60): per spinor of psi
 * (nqp complex spinors of 2 ngrid points) its two spin-block norms; 0 or -1 */
int fbse_write_qp_spins(const char *path, const double *psi, const double *eqp, long nqp, long ngrid, double dv);

/* the atom id of a conf.par label (assign_atom_number, read.c:2452-2545) */
long fbse_atom_number(const char *label);

/* output.dat (save_output, save.c:446-503): tag on the first line, the
 * types' ids from their labels (labels8: ntypes x 8 chars), the grid
 * metadata as init_grid_params leaves it, then axes, eval, sigma and the
 * states.  Returns 0 or -1. */
int fbse_write_output(const char *path, long tag, long natoms, const double *xyz, int ntypes, const char *labels8,
                      long nx, long ny, long nz, double dx, double dy, double dz, const double *gx, const double *gy,
                      const double *gz, double xmin, double ymin, double zmin, double ke_max, double fermi_e, int so,
                      int nl, int use_spinors, int nspin, int cplx, long n, const double *eval, const double *sigma,
                      const double *psi);

/* calc_xton_spin_mtrx + calc_xton_ang_mom_mtrx (bse_cplx/angular.c:692-1043):
 * per exciton n (complex, interleaved) <S> spin[n][3], the two-body spin sum
 * spintot[n] (spins.dat prints 1.5 + 2 Re), <L> orbit[n][3], the <L^2> sum
 * orbittot[n] (orbital.dat) and the <L.S> sum lstot[n] (couple.dat), from the
 * coefficients coeff[ibs][n] (ibs = a * n_h + i) and fbse_bse_qp_ang_mom's
 * matrices.  Returns 0 or -1 (allocation). */
int fbse_xton_ang_stats(long nh, long ne, const double *coeff, const double *s_mom, const double *l_mom,
                        const double *l2_mom, const double *ldots, double *spin, double *spintot, double *orbit,
                        double *orbittot, double *lstot);

/* write_cube_file (filter_mpi/write.c:65-139): rho [ngrid] in grid order,
 * atoms as 8-byte symbol slots (sym8) and xyz (bohr); returns 0 or -1 (an
 * atom symbol the reference's cube table does not know) */
int fbse_write_cube(const char *path, const double *rho, long nx, long ny, long nz, double dx, double dy, double dz,
                    double xmin, double ymin, double zmin, long natoms, const char *sym8, const double *xyz);

#endif
