/* Test-only harness of oracle/_ref/libfbse_ref_fft.so: plain-argument
 * wrappers around the reference's FFT-dependent functions, compiled from the
 * reference tree with the FFTW subset of fftw_shim.c, so the tests can pin
 * the oracle's kinetic term and angular statistics against the reference's
 * own code. */
#include <stdlib.h>
#include <string.h>

#include "fd.h"
#include "angular.h"
#include "hamiltonian.h"

void filter_cycle(double *psi_rank, long jns, zomplex *psi, zomplex *phi, double *pot_local, zomplex *LS, nlc_st *nlc,
                  long *nl, double *ksqr, zomplex *an, double *zn, double *ene_targets, grid_st *grid, index_st *ist,
                  par_st *par, flag_st *flag, parallel_st *parallel, fftw_plan_loc planfw, fftw_plan_loc planbw,
                  fftw_complex *fftwpsi);

/* the job description and projector table of one H psi, in the reference's
 * structs (nlc_st array of structures from the oracle's SoA table) */
struct job {
  index_st ist;
  par_st par;
  flag_st flag;
  parallel_st pl;
  nlc_st *nlc;
  fftw_complex *buf;
  fftw_plan fw, bw;
};

static void job_init(struct job *j, long nx, long ny, long nz, int nspin, int is_complex, int so, int nl, long nat,
                     long npts, long nproj, const int *jxyz, const double *y1, const double *proj, const double *nlp,
                     const int *sgn, double dv)
{
  memset(j, 0, sizeof *j);
  j->ist.nx = nx;
  j->ist.ny = ny;
  j->ist.nz = nz;
  j->ist.ngrid = nx * ny * nz;
  j->ist.nspin = nspin;
  j->ist.nspinngrid = nspin * j->ist.ngrid;
  j->ist.complex_idx = is_complex ? 2 : 1;
  j->ist.n_NL_atoms = nat;
  j->ist.n_NL_gridpts = npts;
  j->ist.nproj = nproj;
  j->ist.n_s_ang_mom = 2;
  j->ist.n_l_ang_mom = 3;
  j->ist.n_j_ang_mom = 6;
  j->par.dv = dv;
  j->par.ham_threads = 1;
  j->flag.SO = so;
  j->flag.NL = nl;
  j->flag.isComplex = is_complex;
  j->flag.useSpinors = nspin == 2;
  j->pl.nthreads = 1;
  j->pl.mpi_rank = 1; /* no progress bar */
  j->nlc = calloc(nat * npts > 0 ? nat * npts : 1, sizeof(nlc_st));
  for (long a = 0; a < nat; a++)
    for (long g = 0; g < npts; g++) {
      const long e = a * npts + g;
      j->nlc[e].jxyz = jxyz[e];
      for (int m = 0; m < 3; m++) {
        j->nlc[e].y1[m].re = y1[e * 6 + 2 * m];
        j->nlc[e].y1[m].im = y1[e * 6 + 2 * m + 1];
      }
      for (long p = 0; p < nproj; p++) {
        j->nlc[e].proj[p] = proj[e * nproj + p];
        j->nlc[e].NL_proj[p] = nlp[e * nproj + p];
        j->nlc[e].NL_proj_sign[p] = sgn[a * nproj + p];
      }
    }
  j->buf = fftw_malloc(j->ist.ngrid * sizeof(fftw_complex));
  j->fw = fftw_plan_dft_3d((int)nz, (int)ny, (int)nx, j->buf, j->buf, FFTW_FORWARD, FFTW_MEASURE);
  j->bw = fftw_plan_dft_3d((int)nz, (int)ny, (int)nx, j->buf, j->buf, FFTW_BACKWARD, FFTW_MEASURE);
}

static void job_free(struct job *j)
{
  fftw_destroy_plan(j->fw);
  fftw_destroy_plan(j->bw);
  fftw_free(j->buf);
  free(j->nlc);
}

/* p_hamiltonian (phamiltonian.c:10-60) on one state: out = H psi (zomplex,
 * nspin * ngrid); pot2 holds the local potential twice as init.c:666 leaves it */
void ref_hamiltonian(double *out, const double *psi, long nx, long ny, long nz, int nspin, int is_complex, int so,
                     int nl, double *pot2, double *ls, double *ksqr, long nat, long npts, long nproj, long *nlcnt,
                     const int *jxyz, const double *y1, const double *proj, const double *nlp, const int *sgn,
                     double dv)
{
  struct job j;
  job_init(&j, nx, ny, nz, nspin, is_complex, so, nl, nat, npts, nproj, jxyz, y1, proj, nlp, sgn, dv);
  zomplex *tmp = calloc(j.ist.nspinngrid, sizeof(zomplex));
  memcpy(out, psi, j.ist.nspinngrid * sizeof(zomplex));
  p_hamiltonian((zomplex *)out, tmp, pot2, (zomplex *)ls, j.nlc, nlcnt, ksqr, &j.ist, &j.par, &j.flag, j.fw, j.bw,
                j.buf, 1);
  free(tmp);
  job_free(&j);
}

/* filter_cycle (filter.c:187-371) of one start: psi_rank holds the start in
 * its first stlen doubles on entry and the m filtered states on return;
 * an [m][ncheby] zomplex, zn [ncheby] */
void ref_filter_cycle(double *psi_rank, long nx, long ny, long nz, int nspin, int is_complex, int so, int nl,
                      double *pot2, double *ls, double *ksqr, long nat, long npts, long nproj, long *nlcnt,
                      const int *jxyz, const double *y1, const double *proj, const double *nlp, const int *sgn,
                      double dv, double *an, double *zn, long ncheby, long m, double vmin, double de)
{
  struct job j;
  job_init(&j, nx, ny, nz, nspin, is_complex, so, nl, nat, npts, nproj, jxyz, y1, proj, nlp, sgn, dv);
  j.ist.ncheby = ncheby;
  j.ist.m_states_per_filter = m;
  j.par.Vmin = vmin;
  j.par.dE = de;
  j.par.dE_1 = 4.0 / de;
  zomplex *psi = calloc(j.ist.nspinngrid, sizeof(zomplex)), *phi = calloc(j.ist.nspinngrid, sizeof(zomplex));
  grid_st grid;
  memset(&grid, 0, sizeof grid);
  filter_cycle(psi_rank, 0, psi, phi, pot2, (zomplex *)ls, j.nlc, nlcnt, ksqr, (zomplex *)an, zn, NULL, &grid, &j.ist,
               &j.par, &j.flag, &j.pl, j.fw, j.bw, j.buf);
  free(psi);
  free(phi);
  job_free(&j);
}

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

long ortho_cplx(MKL_Complex16 *psitot, double dv, long n_cols, index_st *ist, par_st *par, flag_st *flag,
                parallel_st *parallel);
void normalize_all(double *psitot, long n_states, index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);
void diag_H(double *psitot, double *pot_local, vector *G_vecs, vector *k_vecs, zomplex *LS, nlc_st *nlc, long *nl,
            double *ksqr, double *eval, long n_states, int k_idx, index_st *ist, par_st *par, flag_st *flag,
            parallel_st *parallel);
void calc_sigma_E(double *psitot, double *pot_local, zomplex *LS, nlc_st *nlc, long *nl, double *ksqr,
                  double *sigma_E, index_st *ist, par_st *par, flag_st *flag);
int ref_set_lapack(const char *path);

/* mod_ortho's orthogonalisation of n complex states (ortho_cplx,
 * ortho.c:93-185, then normalize_all as mod_ortho.c:84 does) followed by
 * mod_diag's diag_H (Hmat.c:5-297) and normalize_all (mod_diag.c:424-433) and
 * mod_sigma's calc_sigma_E (energy.c:383-539):
 * psitot holds the n states on entry and the kept eigenvectors on return;
 * eval and sigma receive n_kept values; returns n_kept.  Writes hmat-0.dat
 * and eval_aux.dat into the working directory as the reference does. */
long ref_ritz(double *psitot, long n, long nx, long ny, long nz, int nspin, int so, int nl, double *pot2, double *ls,
              double *ksqr, long nat, long npts, long nproj, long *nlcnt, const int *jxyz, const double *y1,
              const double *proj, const double *nlp, const int *sgn, double dv, double *eval, double *sigma)
{
  struct job j;
  job_init(&j, nx, ny, nz, nspin, 1, so, nl, nat, npts, nproj, jxyz, y1, proj, nlp, sgn, dv);
  j.pl.k_rank = 1; /* quiet */
  j.ist.nthreads = 1;
  const long kept = ortho_cplx((MKL_Complex16 *)psitot, dv, n, &j.ist, &j.par, &j.flag, &j.pl);
  normalize_all(psitot, kept, &j.ist, &j.par, &j.flag, &j.pl);
  j.ist.mn_states_tot = kept;
  diag_H(psitot, pot2, NULL, NULL, (zomplex *)ls, j.nlc, nlcnt, ksqr, eval, kept, 0, &j.ist, &j.par, &j.flag, &j.pl);
  normalize_all(psitot, kept, &j.ist, &j.par, &j.flag, &j.pl); /* mod_diag.c:110 */
  calc_sigma_E(psitot, pot2, (zomplex *)ls, j.nlc, nlcnt, ksqr, sigma, &j.ist, &j.par, &j.flag);
  job_free(&j);
  return kept;
}

void get_energy_range(zomplex *psi, zomplex *phi, double *pot_local, grid_st *grid, zomplex *LS, nlc_st *nlc,
                      long *nl, double *ksqr, index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);

/* get_energy_range (energy.c:169-379, iterative branch) of a complex job:
 * vmin and de as it leaves them in par (Vmin, dE).  Writes Emin-init.dat and
 * Emax-init.dat into the working directory as the reference does. */
void ref_energy_range(long nx, long ny, long nz, int nspin, int so, int nl, double *pot2, double *ls, double *ksqr,
                      long nat, long npts, long nproj, long *nlcnt, const int *jxyz, const double *y1,
                      const double *proj, const double *nlp, const int *sgn, double dv, double *vmin, double *de)
{
  struct job j;
  job_init(&j, nx, ny, nz, nspin, 1, so, nl, nat, npts, nproj, jxyz, y1, proj, nlp, sgn, dv);
  grid_st grid;
  memset(&grid, 0, sizeof grid);
  grid.nx = nx;
  grid.ny = ny;
  grid.nz = nz;
  grid.ngrid = nx * ny * nz;
  grid.dv = dv;
  zomplex *psi = calloc(j.ist.nspinngrid, sizeof(zomplex)), *phi = calloc(j.ist.nspinngrid, sizeof(zomplex));
  get_energy_range(psi, phi, pot2, &grid, (zomplex *)ls, j.nlc, nlcnt, ksqr, &j.ist, &j.par, &j.flag, &j.pl);
  *vmin = j.par.Vmin;
  *de = j.par.dE;
  free(psi);
  free(phi);
  job_free(&j);
}

void gen_SO_projectors(double dx, double rcut, long nproj, double *projectors, double *vr);
void init_NL_projectors(nlc_st *nlc, long *nl, double *SO_projectors, grid_st *grid, xyz_st *R, atom_info *atom,
                        index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);

/* gen_SO_projectors (projectors.c:12-84) on init_NL_projectors' radial grid
 * r_j = j sqrt(rc2) / PROJ_LEN: so_tab [nproj][PROJ_LEN]; writes its
 * projector files into the working directory */
void ref_so_projectors(double dx, double rc2, long nproj, double *so_tab)
{
  double *vr = malloc(PROJ_LEN * sizeof(double));
  const double dr = sqrt(rc2) / (double)PROJ_LEN;
  for (long j = 0; j < PROJ_LEN; j++) vr[j] = (double)j * dr;
  gen_SO_projectors(dx, sqrt(rc2), nproj, so_tab, vr);
  free(vr);
}

/* init_NL_projectors (init.c:848-1135) with the NL radial projectors made on
 * the fly by gen_nlc_projectors (projectors.c:87-228; NL_par per atom) and the
 * given SO radial projectors, non-periodic, at one rank.  Outputs the table
 * in the library's layout (nl[nat]; per entry e = atom * npts + point: jxyz,
 * y1 as (re, im) x 3, proj and NL_proj x nproj; sgn [nat][nproj]) and
 * lam = {NL_lambda_min, NL_lambda_max}.  Writes list_NL_grid.dat and the
 * projector files into the working directory. */
void ref_nl_projectors(long nx, long ny, long nz, double dx, double dy, double dz, double *gx, double *gy, double *gz,
                       long nat, const double *xyz, const double *so_par, const double *nl_par, double *so_tab,
                       double rc2, long nproj, long npts, long *nl, int *jxyz, double *y1, double *proj, double *nlp,
                       int *sgn, double *lam)
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
  grid.dx = dx;
  grid.dy = dy;
  grid.dz = dz;
  grid.dv = dx * dy * dz;
  grid.x = gx;
  grid.y = gy;
  grid.z = gz;
  ist.n_NL_atoms = nat;
  ist.n_NL_gridpts = npts;
  ist.nproj = nproj;
  ist.n_l_ang_mom = 3;
  par.R_NLcut2 = rc2;
  pl.nthreads = 1;
  pl.mpi_rank = 1; /* quiet */
  xyz_st *R = calloc(nat, sizeof(xyz_st));
  atom_info *atom = calloc(nat, sizeof(atom_info));
  for (long a = 0; a < nat; a++) {
    R[a].x = xyz[3 * a];
    R[a].y = xyz[3 * a + 1];
    R[a].z = xyz[3 * a + 2];
    atom[a].Zval = 1;
    atom[a].SO_par = so_par[a];
    atom[a].NL_par[0] = nl_par[2 * a];
    atom[a].NL_par[1] = nl_par[2 * a + 1];
  }
  nlc_st *nlc = calloc(nat * npts, sizeof(nlc_st));
  init_NL_projectors(nlc, nl, so_tab, &grid, R, atom, &ist, &par, &flag, &pl);
  for (long a = 0; a < nat; a++) {
    for (long p = 0; p < nproj; p++) sgn[a * nproj + p] = nlc[a * npts].NL_proj_sign[p];
    for (long g = 0; g < nl[a]; g++) {
      const long e = a * npts + g;
      jxyz[e] = (int)nlc[e].jxyz;
      for (int m = 0; m < 3; m++) {
        y1[e * 6 + 2 * m] = nlc[e].y1[m].re;
        y1[e * 6 + 2 * m + 1] = nlc[e].y1[m].im;
      }
      for (long p = 0; p < nproj; p++) {
        proj[e * nproj + p] = nlc[e].proj[p];
        nlp[e * nproj + p] = nlc[e].NL_proj[p];
      }
    }
  }
  lam[0] = par.NL_lambda_min;
  lam[1] = par.NL_lambda_max;
  free(nlc);
  free(atom);
  free(R);
}

/* get_energy_range's approxEnergyRange branch and range inflation
 * (energy.c:302-369): the local potential's Vmin / Vmax, KE_max and the NL
 * bounds in, Vmin (= Emin) and dE out */
void ref_energy_range_approx(int so, int nl, double vmin_loc, double vmax_loc, double ke_max, double lam_min,
                             double lam_max, double *emin, double *de)
{
  struct job j;
  job_init(&j, 1, 1, 1, 1, 1, so, nl, 0, 0, 0, NULL, NULL, NULL, NULL, NULL, 1.0);
  j.flag.approxEnergyRange = 1;
  j.par.Vmin = vmin_loc;
  j.par.Vmax = vmax_loc;
  j.par.KE_max = ke_max;
  j.par.NL_lambda_min = lam_min;
  j.par.NL_lambda_max = lam_max;
  grid_st grid;
  memset(&grid, 0, sizeof grid);
  grid.nx = grid.ny = grid.nz = 1;
  grid.ngrid = 1;
  grid.dv = 1.0;
  get_energy_range(NULL, NULL, NULL, &grid, NULL, j.nlc, NULL, NULL, &j.ist, &j.par, &j.flag, &j.pl);
  *emin = j.par.Vmin;
  *de = j.par.dE;
  job_free(&j);
}

void read_conf(xyz_st *R, atom_info *atom, index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);
void init_grid_params(grid_st *grid, xyz_st *R, index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);
void build_grid_ksqr(double *ksqr, xyz_st *R, grid_st *grid, index_st *ist, par_st *par, flag_st *flag,
                     parallel_st *parallel);
void build_local_pot(double *pot_local, pot_st *pot, xyz_st *R, atom_info *atom, grid_st *grid, index_st *ist,
                     par_st *par, flag_st *flag, parallel_st *parallel);

/* The setup chain of mod_init + mod_pseudopot (mod_init.c, mod_pseudopot.c)
 * at one rank, non-periodic, without strain, LSD or interpolated potentials:
 * read_conf (read.c:998-1172, conf.par in the working directory, centred at
 * the centre of mass), init_grid_params (init.c:5-256) from the input.par
 * grid (n_in, dgrid), build_grid_ksqr (init.c:259-398) and build_local_pot
 * (init.c:481-703, pot<Atm>.par in the working directory).  Outputs into
 * caller buffers: natoms, zval / type index / coordinates per atom (up to
 * cap_atoms), SO_par, NL_par[0], NL_par[1] per atom (sonl, read from
 * SO_<Atm>.par by read_pot when SO or NL is on), the grid counts n[3] and
 * origins lo[3], the axes (up to cap_axis
 * each), ksqr and the local potential (up to cap_grid), Vmin / Vmax,
 * n_NL_atoms and n_NL_gridpts (nlinfo).  Returns 0, or -1 if a capacity is
 * short or conf.par cannot be read. */
int ref_setup(double dgrid, const long *n_in, double ke_max, int so, int nl, long cap_atoms, long cap_axis,
              long cap_grid, long *natoms, long *zval, long *tidx, double *xyz, double *sonl, long *n, double *lo,
              double *gx, double *gy, double *gz, double *ksqr, double *pot, double *vrange, long *nlinfo)
{
  FILE *pf = fopen("conf.par", "r");
  long nat = 0;
  if (!pf || fscanf(pf, "%ld", &nat) != 1) {
    if (pf) fclose(pf);
    return -1;
  }
  fclose(pf);
  if (nat > cap_atoms) return -1;
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
  /* the read_input defaults this chain reads (read.c:9-61) */
  ist.n_max_atom_types = N_MAX_ATOM_TYPES;
  ist.atom_types = calloc(N_MAX_ATOM_TYPES, sizeof(long));
  ist.max_pot_file_len = 8192;
  ist.ngeoms = 1;
  ist.natoms = nat;
  ist.nspin = so ? 2 : 1;
  ist.complex_idx = so ? 2 : 1;
  par.scale_surface_Cs = 1.0;
  par.pot_cut_rad2 = 225.0;
  par.KE_max = ke_max;
  flag.centerConf = 1;
  flag.SO = so;
  flag.NL = nl;
  pl.nthreads = 1;
  pl.mpi_rank = 1; /* quiet */
  grid.nx = n_in[0];
  grid.ny = n_in[1];
  grid.nz = n_in[2];
  grid.dx = grid.dy = grid.dz = dgrid;
  par.R_NLcut2 = 1.5 + 6.0 * log(10.0) + 3.0 * dgrid; /* read.c:908 */
  xyz_st *R = calloc(nat, sizeof(xyz_st));
  atom_info *atom = calloc(nat, sizeof(atom_info));
  int rc = -1;
  read_conf(R, atom, &ist, &par, &flag, &pl);
  init_grid_params(&grid, R, &ist, &par, &flag, &pl);
  if (grid.nx > cap_axis || grid.ny > cap_axis || grid.nz > cap_axis || grid.ngrid > cap_grid) goto out;
  grid.x = gx;
  grid.y = gy;
  grid.z = gz;
  build_grid_ksqr(ksqr, R, &grid, &ist, &par, &flag, &pl);
  pot_st pt;
  memset(&pt, 0, sizeof pt);
  const long atyp_tot = ist.ngeoms * ist.n_atom_types, potfl = atyp_tot * ist.max_pot_file_len;
  pt.file_lens = calloc(atyp_tot, sizeof(long));
  pt.dr = calloc(atyp_tot, sizeof(double));
  pt.r = calloc(potfl, sizeof(double));
  pt.pseudo = calloc(potfl, sizeof(double));
  double *pl2 = calloc(2 * grid.ngrid, sizeof(double));
  build_local_pot(pl2, &pt, R, atom, &grid, &ist, &par, &flag, &pl);
  memcpy(pot, pl2, grid.ngrid * sizeof(double));
  free(pl2);
  free(pt.file_lens);
  free(pt.dr);
  free(pt.r);
  free(pt.pseudo);
  *natoms = nat;
  for (long a = 0; a < nat; a++) {
    zval[a] = atom[a].Zval;
    tidx[a] = atom[a].idx;
    xyz[3 * a] = R[a].x;
    xyz[3 * a + 1] = R[a].y;
    xyz[3 * a + 2] = R[a].z;
    sonl[3 * a] = atom[a].SO_par;
    sonl[3 * a + 1] = atom[a].NL_par[0];
    sonl[3 * a + 2] = atom[a].NL_par[1];
  }
  n[0] = grid.nx;
  n[1] = grid.ny;
  n[2] = grid.nz;
  lo[0] = grid.xmin;
  lo[1] = grid.ymin;
  lo[2] = grid.zmin;
  vrange[0] = par.Vmin;
  vrange[1] = par.Vmax;
  nlinfo[0] = ist.n_NL_atoms;
  nlinfo[1] = ist.n_NL_gridpts;
  rc = 0;
out:
  free(R);
  free(atom);
  free(ist.atom_types);
  return rc;
}

void init_filter_states(double *psi_rank, zomplex *psi, grid_st *grid, long *rand_seed, index_st *ist, par_st *par,
                        flag_st *flag, parallel_st *parallel);

/* init_filter_states (init.c:1138-1255) with init_psi (init.c:1256-1306) at
 * one rank: n_filters random starts, start j at state j * m of psi_rank
 * (m * n_filters states of nspin * ngrid * complex_idx doubles); returns the
 * advanced seed and writes seed-1.dat into the working directory */
long ref_init_filter_states(double *psi_rank, long nx, long ny, long nz, int nspin, int is_complex, double dv,
                            long n_filters, long m, long seed)
{
  struct job j;
  job_init(&j, nx, ny, nz, nspin, is_complex, 0, 0, 0, 0, 0, NULL, NULL, NULL, NULL, NULL, dv);
  j.ist.n_filters_per_rank = n_filters;
  j.ist.m_states_per_filter = m;
  grid_st grid;
  memset(&grid, 0, sizeof grid);
  grid.nx = nx;
  grid.ny = ny;
  grid.nz = nz;
  grid.ngrid = nx * ny * nz;
  grid.dv = dv;
  zomplex *psi = calloc(j.ist.nspinngrid, sizeof(zomplex));
  init_filter_states(psi_rank, psi, &grid, &seed, &j.ist, &j.par, &j.flag, &j.pl);
  free(psi);
  job_free(&j);
  return seed;
}

void set_ene_targets(double *ene_targets, index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);

/* set_ene_targets (init.c:401-478) with setTargets = 1 (n_vb valence and
 * m - n_vb conduction targets); writes ene_targets.dat into the working
 * directory */
void ref_ene_targets(long m, long n_vb, double vbmin, double vbmax, double cbmin, double cbmax, double *targets)
{
  index_st ist;
  par_st par;
  flag_st flag;
  parallel_st pl;
  memset(&ist, 0, sizeof ist);
  memset(&par, 0, sizeof par);
  memset(&flag, 0, sizeof flag);
  memset(&pl, 0, sizeof pl);
  ist.m_states_per_filter = m;
  par.n_targets_VB = n_vb;
  par.n_targets_CB = m - n_vb;
  par.VBmin = vbmin;
  par.VBmax = vbmax;
  par.CBmin = cbmin;
  par.CBmax = cbmax;
  flag.setTargets = 1;
  pl.mpi_rank = 1; /* quiet */
  set_ene_targets(targets, &ist, &par, &flag, &pl);
}

void write_cube_file(double *rho, grid_st *grid, char *fileName);
void write_eval_dat(double *eig_vals, double *sigma_E, long n_elems, char *fileName);
void write_psi_dat(double *psitot, long n_elems, char *fileName);

/* write_cube_file (write.c:65-139; atoms from conf.dat in the working
 * directory), write_eval_dat (write.c:263-282) and write_psi_dat
 * (write.c:285-296) into the working directory.  write_psi_dat leaves its
 * stream open, so the data reaches the file at process exit; fflush(NULL)
 * stands in for that exit here. */
void ref_write_outputs(const double *rho, long nx, long ny, long nz, double dx, double dy, double dz, double xmin,
                       double ymin, double zmin, const double *eval, const double *sigma, long n, const double *psi,
                       long n_doubles)
{
  grid_st grid;
  memset(&grid, 0, sizeof grid);
  grid.nx = nx;
  grid.ny = ny;
  grid.nz = nz;
  grid.dx = dx;
  grid.dy = dy;
  grid.dz = dz;
  grid.xmin = xmin;
  grid.ymin = ymin;
  grid.zmin = zmin;
  write_cube_file((double *)rho, &grid, "ref.cube");
  write_eval_dat((double *)eval, (double *)sigma, n, "ref_eval.dat");
  write_psi_dat((double *)psi, n_doubles, "ref_psi.dat");
  fflush(NULL);
}

void read_input(flag_st *flag, grid_st *grid, index_st *ist, par_st *par, parallel_st *parallel);

/* read_input (read.c:5-995) at a non-zero rank of one (so that it prints no
 * job state) on input.par and conf.par in the working directory.  d[10]: dx,
 * dy, dz, VBmin, VBmax, CBmin, CBmax, KE_max, fermi_E, sigma_E_cut.  l[31]:
 * nx, ny, nz, m_states_per_filter, n_filter_cycles, ncheby, setTargets,
 * n_targets_VB, n_targets_CB, setSeed, rand_seed, useSpinors, SO, NL,
 * getAllStates, approxEnergyRange, printPsiFilt, printPsiDiag,
 * calcFilterOnly, restartFromOrtho, restartFromSigma, n_states_for_ortho,
 * n_states_for_sigma, printCubes, ncubes, readCoeffs, inputPsiFilt,
 * init_psi_start, init_psi_end, calcSpinAngStat, isComplex. */
void ref_read_input(double *d, long *l)
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
  pl.mpi_rank = 1;
  pl.mpi_size = 1;
  pl.nthreads = 1;
  read_input(&flag, &grid, &ist, &par, &pl);
  const double dv[10] = {grid.dx, grid.dy, grid.dz, par.VBmin, par.VBmax, par.CBmin, par.CBmax, par.KE_max,
                         par.fermi_E, par.sigma_E_cut};
  const long lv[31] = {grid.nx, grid.ny, grid.nz, ist.m_states_per_filter, ist.n_filter_cycles, ist.ncheby,
                       flag.setTargets, par.n_targets_VB, par.n_targets_CB, flag.setSeed, par.rand_seed,
                       flag.useSpinors, flag.SO, flag.NL, flag.getAllStates, flag.approxEnergyRange,
                       flag.printPsiFilt, flag.printPsiDiag, flag.calcFilterOnly, flag.restartFromOrtho,
                       flag.restartFromSigma, ist.n_states_for_ortho, ist.n_states_for_sigma, flag.printCubes,
                       ist.ncubes, flag.readCoeffs, flag.inputPsiFilt, ist.init_psi_start, ist.init_psi_end,
                       flag.calcSpinAngStat, flag.isComplex};
  memcpy(d, dv, sizeof dv);
  memcpy(l, lv, sizeof lv);
}

void save_output(char *file_name, double *psitot, double *eig_vals, double *sigma_E, xyz_st *R, grid_st *grid,
                 index_st *ist, par_st *par, flag_st *flag, parallel_st *parallel);

/* save_output (save.c:446-503) into ref_output.dat after read_conf,
 * init_grid_params and the axes of build_grid_ksqr (init.c:259-290) on
 * conf.par in the working directory, for n states of psitot with their
 * eigenvalues and variances.  Returns 0 or -1. */
int ref_save_output(double dgrid, const long *n_in, double ke_max, double fermi_e, int so, int nl, long n,
                    double *eval, double *sigma, double *psitot)
{
  FILE *pf = fopen("conf.par", "r");
  long nat = 0;
  if (!pf || fscanf(pf, "%ld", &nat) != 1) {
    if (pf) fclose(pf);
    return -1;
  }
  fclose(pf);
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
  ist.n_max_atom_types = N_MAX_ATOM_TYPES;
  ist.atom_types = calloc(N_MAX_ATOM_TYPES, sizeof(long));
  ist.natoms = nat;
  flag.centerConf = 1;
  flag.SO = so;
  flag.NL = nl;
  flag.useSpinors = so;
  flag.isComplex = so;
  ist.nspin = so ? 2 : 1;
  ist.complex_idx = so ? 2 : 1;
  ist.mn_states_tot = n;
  par.KE_max = ke_max;
  par.fermi_E = fermi_e;
  pl.nthreads = 1;
  pl.mpi_rank = 1;
  grid.nx = n_in[0];
  grid.ny = n_in[1];
  grid.nz = n_in[2];
  grid.dx = grid.dy = grid.dz = dgrid;
  xyz_st *R = calloc(nat, sizeof(xyz_st));
  atom_info *atom = calloc(nat, sizeof(atom_info));
  read_conf(R, atom, &ist, &par, &flag, &pl);
  init_grid_params(&grid, R, &ist, &par, &flag, &pl);
  grid.x = calloc(grid.nx, sizeof(double));
  grid.y = calloc(grid.ny, sizeof(double));
  grid.z = calloc(grid.nz, sizeof(double));
  double *ksqr = calloc(grid.ngrid, sizeof(double));
  build_grid_ksqr(ksqr, R, &grid, &ist, &par, &flag, &pl);
  save_output("ref_output.dat", psitot, eval, sigma, R, &grid, &ist, &par, &flag, &pl);
  free(ksqr);
  free(grid.x);
  free(grid.y);
  free(grid.z);
  free(R);
  free(atom);
  free(ist.atom_types);
  return 0;
}
