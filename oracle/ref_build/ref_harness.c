/* Test-only harness linked into oracle/_ref/libfbse_ref.so.
 *
 * The reference's hot-path C files are compiled from where they lie (never
 * copied) against type-only stand-in headers.  Their only call into an absent
 * library is FFTW's fftw_execute inside kinetic() (hamiltonian.c:62-99); the
 * oracle never calls kinetic() through this library, so the symbol resolves to
 * a stub that aborts loudly if it is ever reached. */
#include <stdio.h>
#include <stdlib.h>
#include "fftw3.h"

void fftw_execute(const fftw_plan p)
{
  (void)p;
  fprintf(stderr, "oracle/_ref: fftw_execute is not available in the reference subset\n");
  abort();
}

/* ------------------------------------------------------------------------
 * Plain-argument wrappers around the reference's functions, so the tests
 * can call them through ctypes without mirroring the reference's structs.
 * ------------------------------------------------------------------------ */
#include <string.h>
#include "fd.h"
#include "hamiltonian.h"

double samp_points_ashkenazy(zomplex *point, double min, double max, long ncheby);
void gen_newton_coeff(zomplex *an, double *samp, double *ene_targets, index_st *ist, par_st *par, parallel_st *parallel);

double ref_ran(long *seed) { return ran_nrc(seed); }

double ref_samp_points(long ncheby, double *re, double *im)
{
  zomplex *p = calloc(ncheby, sizeof(zomplex));
  double fk = samp_points_ashkenazy(p, -2.0, 2.0, ncheby);
  for (long j = 0; j < ncheby; j++) { re[j] = p[j].re; im[j] = p[j].im; }
  free(p);
  return fk;
}

/* gen_newton_coeff writes zn.dat, coeff-*.dat and func.dat into the cwd. */
void ref_newton_coeff(long ncheby, long m, double vmin, double de, double dt, double *samp, double *targets,
                      double *an)
{
  index_st ist;
  par_st par;
  parallel_st par2;
  memset(&ist, 0, sizeof ist);
  memset(&par, 0, sizeof par);
  memset(&par2, 0, sizeof par2);
  ist.ncheby = ncheby;
  ist.m_states_per_filter = m;
  par.Vmin = vmin;
  par.dE = de;
  par.dE_1 = 4.0 / de;
  par.dt = dt;
  par.ham_threads = 1;
  par2.k_rank = 1; /* silence the width report */
  gen_newton_coeff((zomplex *)an, samp, targets, &ist, &par, &par2);
}

void ref_def_LS(double *ls)
{
  index_st ist;
  par_st par;
  memset(&ist, 0, sizeof ist);
  memset(&par, 0, sizeof par);
  ist.n_s_ang_mom = 2;
  ist.n_l_ang_mom = 3;
  ist.n_j_ang_mom = 6;
  memset(ls, 0, 72 * sizeof(double));
  def_LS((zomplex *)ls, &ist, &par);
}

/* p_potential (SO + NL + local) on one state; psi/out are zomplex arrays of
 * nspin*ngrid; the projector table comes in the oracle's SoA layout. */
void ref_p_potential(double *out, double *psi, double *pot2, double *ls, long ngrid, int nspin, int is_complex,
                     int so, int nl, long nat, long npts, long nproj, long *nlcnt, int *jxyz, double *y1,
                     double *proj, double *nlp, int *sgn, double dv)
{
  index_st ist;
  par_st par;
  flag_st flag;
  memset(&ist, 0, sizeof ist);
  memset(&par, 0, sizeof par);
  memset(&flag, 0, sizeof flag);
  ist.ngrid = ngrid;
  ist.nspin = nspin;
  ist.nspinngrid = nspin * ngrid;
  ist.n_NL_atoms = nat;
  ist.n_NL_gridpts = npts;
  ist.nproj = nproj;
  ist.n_s_ang_mom = 2;
  ist.n_l_ang_mom = 3;
  ist.n_j_ang_mom = 6;
  par.dv = dv;
  flag.SO = so;
  flag.NL = nl;
  flag.isComplex = is_complex;
  nlc_st *nlc = calloc(nat * npts > 0 ? nat * npts : 1, sizeof(nlc_st));
  for (long a = 0; a < nat; a++)
    for (long g = 0; g < npts; g++) {
      long e = a * npts + g;
      nlc[e].jxyz = jxyz[e];
      for (int m = 0; m < 3; m++) { nlc[e].y1[m].re = y1[e * 6 + 2 * m]; nlc[e].y1[m].im = y1[e * 6 + 2 * m + 1]; }
      for (long p = 0; p < nproj; p++) {
        nlc[e].proj[p] = proj[e * nproj + p];
        nlc[e].NL_proj[p] = nlp[e * nproj + p];
        nlc[e].NL_proj_sign[p] = sgn[a * nproj + p];
      }
    }
  vector k0;
  memset(&k0, 0, sizeof k0);
  p_potential((zomplex *)out, (zomplex *)psi, pot2, (zomplex *)ls, nlc, nlcnt, &ist, &par, &flag, 1, k0);
  free(nlc);
}

void ref_normalize_all(double *psitot, long n, long ngrid, int nspin, int is_complex, double dv)
{
  index_st ist;
  par_st par;
  flag_st flag;
  parallel_st pl;
  memset(&ist, 0, sizeof ist);
  memset(&par, 0, sizeof par);
  memset(&flag, 0, sizeof flag);
  memset(&pl, 0, sizeof pl);
  ist.ngrid = ngrid;
  ist.nspinngrid = nspin * ngrid;
  ist.complex_idx = is_complex ? 2 : 1;
  flag.isComplex = is_complex;
  par.dv = dv;
  pl.k_rank = 1;
  normalize_all(psitot, n, &ist, &par, &flag, &pl);
}
