/* Host-side setup for the drop-in executables (declared in fbse_dropin.h). */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "fbse_dropin.h"

#define FBSE_PI 3.14159265358979323846
#define FBSE_EPSDX 1.0e-20 /* EPSDX, filter_mpi/fd.h */

static void seterr(char *err, size_t n, const char *msg, const char *what)
{
  if (err && n) snprintf(err, n, "%s%s%s", msg, what ? ": " : "", what ? what : "");
}

/* ---------------------------------------------------------------------------
 * input.par: "key = value" pairs; a few keys take extra values on the same
 * line (setTargets 1 nVB nCB, setSeed 1 seed, getAllStates 0 sigmaECut),
 * read as the reference reads them (fscanf after the pair, read.c:405-439).
 * ------------------------------------------------------------------------- */
static int parse_long(const char *s, long *v)
{
  char *e;
  *v = strtol(s, &e, 10);
  return *e == '\0' ? 0 : -1;
}
static int parse_double(const char *s, double *v)
{
  char *e;
  *v = strtod(s, &e);
  return *e == '\0' ? 0 : -1;
}

/* keys that only steer threading, printing or checkpoints of the reference:
 * accepted and ignored.  saveCheckpoints among them: the reference's
 * checkpoint_<id>.dat reader (filter_mpi/save.c:389) takes three of the
 * five flags its writer puts on that line (save.c:283), so its checkpoints do
 * not restart; the file-level restarts (restartFromOrtho from psi-filt.dat,
 * restartFromSigma from psi-diag.dat) are implemented instead. */
static const char *k_ignored[] = {"nThreads", "hamThreads", "nestedOMP", "useFastHam", "useMPIOMP", "MPIOrtho",
                                  "MPIDiag", "parallelSigma", "timeHamiltonian", "printNorm",
                                  "printGaussCubes", "saveCheckpoints", "printPsiOrtho",
                                  "fftWisdomDir", "saveOutput", "calcPotOverlap",
                                  "retryFilter", "centerConf", "noTimeRev", "psiZeroCut",
                                  "calcDarkStates", "timingSpecs", "crystalStructure", "outmostMaterial", NULL};
/* keys whose non-zero value selects a path this library does not implement */
static const char *k_unsupported[] = {"periodic", "useStrain", "longRange", "localStructureDependent",
                                      "useGaussianBasis", "readProj",
                                      "restartFromCheckpoint", "interpolatePot", NULL};

static int in_list(const char *k, const char **l)
{
  for (int i = 0; l[i]; i++)
    if (!strcmp(k, l[i])) return 1;
  return 0;
}

int fbse_read_filter_params(const char *path, fbse_filter_params *p, char *err, size_t errlen)
{
  memset(p, 0, sizeof(*p));
  p->ke_max = 20.0;      /* read.c:32 */
  p->fermi_e = -0.18;    /* read.c:87 */
  p->sigma_e_cut = 0.01; /* read.c:89 */
  p->get_all_states = 1; /* read.c:85 */
  p->print_psi_filt = 1; /* read.c:34 */
  p->precision = 0;
  FILE *f = fopen(path, "r");
  if (!f) { seterr(err, errlen, "cannot open", path); return -1; }
  char key[1000], val[1000];
  int rc = 0, count = 0;
  while (rc == 0 && count < 100 && fscanf(f, "%999s = %999s", key, val) == 2) {
    long lv = 0;
    double dv = 0;
    count++;
    if (!strcmp(key, "nx")) rc = parse_long(val, &p->nx);
    else if (!strcmp(key, "ny")) rc = parse_long(val, &p->ny);
    else if (!strcmp(key, "nz")) rc = parse_long(val, &p->nz);
    else if (!strcmp(key, "dGrid")) { rc = parse_double(val, &p->dx); p->dy = p->dz = p->dx; }
    else if (!strcmp(key, "dx")) rc = parse_double(val, &p->dx);
    else if (!strcmp(key, "dy")) rc = parse_double(val, &p->dy);
    else if (!strcmp(key, "dz")) rc = parse_double(val, &p->dz);
    else if (!strcmp(key, "mStatesPerFilter")) rc = parse_long(val, &p->m_states_per_filter);
    else if (!strcmp(key, "nFilterCycles")) rc = parse_long(val, &p->n_filter_cycles);
    else if (!strcmp(key, "nCheby")) rc = parse_long(val, &p->ncheby);
    else if (!strcmp(key, "VBmin")) rc = parse_double(val, &p->vbmin);
    else if (!strcmp(key, "VBmax")) rc = parse_double(val, &p->vbmax);
    else if (!strcmp(key, "CBmin")) rc = parse_double(val, &p->cbmin);
    else if (!strcmp(key, "CBmax")) rc = parse_double(val, &p->cbmax);
    else if (!strcmp(key, "KEmax")) rc = parse_double(val, &p->ke_max);
    else if (!strcmp(key, "fermiEnergy")) rc = parse_double(val, &p->fermi_e);
    else if (!strcmp(key, "sigmaECut")) rc = parse_double(val, &p->sigma_e_cut);
    else if (!strcmp(key, "setTargets")) {
      rc = parse_long(val, &lv);
      p->set_targets = (int)lv;
      if (!rc && lv == 1 && fscanf(f, "%ld %ld", &p->n_targets_vb, &p->n_targets_cb) != 2) rc = -1;
    } else if (!strcmp(key, "setSeed")) {
      rc = parse_long(val, &lv);
      p->set_seed = (int)lv;
      if (!rc && lv == 1 && fscanf(f, "%ld", &p->seed) != 1) rc = -1;
    } else if (!strcmp(key, "getAllStates")) {
      rc = parse_long(val, &lv);
      p->get_all_states = (int)lv;
      if (!rc && lv == 0 && fscanf(f, "%lg", &p->sigma_e_cut) != 1) rc = -1;
    } else if (!strcmp(key, "useSpinors")) { rc = parse_long(val, &lv); p->use_spinors = (int)lv; }
    else if (!strcmp(key, "spinOrbit")) { rc = parse_long(val, &lv); p->so = (int)lv; }
    else if (!strcmp(key, "NonLocal")) { rc = parse_long(val, &lv); p->nl = (int)lv; }
    else if (!strcmp(key, "approxEnergyRange")) { rc = parse_long(val, &lv); p->approx_energy_range = (int)lv; }
    else if (!strcmp(key, "mixedPrecision")) { rc = parse_long(val, &lv); p->precision = lv ? 1 : 0; }
    else if (!strcmp(key, "printPsiFilt")) { rc = parse_long(val, &lv); p->print_psi_filt = (int)lv; }
    else if (!strcmp(key, "readCoeffs")) { rc = parse_long(val, &lv); p->read_coeffs = (int)lv; }
    else if (!strcmp(key, "inputPsiFilt")) {
      /* "inputPsiFilt = 1 <start> <end>" (read.c:440-451) */
      rc = parse_long(val, &lv);
      p->input_psi_filt = (int)lv;
      if (!rc && lv == 1 && (fscanf(f, "%ld %ld", &p->init_psi_start, &p->init_psi_end) != 2 ||
                             p->init_psi_start < 0 || p->init_psi_end <= p->init_psi_start))
        rc = -1;
    }
    else if (!strcmp(key, "printPsiDiag")) { rc = parse_long(val, &lv); p->print_psi_diag = (int)lv; }
    else if (!strcmp(key, "calcSpinAngStat")) { rc = parse_long(val, &lv); p->calc_spin_ang_stat = (int)lv; }
    else if (!strcmp(key, "calcFilterOnly")) { rc = parse_long(val, &lv); p->calc_filter_only = (int)lv; }
    else if (!strcmp(key, "restartFromOrtho")) {
      /* "restartFromOrtho = 1 <states in psi-filt.dat>" (read.c:762-773) */
      rc = parse_long(val, &lv);
      p->restart_from_ortho = (int)lv;
      if (!rc && lv == 1 && (fscanf(f, "%ld", &p->n_states_for_ortho) != 1 || p->n_states_for_ortho < 1)) rc = -1;
    } else if (!strcmp(key, "restartFromSigma")) {
      /* "restartFromSigma = 1 <states in psi-diag.dat>" (read.c:775-786) */
      rc = parse_long(val, &lv);
      p->restart_from_sigma = (int)lv;
      if (!rc && lv == 1 && (fscanf(f, "%ld", &p->n_states_for_sigma) != 1 || p->n_states_for_sigma < 1)) rc = -1;
    } else if (in_list(key, k_unsupported)) {
      if (parse_double(val, &dv) == 0 && dv != 0.0) {
        seterr(err, errlen, "input.par key not supported by this library (set it to 0)", key);
        fclose(f);
        return -1;
      }
    } else if (!strcmp(key, "printCubes")) {
      /* "printCubes = 1 <states per side>" (read.c:691-715) */
      rc = parse_long(val, &lv);
      p->print_cubes = (int)lv;
      if (!rc && lv == 1 && (fscanf(f, "%ld", &p->ncubes) != 1 || p->ncubes < 0)) rc = -1;
    } else if (in_list(key, k_ignored)) {
    } else {
      seterr(err, errlen, "unknown input.par key", key);
      fclose(f);
      return -1;
    }
    if (rc) seterr(err, errlen, "cannot convert the value of", key);
  }
  fclose(f);
  if (rc) return -1;
  if (p->so) p->use_spinors = 1; /* read.c:897-900 */
  if (p->dx <= 0 || p->dy <= 0 || p->dz <= 0) { seterr(err, errlen, "grid spacing missing", "dGrid"); return -1; }
  if (p->m_states_per_filter < 2 || p->n_filter_cycles < 1 || p->ncheby < 2) {
    seterr(err, errlen, "mStatesPerFilter, nFilterCycles and nCheby must be set", NULL);
    return -1;
  }
  if (p->set_targets != 1) { /* set_ene_targets, init.c:420-424 */
    p->n_targets_cb = p->m_states_per_filter / 2;
    p->n_targets_vb = p->m_states_per_filter - p->n_targets_cb;
  }
  if (p->n_targets_vb + p->n_targets_cb != p->m_states_per_filter || p->n_targets_vb < 1 || p->n_targets_cb < 1) {
    seterr(err, errlen, "n_targets_VB + n_targets_CB must equal mStatesPerFilter, at least one of each", NULL);
    return -1;
  }
  return 0;
}

int fbse_read_bse_params(const char *path, fbse_bse_params *p, char *err, size_t errlen)
{
  memset(p, 0, sizeof(*p));
  /* the defaults of bse_cplx/read.c:38-63; the dielectric constants have
   * none there (zero, which leaves the screened interaction unusable), so
   * they default to vacuum here */
  p->max_hole_states = -1;
  p->max_elec_states = -1;
  p->sigma_e_cut = 0.0001;
  p->eps_x = p->eps_y = p->eps_z = 1.0;
  p->fermi_e = -0.18;
  p->calc_spin_ang_stat = 1;
  FILE *f = fopen(path, "r");
  if (!f) { seterr(err, errlen, "cannot open", path); return -1; }
  char key[1000], val[1000];
  int rc = 0, count = 0;
  while (rc == 0 && count < 100 && fscanf(f, "%999s = %999s", key, val) == 2) {
    long lv = 0;
    double dv = 0;
    count++;
    if (!strcmp(key, "maxHoleStates")) rc = parse_long(val, &p->max_hole_states);
    else if (!strcmp(key, "maxElecStates")) rc = parse_long(val, &p->max_elec_states);
    else if (!strcmp(key, "sigmaECut")) rc = parse_double(val, &p->sigma_e_cut);
    else if (!strcmp(key, "epsX")) rc = parse_double(val, &p->eps_x);
    else if (!strcmp(key, "epsY")) rc = parse_double(val, &p->eps_y);
    else if (!strcmp(key, "epsZ")) rc = parse_double(val, &p->eps_z);
    else if (!strcmp(key, "fermiEnergy")) rc = parse_double(val, &p->fermi_e);
    else if (!strcmp(key, "deltaEhole")) rc = parse_double(val, &p->delta_e_hole);
    else if (!strcmp(key, "deltaEelec")) rc = parse_double(val, &p->delta_e_elec);
    else if (!strcmp(key, "mixedPrecision")) { rc = parse_long(val, &lv); p->precision = lv ? 1 : 0; }
    else if (!strcmp(key, "coulombDone")) { rc = parse_long(val, &lv); p->coulomb_done = (int)lv; }
    else if (!strcmp(key, "restartCoulomb")) { rc = parse_long(val, &lv); p->restart_coulomb = (int)lv; }
    else if (!strcmp(key, "calcCoulombOnly")) { rc = parse_long(val, &lv); p->calc_coulomb_only = (int)lv; }
    else if (!strcmp(key, "calcSpinAngStat")) { rc = parse_long(val, &lv); p->calc_spin_ang_stat = (int)lv; }
    else if (!strcmp(key, "spinOrbit") || !strcmp(key, "NonLocal") || !strcmp(key, "KEmax")) {
      rc = parse_double(val, &dv); /* carried by output.dat; the value here is not used */
    } else if (in_list(key, k_ignored)) {
    } else {
      seterr(err, errlen, "unknown input.par key", key);
      fclose(f);
      return -1;
    }
    if (rc) seterr(err, errlen, "cannot convert the value of", key);
  }
  fclose(f);
  return rc ? -1 : 0;
}

/* ---------------------------------------------------------------------------
 * conf.par and tables
 * ------------------------------------------------------------------------- */
int fbse_read_conf(const char *path, long *natoms, double **xyz, int **types, char names[][8], int *ntypes,
                   char *err, size_t errlen)
{
  FILE *f = fopen(path, "r");
  if (!f) { seterr(err, errlen, "cannot open", path); return -1; }
  long n = 0;
  if (fscanf(f, "%ld", &n) != 1 || n < 1) { fclose(f); seterr(err, errlen, "bad atom count in", path); return -1; }
  double *x = malloc(3 * n * sizeof(double));
  int *t = malloc(n * sizeof(int));
  *ntypes = 0;
  double c[3] = {0, 0, 0};
  for (long i = 0; i < n; i++) {
    char nm[64];
    if (fscanf(f, "%63s %lf %lf %lf", nm, &x[3 * i], &x[3 * i + 1], &x[3 * i + 2]) != 4 || strlen(nm) > 7) {
      fclose(f);
      free(x);
      free(t);
      seterr(err, errlen, "bad atom line in", path);
      return -1;
    }
    int k;
    for (k = 0; k < *ntypes; k++)
      if (!strcmp(names[k], nm)) break;
    if (k == *ntypes) {
      if (*ntypes == FBSE_MAX_TYPES) { fclose(f); free(x); free(t); seterr(err, errlen, "too many atom types", NULL); return -1; }
      strcpy(names[k], nm);
      (*ntypes)++;
    }
    t[i] = k;
    for (int a = 0; a < 3; a++) c[a] += x[3 * i + a];
  }
  fclose(f);
  /* centerConf (read.c:1135-1148): shift the centre of the atoms to the origin */
  for (int a = 0; a < 3; a++) c[a] /= (double)n;
  for (long i = 0; i < n; i++)
    for (int a = 0; a < 3; a++) x[3 * i + a] -= c[a];
  *natoms = n;
  *xyz = x;
  *types = t;
  return 0;
}

void fbse_ene_targets(long m, long n_vb, double vbmin, double vbmax, double cbmin, double cbmax, double *targets)
{ /* set_ene_targets (filter_mpi/init.c:438-455): n_vb targets spaced down from
   * VBmax (VBmax included), the other m - n_vb spaced up from CBmin */
  const long n_cb = m - n_vb;
  double del = (vbmax - vbmin) / (double)n_vb;
  for (long j = 0; j < n_vb; j++) targets[n_vb - j - 1] = vbmax - (double)j * del;
  del = (cbmax - cbmin) / (double)n_cb;
  for (long j = n_vb; j < m; j++) targets[j] = cbmin + (double)(j - n_vb) * del;
}

long fbse_qp_basis(const double *eval, const double *sigma, long n, double sigma_cut, double fermi_e,
                   long max_holes, long max_elecs, long *sel, long *n_holes, long *n_elecs)
{ /* get_qp_basis_indices (bse_cplx/basis.c:7-254): the converged states
   * (sigma < cut) below and above the Fermi energy, in eval.dat order; with a
   * maximum, the holes nearest the gap and the first electrons */
  long nh = 0, ne = 0;
  for (long i = 0; i < n; i++)
    if (sigma[i] < sigma_cut && eval[i] < fermi_e) nh++;
  long h = 0, e = 0;
  const long h0 = (max_holes != -1 && nh > max_holes) ? nh - max_holes : 0;
  const long nh_keep = nh - h0;
  for (long i = 0; i < n; i++) {
    if (sigma[i] < sigma_cut && eval[i] < fermi_e) {
      if (h >= h0) sel[h - h0] = i;
      h++;
    }
    if (sigma[i] < sigma_cut && eval[i] > fermi_e) {
      if (max_elecs == -1 || e < max_elecs) sel[nh_keep + e] = i;
      e++;
    }
  }
  ne = (max_elecs != -1 && e > max_elecs) ? max_elecs : e;
  *n_holes = nh_keep;
  *n_elecs = ne;
  return nh_keep + ne;
}

int fbse_is_ligand(const char *t)
{ /* the ligand labels of read_pot's SO loop (filter_mpi/read.c:1739-1746) */
  static const char *lig[] = {"P1", "P2", "P3", "P4", "PC5", "PC6", "PR1", "PR2", "PR3",
                              "PA1", "PA2", "PA3", "C1", "C2", "C3", NULL};
  for (int i = 0; lig[i]; i++)
    if (!strcmp(t, lig[i])) return 1;
  return 0;
}

int fbse_read_so_params(const char *atyp, double *so_par, double *nl_par, char *err, size_t errlen)
{ /* SO_<Atm>.par (filter_mpi/read.c:1732-1782): SO_par, NL_par[0], NL_par[1],
   * the first value of each of the first three lines */
  char path[64];
  snprintf(path, sizeof path, "SO_%s.par", atyp);
  FILE *f = fopen(path, "r");
  if (!f) { seterr(err, errlen, "No SO(+NL) pot found in", path); return -1; }
  const int ok = fscanf(f, "%lg %*g", so_par) == 1 && fscanf(f, "%lg %*g", &nl_par[0]) == 1 &&
                 fscanf(f, "%lg %*g", &nl_par[1]) == 1;
  fclose(f);
  if (!ok) { seterr(err, errlen, "cannot read", path); return -1; }
  return 0;
}

long fbse_read_table(const char *path, double **r, double **v)
{
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  long cap = 1024, n = 0;
  double *a = malloc(cap * sizeof(double)), *b = malloc(cap * sizeof(double));
  double x, y;
  while (fscanf(f, "%lf %lf", &x, &y) == 2) {
    if (n == cap) {
      cap *= 2;
      a = realloc(a, cap * sizeof(double));
      b = realloc(b, cap * sizeof(double));
    }
    a[n] = x;
    b[n] = y;
    n++;
  }
  fclose(f);
  *r = a;
  *v = b;
  return n;
}

/* ---------------------------------------------------------------------------
 * grid
 * ------------------------------------------------------------------------- */
void fbse_grid_rule(const double *xyz, long natoms, double d, long n_in, int axis, long *n, double *xmin)
{
  /* init_grid_params (init.c:5-255): the largest coordinate separation sets a
   * half-width xd = nint(ext/2 + 5); the axis grows to cover [-xd, xd - d]
   * (made even) when that exceeds the requested size; box = n d (even n) or
   * (n - 1) d (odd n) centred on the origin */
  double ext = 0.0;
  for (long i = 0; i < natoms; i++)
    for (long j = 0; j < natoms; j++) {
      const double s = fabs(xyz[3 * i + axis] - xyz[3 * j + axis]);
      if (s > ext) ext = s;
    }
  const double xd = rint(0.5 * ext + 5.0);
  const long ntmp = (long)(((xd - d) - (-xd)) / d);
  long nn = n_in;
  if (ntmp > nn) nn = ntmp + (ntmp % 2);
  const double box = (nn % 2 == 0) ? (double)nn * d : (double)(nn - 1) * d;
  *n = nn;
  *xmin = -box / 2.0;
}

void fbse_grid_axis(long n, double lo, double d, double *out)
{
  double v = lo;
  for (long j = 0; j < n; j++) {
    out[j] = v;
    v += d;
  }
}

double fbse_r_nlcut2(double dx) { return 1.5 + 6.0 * log(10.0) + 3.0 * dx; }

/* The extreme single-channel eigenvalues of the NL (KB) operator: each
 * (atom, projector, m) channel sgn dv |b Y_1m><b Y_1m| has eigenvalue
 * sgn dv sum_points b^2 |Y_1m|^2; lam_min / lam_max are the most negative /
 * most positive of them, 0 when none is (init.c:1095-1130). */
void fbse_nl_bounds(long nat, long npts, int nproj, const long *nl, const double *y1, const double *nlp,
                    const int *sgn, double dv, double *lam_min, double *lam_max)
{
  double lo = 0.0, hi = 0.0;
  for (long a = 0; a < nat; a++)
    for (int q = 0; q < nproj; q++) {
      double gm[3] = {0.0, 0.0, 0.0};
      for (long g = 0; g < nl[a]; g++) {
        const long e = a * npts + g;
        const double b2 = nlp[e * nproj + q] * nlp[e * nproj + q];
        for (int m = 0; m < 3; m++)
          gm[m] += b2 * (y1[e * 6 + 2 * m] * y1[e * 6 + 2 * m] + y1[e * 6 + 2 * m + 1] * y1[e * 6 + 2 * m + 1]);
      }
      for (int m = 0; m < 3; m++) {
        const double l = (double)sgn[a * nproj + q] * dv * gm[m];
        if (l < lo) lo = l;
        if (l > hi) hi = l;
      }
    }
  *lam_min = lo;
  *lam_max = hi;
}

/* The spectrum range rule of get_energy_range (energy.c:302-369).  approx = 1:
 * [-0.8, Vmax + KE_max], + 3.5 on Emax with spin-orbit, and with NL projectors
 * 1.15 lam_max onto Emax and 1.15 lam_min onto Emin (each only with its sign).
 * approx = 0: emin / emax come in as the iterated extremes.  Then the
 * inflation: NL without SO and lam_min < 0: Emax x 1.05, Emin - 0.1 |Emin|,
 * clamped to 1.05 (Vmin_local + lam_min); otherwise Emax x 1.2,
 * Emin - 0.2 |Emin|. */
void fbse_energy_range_rule(int approx, int so, int nl, double vmin_loc, double vmax_loc, double ke_max,
                            double lam_min, double lam_max, double *emin, double *emax)
{
  double lo = *emin, hi = *emax;
  if (approx) {
    lo = -0.8;
    hi = vmax_loc + ke_max;
    if (so) hi += 3.5;
    if (nl) {
      if (lam_max > 0.0) hi += 1.15 * lam_max;
      if (lam_min < 0.0) lo += 1.15 * lam_min;
    }
  }
  if (nl && !so && lam_min < 0.0) {
    hi *= 1.05;
    lo -= 0.1 * fabs(lo);
    const double weyl = 1.05 * (vmin_loc + lam_min);
    if (lo > weyl) lo = weyl;
  } else {
    hi *= 1.2;
    lo -= 0.2 * fabs(lo);
  }
  *emin = lo;
  *emax = hi;
}

/* ---------------------------------------------------------------------------
 * radial projectors (filter_mpi/projectors.c:12-228).  The reference forms
 * the PROJ_LEN x PROJ_LEN matrix
 *   A[i][j] = sum_{r>0} r^2 j1(k_i r) w(r) j1(k_j r) dr
 * (j1 the spherical Bessel function, w the SO Gaussian or the NL profile)
 * and keeps the nproj eigenvectors of largest |eigenvalue|.  Here A is never
 * formed: a block subspace iteration (block 12) with Rayleigh-Ritz steps
 * (Jacobi on the small projected matrix) applies A as J diag(w r^2 dr) J^T.
 * The kernel's spectrum falls off fast, so a handful of iterations reaches
 * round-off.  Eigenvector signs are free; the projectors enter as products.
 * ------------------------------------------------------------------------- */
static double bessel1(double x, double x1) { return (x < 1e-10) ? 0.0 : (sin(x) * (x1 * x1) - cos(x) * x1); }

/* cyclic Jacobi eigen-decomposition of a small symmetric matrix a[n][n]:
 * eigenvalues in w, eigenvectors in the columns of v */
static void jacobi_small(int n, double *a, double *w, double *v)
{
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) v[i * n + j] = (i == j);
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) off += a[p * n + q] * a[p * n + q];
    if (off < 1e-300) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        const double apq = a[p * n + q];
        if (fabs(apq) < 1e-300) continue;
        const double th = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; k++) {
          const double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          const double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; k++) {
          const double vkp = v[k * n + p], vkq = v[k * n + q];
          v[k * n + p] = c * vkp - s * vkq;
          v[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; i++) w[i] = a[i * n + i];
}

int fbse_radial_projectors(double dx, double rcut, int kind, double lam1, double lam2, int nproj, double *out,
                           int *sgn)
{
  const long N = FBSE_PROJ_LEN;
  enum { B = 12 };
  if (nproj < 1 || nproj > B / 2) return -1;
  if (kind == 1 && lam1 == 0.0 && lam2 == 0.0) { /* gen_nlc_projectors: no NL term */
    memset(out, 0, (size_t)nproj * N * sizeof(double));
    for (int p = 0; p < nproj; p++) sgn[p] = 0;
    return 0;
  }
  const double kmax = 1.5 * FBSE_PI / dx, dk = kmax / (double)N, dr = rcut / (double)N;
  double *J = malloc((size_t)N * N * sizeof(double)); /* J[i * N + rp] = j1(k_i r_rp) */
  double *wr = calloc(N, sizeof(double));
  double *X = malloc((size_t)B * N * sizeof(double)), *Y = malloc((size_t)B * N * sizeof(double));
  double *t = malloc(N * sizeof(double));
  if (!J || !wr || !X || !Y || !t) { free(J); free(wr); free(X); free(Y); free(t); return -1; }
  for (long i = 0; i < N; i++) {
    const double ki = (double)i * dk;
    J[i * N] = 0.0;
    for (long rp = 1; rp < N; rp++) {
      const double r = (double)rp * dr;
      J[i * N + rp] = bessel1(ki * r, 1.0 / (ki * r + 1e-10));
    }
  }
  for (long rp = 1; rp < N; rp++) {
    const double r = (double)rp * dr;
    const double w = (kind == 0) ? exp(-((r / 0.7) * (r / 0.7)))
                                 : lam1 * exp(-(r * r)) + lam2 * exp(-((r - 1.5) * (r - 1.5)));
    wr[rp] = r * r * w * dr;
  }
  /* start block: deterministic, well spread */
  uint64_t s = 0x9E3779B97F4A7C15ull;
  for (long i = 0; i < (long)B * N; i++) {
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    X[i] = (double)(s >> 11) / 9007199254740992.0 - 0.5;
  }
  double Hs[B * B], ev[B], V[B * B];
  for (int it = 0; it < 60; it++) {
    /* Y = A X */
    for (int b = 0; b < B; b++) {
      const double *x = X + (long)b * N;
      for (long rp = 0; rp < N; rp++) t[rp] = 0.0;
      for (long i = 0; i < N; i++) {
        const double xi = x[i];
        const double *Ji = J + i * N;
        for (long rp = 1; rp < N; rp++) t[rp] += Ji[rp] * xi;
      }
      for (long rp = 0; rp < N; rp++) t[rp] *= wr[rp];
      double *y = Y + (long)b * N;
      for (long i = 0; i < N; i++) {
        const double *Ji = J + i * N;
        double acc = 0.0;
        for (long rp = 1; rp < N; rp++) acc += Ji[rp] * t[rp];
        y[i] = acc;
      }
    }
    /* orthonormalise Y (modified Gram-Schmidt, twice) into X */
    for (int pass = 0; pass < 2; pass++)
      for (int b = 0; b < B; b++) {
        double *y = Y + (long)b * N;
        for (int c = 0; c < b; c++) {
          const double *z = Y + (long)c * N;
          double d = 0;
          for (long i = 0; i < N; i++) d += z[i] * y[i];
          for (long i = 0; i < N; i++) y[i] -= d * z[i];
        }
        double nrm = 0;
        for (long i = 0; i < N; i++) nrm += y[i] * y[i];
        nrm = sqrt(nrm);
        if (nrm == 0) nrm = 1;
        for (long i = 0; i < N; i++) y[i] /= nrm;
      }
    memcpy(X, Y, (size_t)B * N * sizeof(double));
    /* Rayleigh-Ritz: Hs = X^T A X */
    for (int b = 0; b < B; b++) {
      const double *x = X + (long)b * N;
      for (long rp = 0; rp < N; rp++) t[rp] = 0.0;
      for (long i = 0; i < N; i++) {
        const double *Ji = J + i * N;
        for (long rp = 1; rp < N; rp++) t[rp] += Ji[rp] * x[i];
      }
      for (long rp = 0; rp < N; rp++) t[rp] *= wr[rp];
      double *y = Y + (long)b * N;
      for (long i = 0; i < N; i++) {
        const double *Ji = J + i * N;
        double acc = 0.0;
        for (long rp = 1; rp < N; rp++) acc += Ji[rp] * t[rp];
        y[i] = acc;
      }
    }
    for (int a = 0; a < B; a++)
      for (int b = 0; b < B; b++) {
        double d = 0;
        for (long i = 0; i < N; i++) d += X[(long)a * N + i] * Y[(long)b * N + i];
        Hs[a * B + b] = d;
      }
    for (int a = 0; a < B; a++)
      for (int b = a + 1; b < B; b++) Hs[a * B + b] = Hs[b * B + a] = 0.5 * (Hs[a * B + b] + Hs[b * B + a]);
    jacobi_small(B, Hs, ev, V);
    /* rotate X to the Ritz vectors, and Y (= A X) with it for the residuals */
    double *Z = malloc((size_t)B * N * sizeof(double)), *AZ = malloc((size_t)B * N * sizeof(double));
    for (int b = 0; b < B; b++)
      for (long i = 0; i < N; i++) {
        double z = 0, az = 0;
        for (int a = 0; a < B; a++) {
          z += X[(long)a * N + i] * V[a * B + b];
          az += Y[(long)a * N + i] * V[a * B + b];
        }
        Z[(long)b * N + i] = z;
        AZ[(long)b * N + i] = az;
      }
    memcpy(X, Z, (size_t)B * N * sizeof(double));
    /* order by |eigenvalue| (the selection of projectors.c:166-186), check the
     * residuals of the wanted ones */
    int idx[B];
    for (int b = 0; b < B; b++) idx[b] = b;
    for (int a = 0; a < B; a++)
      for (int b = a + 1; b < B; b++)
        if (fabs(ev[idx[b]]) > fabs(ev[idx[a]])) { int tmp = idx[a]; idx[a] = idx[b]; idx[b] = tmp; }
    double worst = 0, scale = fabs(ev[idx[0]]) > 0 ? fabs(ev[idx[0]]) : 1.0;
    for (int p = 0; p < nproj; p++) {
      const int b = idx[p];
      double r2 = 0;
      for (long i = 0; i < N; i++) {
        const double rres = AZ[(long)b * N + i] - ev[b] * Z[(long)b * N + i];
        r2 += rres * rres;
      }
      if (sqrt(r2) / scale > worst) worst = sqrt(r2) / scale;
    }
    if (worst < 1e-13 || it == 59) {
      /* radial functions (projectors.c:62-78, 197-216) */
      for (int p = 0; p < nproj; p++) {
        const int b = idx[p];
        const double *vec = X + (long)b * N;
        const double pre = (2.00 / FBSE_PI) * sqrt(fabs(ev[b]));
        if (sgn) sgn[p] = ev[b] < 0 ? -1 : 1;
        for (long rp = 0; rp < N; rp++) {
          const double r = (double)rp * dr;
          double sum = 0.0;
          for (long kp = 0; kp < N; kp++) {
            const double k = (double)kp * dk;
            sum += k * k * bessel1(k * r, 1 / (k * r + 1e-10)) * vec[kp] * dk;
          }
          out[(long)p * N + rp] = sum * pre;
        }
      }
      free(Z);
      free(AZ);
      break;
    }
    free(Z);
    free(AZ);
  }
  free(J);
  free(wr);
  free(X);
  free(Y);
  free(t);
  return 0;
}

/* ---------------------------------------------------------------------------
 * outputs
 * ------------------------------------------------------------------------- */
int fbse_write_eval(const char *path, const double *eval, const double *sigma, long n)
{
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  for (long i = 0; i < n; i++) fprintf(f, "%ld %.16g %g\n", i, eval[i], sigma[i]); /* write.c:279 */
  fclose(f);
  return 0;
}

/* atomic numbers of the cube files: cube_atom_number's ligand entries
 * (filter_mpi/write.c:7-50), then the element list of assign_atom_number
 * (read.c:2452-2545) */
static long cube_z(const char *s)
{
  static const struct { const char *sym; long z; } tab[] = {
      {"C1", 2},  {"C2", 3},  {"C3", 4},   {"P1", 84},  {"P2", 85},  {"P3", 86},  {"PC5", 87}, {"PC6", 88},
      {"PA1", 3}, {"PA2", 4}, {"I0", 53},  {"I1", 53},  {"Br0", 35}, {"Br1", 35}, {"PA3", 1},  {"PR1", 1},
      {"PR2", 1}, {"PR3", 1}, {"H", 1},    {"C", 6},    {"Si", 14},  {"P", 15},   {"S", 16},   {"Cl", 17},
      {"Zn", 30}, {"Ga", 31}, {"As", 33},  {"Se", 34},  {"Br", 35},  {"Cd", 48},  {"In", 49},  {"Te", 52},
      {"I", 53},  {"Cs", 55}, {"Pb", 82},  {NULL, 0}};
  for (int i = 0; tab[i].sym; i++)
    if (!strcmp(s, tab[i].sym)) return tab[i].z;
  return -1;
}

int fbse_write_cube(const char *path, const double *rho, long nx, long ny, long nz, double dx, double dy, double dz,
                    double xmin, double ymin, double zmin, long natoms, const char *sym8, const double *xyz)
{ /* write_cube_file (filter_mpi/write.c:65-139): x outer, z inner, 6 per line */
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  fprintf(f, "CUBE FILE\n");
  fprintf(f, "OUTER LOOP: X, MIDDLE LOOP: Y, INNER LOOP: Z\n");
  fprintf(f, "%5li%12.6f%12.6f%12.6f\n", natoms, xmin, ymin, zmin);
  fprintf(f, "%5li%12.6f%12.6f%12.6f\n", nx, dx, 0.0, 0.0);
  fprintf(f, "%5li%12.6f%12.6f%12.6f\n", ny, 0.0, dy, 0.0);
  fprintf(f, "%5li%12.6f%12.6f%12.6f\n", nz, 0.0, 0.0, dz);
  for (long a = 0; a < natoms; a++) {
    char s[8];
    memcpy(s, sym8 + 8 * a, 7);
    s[7] = '\0';
    const long z = cube_z(s);
    if (z < 0) { fclose(f); return -1; }
    fprintf(f, "%5li%12.6f%12.6f%12.6f%12.6f\n", z, 0.0, xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]);
  }
  for (long ix = 0; ix < nx; ix++)
    for (long iy = 0; iy < ny; iy++) {
      for (long iz = 0; iz < nz; iz++) {
        fprintf(f, "%.5g ", rho[nx * (ny * iz + iy) + ix]);
        if (iz % 6 == 5) fputc('\n', f);
      }
      fputc('\n', f);
    }
  fclose(f);
  return 0;
}

/* direct-<rank>.dat / exchange-<rank>.dat (bse_cplx/coulomb.c:289-371,
 * 534-602; one rank): "a b i j ibs jbs re im" per element.  direct: every
 * (a, b, i, j) in a, b, i, j order, zero above the diagonal (coulomb.c:360-371);
 * exchange: (a, i, b, j) order, lower triangle only (coulomb.c:586-600).
 * dir / exc: [n_xton][n_xton] as (re, im) pairs; real = 1 prints the real
 * parts alone, as bse_real does. */
static void kernel_line(FILE *f, long a, long b, long i, long j, long ibs, long jbs, const double *v, int real)
{
  if (real) /* bse_real/coulomb.c:352, 583: one value */
    fprintf(f, "%03ld %03ld %03ld %03ld %ld %ld %.12f\n", a, b, i, j, ibs, jbs, v[0]);
  else
    fprintf(f, "%03ld %03ld %03ld %03ld %ld %ld %.12f %.12f\n", a, b, i, j, ibs, jbs, v[0], v[1]);
}

int fbse_write_kernel_files(const double *dir, const double *exc, long nh, long ne, long lumo, int real)
{
  const long nx = nh * ne;
  FILE *f = fopen("direct-0.dat", "w");
  if (!f) return -1;
  for (long a = lumo; a < lumo + ne; a++)
    for (long b = lumo; b < lumo + ne; b++)
      for (long i = 0; i < nh; i++)
        for (long j = 0; j < nh; j++) {
          const long ibs = (a - lumo) * nh + i, jbs = (b - lumo) * nh + j;
          kernel_line(f, a, b, i, j, ibs, jbs, dir + 2 * (ibs * nx + jbs), real);
        }
  fclose(f);
  f = fopen("exchange-0.dat", "w");
  if (!f) return -1;
  for (long a = lumo; a < lumo + ne; a++)
    for (long i = 0; i < nh; i++)
      for (long b = lumo; b < lumo + ne; b++)
        for (long j = 0; j < nh; j++) {
          const long ibs = (a - lumo) * nh + i, jbs = (b - lumo) * nh + j;
          if (ibs < jbs) continue;
          kernel_line(f, a, b, i, j, ibs, jbs, exc + 2 * (ibs * nx + jbs), real);
        }
  return fclose(f) ? -1 : 0;
}

static int write_part(const char *path, const double *m, long n, int part, const char *fmt, int prec)
{
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  for (long i = 0; i < n; i++, fputc('\n', f))
    for (long j = 0; j < n; j++) fprintf(f, fmt, prec, m[2 * (i * n + j) + part]);
  return fclose(f) ? -1 : 0;
}

/* the matrix files of build_h0_mat, build_BSE_mat and bethe_salpeter:
 * h0.dat (mod_bse.c:73-84, "%.6g "), bsRE/bsIM.dat = K^d + K^x
 * (mod_bse.c:126-144), HBSmatRE/IM.dat = h0 - K (bethe-salpeter.c:71-95) and
 * BSEcoeffRE/IM.dat, column j = exciton j (bethe-salpeter.c:115-133), all with
 * PR_LEN = 6 significant digits (bse_cplx/fd.h:131).  dir / exc: the full
 * kernels, coef the eigenvectors, each [n_xton][n_xton] as (re, im) pairs;
 * the files go to the working directory. */
int fbse_write_bse_matrices(const double *dir, const double *exc, const double *coef, const double *eqp, long nh,
                            long ne, long lumo, int real)
{
  const long n = nh * ne;
  const size_t bytes = (size_t)n * n * 2 * sizeof(double);
  double *dm = malloc(bytes), *xm = malloc(bytes);
  const double *cm = coef;
  int rc = 0;
  if (!dm || !xm) { free(dm); free(xm); return -1; }
  memcpy(dm, dir, bytes);
  memcpy(xm, exc, bytes);
  FILE *f = fopen("h0.dat", "w");
  if (!f) { free(dm); free(xm); return -1; }
  for (long i = 0; i < n; i++, fputc('\n', f))
    for (long j = 0; j < n; j++) fprintf(f, "%.6g ", i == j ? eqp[lumo + i / nh] - eqp[i % nh] : 0.0);
  fclose(f);
  for (size_t k = 0; k < (size_t)n * n * 2; k++) dm[k] += xm[k]; /* K = K^d + K^x */
  for (long i = 0; i < n; i++) dm[2 * (i * n + i) + 1] = 0.0;   /* Hermitian diagonal (mod_bse.c:117-121) */
  if (real) {
    /* bse_real: bs.dat, HBSmat.dat, BSEcoeff.dat with row j = exciton j
     * (bse_real/mod_bse.c:124-131, bethe-salpeter.c:78-114) */
    rc |= write_part("bs.dat", dm, n, 0, "%.*g ", 6);
  } else {
    rc |= write_part("bsRE.dat", dm, n, 0, "%.*g ", 6);
    rc |= write_part("bsIM.dat", dm, n, 1, "%.*g ", 6);
  }
  /* H = h0 - K with a real h0, as C evaluates real - complex
   * (bethe-salpeter.c:71-74): real part h0 - Re K, imaginary part -Im K */
  for (long i = 0; i < n; i++)
    for (long j = 0; j < n; j++) {
      const double h0 = i == j ? eqp[lumo + i / nh] - eqp[i % nh] : 0.0;
      dm[2 * (i * n + j)] = h0 - dm[2 * (i * n + j)];
      dm[2 * (i * n + j) + 1] = -dm[2 * (i * n + j) + 1];
    }
  if (real) {
    rc |= write_part("HBSmat.dat", dm, n, 0, "%.*g \t", 6);
    for (long i = 0; i < n; i++) /* transpose */
      for (long j = 0; j < n; j++) xm[2 * (i * n + j)] = cm[2 * (j * n + i)];
    rc |= write_part("BSEcoeff.dat", xm, n, 0, "%.*g\t", 6);
  } else {
    rc |= write_part("HBSmatRE.dat", dm, n, 0, "%.*g \t", 6);
    rc |= write_part("HBSmatIM.dat", dm, n, 1, "%.*g \t", 6);
    rc |= write_part("BSEcoeffRE.dat", cm, n, 0, "%.*g\t", 6);
    rc |= write_part("BSEcoeffIM.dat", cm, n, 1, "%.*g\t", 6);
  }
  free(dm);
  free(xm);
  return rc ? -1 : 0;
}

int fbse_write_qp_spins(const char *path, const double *psi, const double *eqp, long nqp, long ngrid, double dv)
{ /* qp_spin_frac (bse_cplx/spin.c:3-60): the norm of each spin block of every
   * quasiparticle spinor (complex, interleaved, up block then down block) */
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  for (long i = 0; i < nqp; i++) {
    fprintf(f, "\nStats on state%lu: (E=%lg)\n", (unsigned long)i, eqp[i]);
    for (int s = 0; s < 2; s++) {
      const double *q = psi + (i * 2 + s) * 2 * ngrid;
      double pct = 0.0;
      for (long g = 0; g < ngrid; g++) pct += q[2 * g] * q[2 * g] + q[2 * g + 1] * q[2 * g + 1];
      fprintf(f, " Spin %d fraction: %f\n", s, pct * dv);
    }
  }
  return fclose(f) ? -1 : 0;
}

long fbse_atom_number(const char *label)
{ /* the atom ids of read_conf (assign_atom_number, filter_mpi/read.c:2452-2545):
   * elements by atomic number, the ligand and pseudo-atom labels by their own
   * small ids, 0 for a label outside the list */
  static const struct { const char *sym; long id; } tab[] = {
      {"H", 1},    {"P1", 2},   {"P2", 3},   {"P3", 4},   {"PC5", 5},  {"C", 6},    {"PC6", 7},  {"PR1", 8},
      {"PR2", 9},  {"PR3", 10}, {"PA1", 11}, {"PA2", 12}, {"PA3", 13}, {"Si", 14},  {"P", 15},   {"S", 16},
      {"Cl", 17},  {"C1", 18},  {"C2", 19},  {"C3", 20},  {"Zn", 30},  {"Ga", 31},  {"As", 33},  {"Se", 34},
      {"Br", 35},  {"Cd", 48},  {"In", 49},  {"Te", 52},  {"I", 53},   {"Cs", 55},  {"Pb", 82},  {"Br0", 100},
      {"Br1", 101}, {"I0", 102}, {"I1", 103}, {NULL, 0}};
  for (int i = 0; tab[i].sym; i++)
    if (!strcmp(label, tab[i].sym)) return tab[i].id;
  return 0;
}

int fbse_write_output(const char *path, long tag, long natoms, const double *xyz, int ntypes, const char *labels8,
                      long nx, long ny, long nz, double dx, double dy, double dz, const double *gx, const double *gy,
                      const double *gz, double xmin, double ymin, double zmin, double ke_max, double fermi_e, int so,
                      int nl, int use_spinors, int nspin, int cplx, long n, const double *eval, const double *sigma,
                      const double *psi)
{ /* save_output (filter_mpi/save.c:446-503) with the grid as init_grid_params
   * leaves it (init.c:5-256): box n d (even n) or (n - 1) d (odd n), max
   * (n - 1) d / 2, dk = 2 pi / box */
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  const long ngrid = nx * ny * nz;
  const long n3[3] = {nx, ny, nz};
  const double d3[3] = {dx, dy, dz};
  double dk[3], mx[3];
  for (int a = 0; a < 3; a++) {
    const double box = (n3[a] % 2 == 0) ? (double)n3[a] * d3[a] : (double)(n3[a] - 1) * d3[a];
    dk[a] = 6.283185307179586476925 / box;
    mx[a] = ((double)(n3[a] - 1) * d3[a]) / 2.0;
  }
  fprintf(f, "%ld\n", tag);
  fprintf(f, "%ld %ld\n", ngrid, nspin * ngrid);
  fprintf(f, "%ld\n", n);
  fprintf(f, "%ld %d\n", natoms, ntypes);
  for (int j = 0; j < ntypes; j++) fprintf(f, "%ld ", fbse_atom_number(labels8 + 8 * j));
  fprintf(f, "%d\n", nspin);
  fprintf(f, "%d\n", cplx + 1);
  fprintf(f, "%g %g\n", ke_max, fermi_e);
  fprintf(f, "%d %d %d %d %d\n", so, nl, 0, use_spinors, cplx);
  for (long j = 0; j < natoms; j++) fprintf(f, "%g %g %g\n", xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2]);
  fprintf(f, "%g %g %g %g %g %g %g %g\n", dx, dy, dz, sqrt(dx * dx + dy * dy + dz * dz), dx * dy * dz, dk[0], dk[1],
          dk[2]);
  fprintf(f, "%g %g %g %g %g %g\n", xmin, mx[0], ymin, mx[1], zmin, mx[2]);
  fprintf(f, "%ld %ld %ld\n", nx, ny, nz);
  fprintf(f, "%g %g %g\n", 1.0 / (double)nx, 1.0 / (double)ny, 1.0 / (double)nz);
  fprintf(f, "%ld", ngrid);
  fwrite(gx, sizeof(double), nx, f);
  fwrite(gy, sizeof(double), ny, f);
  fwrite(gz, sizeof(double), nz, f);
  fwrite(eval, sizeof(double), n, f);
  fwrite(sigma, sizeof(double), n, f);
  fwrite(psi, sizeof(double), (size_t)(cplx + 1) * nspin * ngrid * n, f);
  fprintf(f, "\n\nEOF\n");
  return fclose(f) ? -1 : 0;
}

int fbse_write_psi(const char *path, const double *psi, long n_doubles)
{
  FILE *f = fopen(path, "wb");
  if (!f) return -1;
  const size_t w = fwrite(psi, sizeof(double), (size_t)n_doubles, f);
  fclose(f);
  return w == (size_t)n_doubles ? 0 : -1;
}
