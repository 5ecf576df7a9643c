/* fbse_filter: drop-in for the reference's filter executable (filter_mpi).
 *
 * Reads input.par, conf.par, pot<Atm>.par and SO_<Atm>.par from the working
 * directory as the reference does (filter_mpi/read.c), runs the filter stage
 * on one GPU through libfbse_gpu (energy range, Newton filter of every random
 * start, orthogonalisation, subspace diagonalisation, sigma_E) and writes
 * eval.dat, psi.dat and output.dat in the reference's layouts
 * (filter_mpi/write.c:263-299, mod_output.c:5-162, save.c:446-503).
 * Also eval_aux.dat (calc_sigma_E), the per-start psi-filt-<start>-0.dat
 * files (printPsiFilt, on by default as in the reference) and psi-diag.dat
 * (printPsiDiag), and the restarts from them: "restartFromOrtho = 1 <n>"
 * reads psi-filt.dat and starts at the orthogonalisation, "restartFromSigma
 * = 1 <n>" reads psi-diag.dat and only computes energies and sigma_E
 * (main.c:128-305, read.c:954-967); calcFilterOnly stops after the filter.
 * The starts come from psi-init.dat with "inputPsiFilt = 1 <start> <end>".
 * Also written: conf.dat, seed-0.dat, zn.dat / coeff-<t>.dat (read back
 * instead of computed with readCoeffs = 1) and, with "printCubes = 1 <n>",
 * the homo-i / lumo+i cube files of mod_optional_output; with
 * "calcSpinAngStat = 1", angular.dat (calc_angular_exp).
 * Errors go to stderr and the process exits with EXIT_FAILURE, like the
 * reference.  One non-reference key: "mixedPrecision = 1" selects the FP32
 * recursion (default: the plain FP64 method). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#include "../../include/fbse.h"
#include "fbse_dropin.h"

static void die(const char *msg, const char *detail)
{
  fprintf(stderr, "ERROR: %s%s%s\n", msg, detail ? ": " : "", detail ? detail : "");
  exit(EXIT_FAILURE);
}

static void check(fbse_ctx *c, int rc, const char *what)
{
  if (rc) {
    fprintf(stderr, "ERROR: %s failed (%d): %s\n", what, rc, c ? fbse_last_error(c) : "");
    exit(EXIT_FAILURE);
  }
}

/* homo_idx / lumo_idx of print_eigstate_densities (mod_optional_output.c:
 * 103-147): homo is the last converged state below fermiEnergy, lumo the next
 * converged one (0 when there is none), in eval.dat's order */
static void homo_lumo(const fbse_filter_params *p, const double *eval, const double *sigma, long n, long *homo,
                      long *lumo)
{
  *homo = *lumo = 0;
  for (long i = 0; i < n; i++)
    if (eval[i] < p->fermi_e && sigma[i] < p->sigma_e_cut) *homo = i;
  for (long i = *homo + 1; i < n; i++)
    if (sigma[i] < p->sigma_e_cut) { *lumo = i; break; }
}

/* print_eigstate_densities (mod_optional_output.c:74-240): the cubes of
 * homo-i and lumo+i (i < ncubes) hold |psi|^2 signed by the dominant component
 * (density_phase_sign, write.c:52-60), per spin block.  The states are the
 * ones written to psi.dat, in eval.dat's order. */
static void write_cubes(const fbse_filter_params *p, const double *psi, const double *eval, const double *sigma,
                        long n, long nx, long ny, long nz, double xmin, double ymin, double zmin, int nspin, int cplx,
                        long natoms, const double *xyz, const int *atype, char names[][8])
{
  long homo, lumo;
  homo_lumo(p, eval, sigma, n, &homo, &lumo);
  printf("homo_idx = %ld; lumo_idx = %ld\n", homo, lumo);
  if (homo == 0 || lumo == 0) {
    printf("Did not converge enough electron or hole states to visualize cube files.\n");
    return;
  }
  const long ngrid = nx * ny * nz, stlen = (long)(cplx + 1) * nspin * ngrid;
  const long total_homo = homo, total_lumo = n - homo;
  double *rho = malloc(ngrid * sizeof(double));
  char *sym8 = calloc((size_t)natoms * 8, 1);
  if (!rho || !sym8) die("host allocation", NULL);
  for (long a = 0; a < natoms; a++) memcpy(sym8 + 8 * a, names[atype[a]], 7);
  for (int side = 0; side < 2; side++)
    for (long i = 0; i < (side ? total_lumo : total_homo) && i < p->ncubes; i++) {
      const long st = side ? lumo + i : homo - i;
      for (int s = 0; s < nspin; s++) {
        const double *q = psi + st * stlen + (long)(cplx + 1) * s * ngrid;
        for (long g = 0; g < ngrid; g++) {
          const double re = q[(cplx + 1) * g], im = cplx ? q[2 * g + 1] : 0.0;
          const double dom = fabs(re) >= fabs(im) ? re : im;
          rho[g] = (re * re + im * im) * (dom > 0.0 ? 1.0 : (dom < 0.0 ? -1.0 : 0.0));
        }
        char path[64];
        snprintf(path, sizeof path, side ? "lumo+%ld-%s.cube" : "homo-%ld-%s.cube", i, s ? "Dn" : "Up");
        if (fbse_write_cube(path, rho, nx, ny, nz, p->dx, p->dy, p->dz, xmin, ymin, zmin, natoms, sym8, xyz))
          die("cannot write cube file (unknown atom symbol?)", path);
      }
    }
  free(rho);
  free(sym8);
}

/* calcSpinAngStat (mod_optional_output.c:51-62 -> calc_angular_exp,
 * angular.c:4-165): angular.dat with <Jx>, <Jx^2>, <Jy>, <Jy^2>, <Jz>, <Jz^2>,
 * <J^2> and the norm of the states homo - 4 ... lumo + 11 of psi.dat.  The
 * reference takes homo / lumo from print_eigstate_densities, which runs only
 * with printCubes = 1 (otherwise the indices are never set), and reads outside
 * psitot when homo < 4 or lumo + 12 exceeds the states; here the indices are
 * found the same way in either case and the range is clipped to the states
 * written. */
static void write_angular(fbse_ctx *ctx, const fbse_filter_params *p, const double *psi, const double *eval,
                          const double *sigma, long n, long stlen, const double *gx, const double *gy,
                          const double *gz)
{
  long homo, lumo;
  homo_lumo(p, eval, sigma, n, &homo, &lumo);
  long start = homo - 4, stop = lumo + 12;
  if (start < 0) start = 0;
  if (stop > n) stop = n;
  FILE *f = fopen("angular.dat", "w");
  if (!f) die("cannot write", "angular.dat");
  fprintf(f, "###    Jx        Jx^2       Jy        Jy^2      Jz       Jz^2       J^2      norm\n");
  if (stop > start) {
    const long cnt = stop - start;
    const size_t bytes = (size_t)cnt * stlen * sizeof(double);
    void *d = NULL;
    double *st = malloc((size_t)cnt * 8 * sizeof(double));
    if (!st) die("host allocation", NULL);
    check(ctx, fbse_alloc(ctx, &d, bytes), "angular statistics buffer");
    check(ctx, fbse_upload(ctx, d, psi + start * stlen, bytes), "upload");
    check(ctx, fbse_angular_stats(ctx, d, cnt, gx, gy, gz, st), "spin / angular statistics");
    check(ctx, fbse_free(ctx, d), "free");
    for (long i = 0; i < cnt; i++) {
      const double *r = st + 8 * i;
      fprintf(f, "%i\t%f\t%f\t%f\t%f\t%f\t%f\t%f\t%f\n", (int)(start + i), r[0], r[1], r[2], r[3], r[4], r[5],
              r[6], r[7]);
    }
    free(st);
  }
  fclose(f);
  printf("angular.dat: states %ld to %ld\n", start, stop - 1);
}

/* zn.dat and coeff-<t>.dat as gen_newton_coeff writes them (coeff.c:66-108):
 * "%ld %lg" nodes, "%ld %g %g" coefficients */
static void write_coeff_files(const double *zn, const double *an, long nc, long m)
{
  FILE *f = fopen("zn.dat", "w");
  if (!f) die("cannot write", "zn.dat");
  for (long j = 0; j < nc; j++) fprintf(f, "%ld %lg\n", j, zn[j]);
  fclose(f);
  for (long t = 0; t < m; t++) {
    char path[64];
    snprintf(path, sizeof path, "coeff-%ld.dat", t);
    f = fopen(path, "w");
    if (!f) die("cannot write", path);
    for (long j = 0; j < nc; j++) fprintf(f, "%ld %g %g\n", j, an[2 * (t * nc + j)], an[2 * (t * nc + j) + 1]);
    fclose(f);
  }
}

/* read_newton_coeff (coeff.c:176-212): the same files back */
static void read_coeff_files(double *zn, double *an, long nc, long m)
{
  FILE *f = fopen("zn.dat", "r");
  if (!f) die("could not open", "zn.dat");
  long idx;
  for (long j = 0; j < nc; j++)
    if (fscanf(f, "%ld %lg", &idx, &zn[j]) != 2) die("fewer nodes than nCheby in", "zn.dat");
  fclose(f);
  for (long t = 0; t < m; t++) {
    char path[64];
    snprintf(path, sizeof path, "coeff-%ld.dat", t);
    f = fopen(path, "r");
    if (!f) die("could not open", path);
    for (long j = 0; j < nc; j++)
      if (fscanf(f, "%ld %lg %lg", &idx, &an[2 * (t * nc + j)], &an[2 * (t * nc + j) + 1]) != 3)
        die("fewer coefficients than nCheby in", path);
    fclose(f);
  }
}

/* n states of stlen doubles from a raw state file (psi-filt.dat, psi-diag.dat) */
static double *read_states(const char *path, long n, long stlen)
{
  FILE *f = fopen(path, "rb");
  if (!f) die("could not open", path);
  double *buf = malloc((size_t)n * stlen * sizeof(double));
  if (!buf) die("host allocation", path);
  if (fread(buf, sizeof(double), (size_t)n * stlen, f) != (size_t)n * stlen) die("fewer states than requested in", path);
  fclose(f);
  return buf;
}

static void write_states(const char *path, const double *x, long count)
{
  FILE *f = fopen(path, "wb");
  if (!f || fwrite(x, sizeof(double), (size_t)count, f) != (size_t)count) die("cannot write", path);
  fclose(f);
}

int main(void)
{
  char err[512];
  fbse_filter_params p;
  if (fbse_read_filter_params("input.par", &p, err, sizeof err)) die(err, NULL);
  if (p.calc_spin_ang_stat == 1 && !p.use_spinors) /* read.c:82: statistics need spin-orbit (spinor) states */
    die("calcSpinAngStat = 1 needs spinor states (useSpinors = 1)", NULL);
  long natoms;
  double *xyz;
  int *atype, ntypes;
  char names[FBSE_MAX_TYPES][8];
  if (fbse_read_conf("conf.par", &natoms, &xyz, &atype, names, &ntypes, err, sizeof err)) die(err, NULL);
  const int nspin = p.use_spinors ? 2 : 1, cplx = p.use_spinors ? 1 : 0;
  /* conf.dat: the centred configuration the run uses (read.c:1150-1157) */
  FILE *fc = fopen("conf.dat", "w");
  if (!fc) die("cannot write", "conf.dat");
  fprintf(fc, "%ld\n", natoms);
  for (long a = 0; a < natoms; a++)
    fprintf(fc, "%3s % .16g % .16g % .16g\n", names[atype[a]], xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2]);
  fclose(fc);
  printf("fbse_filter: %ld atoms, %d types, nspin %d, SO %d, NL %d, %s\n", natoms, ntypes, nspin, p.so, p.nl,
         p.precision ? "mixed precision" : "FP64");

  /* grid (init_grid_params) */
  long nx, ny, nz;
  double xmin, ymin, zmin;
  fbse_grid_rule(xyz, natoms, p.dx, p.nx, 0, &nx, &xmin);
  fbse_grid_rule(xyz, natoms, p.dy, p.ny, 1, &ny, &ymin);
  fbse_grid_rule(xyz, natoms, p.dz, p.nz, 2, &nz, &zmin);
  const long ngrid = nx * ny * nz;
  double *gx = malloc(nx * sizeof(double)), *gy = malloc(ny * sizeof(double)), *gz = malloc(nz * sizeof(double));
  fbse_grid_axis(nx, xmin, p.dx, gx);
  fbse_grid_axis(ny, ymin, p.dy, gy);
  fbse_grid_axis(nz, zmin, p.dz, gz);
  printf("grid %ld x %ld x %ld, d = %g %g %g, origin %g %g %g\n", nx, ny, nz, p.dx, p.dy, p.dz, xmin, ymin, zmin);

  /* local potential (build_local_pot on the GPU) */
  double *tr = NULL, *tv = NULL;
  long *toff = malloc(ntypes * sizeof(long)), *tlen = malloc(ntypes * sizeof(long)), tot = 0;
  for (int t = 0; t < ntypes; t++) {
    char path[64];
    double *r, *v;
    snprintf(path, sizeof path, "pot%s.par", names[t]);
    const long n = fbse_read_table(path, &r, &v);
    if (n < 2) die("cannot read potential table", path);
    tr = realloc(tr, (tot + n) * sizeof(double));
    tv = realloc(tv, (tot + n) * sizeof(double));
    memcpy(tr + tot, r, n * sizeof(double));
    memcpy(tv + tot, v, n * sizeof(double));
    toff[t] = tot;
    tlen[t] = n;
    tot += n;
    free(r);
    free(v);
  }
  double *pot = malloc(ngrid * sizeof(double));
  check(NULL, fbse_build_local_pot(nx, ny, nz, gx, gy, gz, natoms, xyz, atype, ntypes, tr, tv, toff, tlen, pot),
        "build_local_pot");
  double vmin_loc = pot[0], vmax_loc = pot[0];
  for (long i = 1; i < ngrid; i++) {
    if (pot[i] < vmin_loc) vmin_loc = pot[i];
    if (pot[i] > vmax_loc) vmax_loc = pot[i];
  }

  /* projectors (gen_SO_projectors / gen_nlc_projectors, init_NL_projectors) */
  fbse_proj_desc pd;
  memset(&pd, 0, sizeof pd);
  long *nl = NULL;
  int *jx = NULL, *sgn = NULL;
  double *y1 = NULL, *sop = NULL, *nlp = NULL, nl_lam_min = 0.0, nl_lam_max = 0.0;
  if (p.so || p.nl) {
    const int np = FBSE_NPROJ;
    const long N = FBSE_PROJ_LEN;
    const double rc2 = fbse_r_nlcut2(p.dx), rc = sqrt(rc2);
    double so_par[FBSE_MAX_TYPES], lam[FBSE_MAX_TYPES][2];
    for (int t = 0; t < ntypes; t++) {
      so_par[t] = lam[t][0] = lam[t][1] = 0.0;
      if (fbse_is_ligand(names[t])) continue;
      if (fbse_read_so_params(names[t], &so_par[t], lam[t], err, sizeof err)) die(err, NULL);
    }
    long nat = 0;
    for (long a = 0; a < natoms; a++)
      if (!fbse_is_ligand(names[atype[a]])) nat++;
    double *pxyz = malloc(3 * (nat ? nat : 1) * sizeof(double)), *psp = malloc((nat ? nat : 1) * sizeof(double));
    double *so_tab = calloc(np * N, sizeof(double));
    double *nl_tab = calloc((size_t)(nat ? nat : 1) * np * N, sizeof(double));
    double *type_nl = calloc((size_t)ntypes * np * N, sizeof(double));
    int *type_sg = calloc((size_t)ntypes * np, sizeof(int));
    sgn = calloc((size_t)(nat ? nat : 1) * np, sizeof(int));
    if (p.so && fbse_radial_projectors(p.dx, rc, 0, 0.0, 0.0, np, so_tab, NULL)) die("SO projectors", NULL);
    if (p.nl)
      for (int t = 0; t < ntypes; t++)
        if (!fbse_is_ligand(names[t]) &&
            fbse_radial_projectors(p.dx, rc, 1, lam[t][0], lam[t][1], np, type_nl + (long)t * np * N,
                                   type_sg + t * np))
          die("NL projectors", names[t]);
    long k = 0;
    for (long a = 0; a < natoms; a++) {
      const int t = atype[a];
      if (fbse_is_ligand(names[t])) continue;
      memcpy(pxyz + 3 * k, xyz + 3 * a, 3 * sizeof(double));
      psp[k] = so_par[t];
      if (p.nl) {
        memcpy(nl_tab + (size_t)k * np * N, type_nl + (long)t * np * N, np * N * sizeof(double));
        memcpy(sgn + k * np, type_sg + t * np, np * sizeof(int));
      }
      k++;
    }
    long npts;
    if (fbse_build_nlc(nx, ny, nz, gx, gy, gz, nat, pxyz, psp, p.so ? so_tab : NULL, p.nl ? nl_tab : NULL, np, rc2,
                       &npts, &nl, &jx, &y1, &sop, &nlp))
      die("projector table", NULL);
    printf("projectors: %ld atoms, %ld grid points per sphere\n", nat, npts);
    if (p.nl) /* NL spectral bounds (filter_mpi/init.c:1095-1130) for the range rule */
      fbse_nl_bounds(nat, npts, np, nl, y1, nlp, sgn, p.dx * p.dy * p.dz, &nl_lam_min, &nl_lam_max);
    pd.n_atoms = nat;
    pd.npts = npts;
    pd.nproj = np;
    pd.nl = nl;
    pd.jxyz = jx;
    pd.y1 = y1;
    pd.so_proj = sop;
    pd.nl_proj = nlp;
    pd.nl_sign = sgn;
    pd.LS = NULL;
    free(pxyz);
    free(psp);
    free(so_tab);
    free(nl_tab);
    free(type_nl);
    free(type_sg);
  }

  fbse_grid_desc gd;
  memset(&gd, 0, sizeof gd);
  gd.nx = nx; gd.ny = ny; gd.nz = nz;
  gd.dx = p.dx; gd.dy = p.dy; gd.dz = p.dz;
  gd.ke_max = p.ke_max;
  gd.nspin = nspin;
  gd.is_complex = cplx;
  gd.so = p.so;
  gd.nl = p.nl;
  fbse_ctx *ctx = NULL;
  int rc = fbse_create(&ctx, &gd, pot, (p.so || p.nl) ? &pd : NULL, p.precision ? FBSE_MIXED : FBSE_FP64);
  check(ctx, rc, "fbse_create");

  const long stlen = (long)(cplx + 1) * nspin * ngrid;
  const size_t sbytes = (size_t)stlen * sizeof(double);
  long n = 0;         /* states entering ortho (or sigma) */
  void *d_psi = NULL; /* psitot on the device */
  double *host_psi = NULL;
  if (p.restart_from_sigma) {
    /* restart_from_sigma (mod_sigma.c:67-124): psi-diag.dat holds the
     * diagonalised states, stlen doubles each */
    n = p.n_states_for_sigma;
    host_psi = read_states("psi-diag.dat", n, stlen);
    check(ctx, fbse_alloc(ctx, &d_psi, n * sbytes), "state buffer");
    check(ctx, fbse_upload(ctx, d_psi, host_psi, n * sbytes), "upload psi-diag.dat");
  } else if (p.restart_from_ortho) {
    /* restart_from_ortho (ortho.c:189-240): psi-filt.dat holds the filtered
     * states (the psi-filt-<start>-<rank>.dat files one after the other) */
    n = p.n_states_for_ortho;
    host_psi = read_states("psi-filt.dat", n, stlen);
    check(ctx, fbse_alloc(ctx, &d_psi, n * sbytes), "state buffer");
    check(ctx, fbse_upload(ctx, d_psi, host_psi, n * sbytes), "upload psi-filt.dat");
    free(host_psi);
    host_psi = NULL;
  } else {
    /* energy range (get_energy_range, filter_mpi/energy.c:169-379) */
    double emin = 0.0, emax = 0.0;
    if (!p.approx_energy_range) {
      long iters = 0;
      check(ctx, fbse_energy_range(ctx, -874917403, 1500, &emin, &emax, &iters), "energy range");
      printf("energy range: Emin %g, Emax %g (%ld iterations)\n", emin, emax, iters);
    }
    /* the approximate range with its projector pads, then the inflation (energy.c:302-369) */
    fbse_energy_range_rule(p.approx_energy_range, p.so, p.nl, vmin_loc, vmax_loc, p.ke_max, nl_lam_min, nl_lam_max,
                           &emin, &emax);
    const double de = emax - emin;
    printf("Emin = %g, Emax = %g, dE = %g\n", emin, emax, de);

    /* targets (set_ene_targets, init.c:401-478) and Newton coefficients */
    const long m = p.m_states_per_filter, nc = p.ncheby, ns = p.n_filter_cycles;
    double *targets = malloc(m * sizeof(double));
    fbse_ene_targets(m, p.n_targets_vb, p.vbmin, p.vbmax, p.cbmin, p.cbmax, targets);
    double *zn = malloc(nc * sizeof(double)), *an = malloc(2 * m * nc * sizeof(double));
    if (p.read_coeffs == 1) {
      read_coeff_files(zn, an, nc, m);
    } else {
      fbse_samp_points(nc, zn);
      const double dt = ((double)nc / (2.5 * de)) * ((double)nc / (2.5 * de)); /* mod_filter.c:114 */
      if (fbse_newton_coeff(nc, m, zn, targets, emin, de, dt, an)) die("Newton coefficients", NULL);
      write_coeff_files(zn, an, nc, m);
    }

    /* random starts (mod_filter.c:152-160, init_filter_states) */
    long seed;
    if (p.set_seed == 1) seed = -p.seed;
    else {
      srandom((unsigned)(time(NULL) ^ (getpid() << 8)));
      seed = -random();
    }
    double *starts = malloc((size_t)ns * sbytes);
    if (!starts) die("host allocation", NULL);
    if (p.input_psi_filt == 1) {
      /* read_psi_dat (aux.c:131-156): from state `start`, every second state
       * for spinors (Kramers partners skipped), the one after each skip; the
       * read states fill psi_rank contiguously and cycle jns starts from the
       * first state of its block, jns * m (filter.c:253-275) */
      const long every = nspin == 2 ? 2 : 1;
      const long nread = (p.init_psi_end - p.init_psi_start + every - 1) / every;
      if ((ns - 1) * m >= nread) die("psi-init.dat range holds fewer states than nFilterCycles x mStatesPerFilter", NULL);
      FILE *fi = fopen("psi-init.dat", "rb");
      if (!fi) die("could not open", "psi-init.dat");
      for (long j = 0; j < ns; j++) {
        const long q = j * m; /* read index of this start */
        const long state = p.init_psi_start + q * every + (every - 1);
        if (fseek(fi, (long)(state * sbytes), SEEK_SET) || fread(starts + j * stlen, sizeof(double), stlen, fi) != (size_t)stlen)
          die("truncated", "psi-init.dat");
      }
      fclose(fi);
    } else {
      long *seeds = malloc((size_t)ns * nspin * sizeof(long));
      if (!seeds) die("host allocation", NULL);
      fbse_init_filter_states(starts, ns, ngrid, nspin, cplx, p.dx * p.dy * p.dz, seed, seeds);
      FILE *fsd = fopen("seed-0.dat", "w"); /* init.c:1204-1212 */
      if (!fsd) die("cannot write", "seed-0.dat");
      fprintf(fsd, "idx  seed\n");
      for (long k = 0; k < ns * nspin; k++) fprintf(fsd, "%ld %ld\n", k, seeds[k]);
      fclose(fsd);
      free(seeds);
    }

    /* the filter cycles of every start at once (run_filter_cycles) */
    void *d_starts = NULL;
    n = ns * m;
    check(ctx, fbse_alloc(ctx, &d_starts, ns * sbytes), "start buffer");
    check(ctx, fbse_alloc(ctx, &d_psi, n * sbytes), "state buffer");
    check(ctx, fbse_upload(ctx, d_starts, starts, ns * sbytes), "upload starts");
    check(ctx, fbse_newton_filter(ctx, zn, an, nc, m, emin, de, d_starts, ns, d_psi), "Newton filter");
    check(ctx, fbse_free(ctx, d_starts), "free");
    free(starts);
    free(targets);
    free(zn);
    free(an);
    if (p.print_psi_filt) {
      /* printPsiFilt (filter.c:118-138): the m filtered states of start jns,
       * before normalisation, in psi-filt-<jns>-<rank>.dat */
      double *blk = malloc(m * sbytes);
      if (!blk) die("host allocation", NULL);
      for (long j = 0; j < ns; j++) {
        char path[64];
        snprintf(path, sizeof path, "psi-filt-%ld-0.dat", j);
        check(ctx, fbse_download(ctx, blk, (char *)d_psi + (size_t)j * m * sbytes, m * sbytes), "download");
        write_states(path, blk, m * stlen);
      }
      free(blk);
    }
    if (p.calc_filter_only) { /* main.c:160-163 */
      printf("calcFilterOnly: %ld filtered states, stopping after the filter\n", n);
      fbse_destroy(ctx);
      return 0;
    }
  }

  double *eval = malloc(n * sizeof(double)), *sigma = malloc(n * sizeof(double));
  if (!eval || !sigma) die("host allocation", NULL);
  long nk = n;
  if (p.restart_from_sigma) {
    /* mod_sigma -> calc_sigma_E (energy.c:383-539) */
    check(ctx, fbse_sigma_e(ctx, d_psi, n, eval, sigma), "sigma_E");
  } else {
    /* normalize_all after the filter (filter.c:152) or on restart
     * (ortho.c:242), then ortho + diag + sigma_E */
    check(ctx, fbse_normalize_all(ctx, d_psi, n, NULL), "normalize_all");
    check(ctx, fbse_ortho_diag_sigma(ctx, d_psi, n, &nk, eval, sigma), "ortho/diag/sigma");
    printf("%ld states after orthogonalisation\n", nk);
  }
  FILE *fa = fopen("eval_aux.dat", "w"); /* calc_sigma_E (energy.c:528) */
  if (!fa) die("cannot write", "eval_aux.dat");
  for (long i = 0; i < nk; i++) fprintf(fa, "%ld %.16lg %.16lg\n", i, eval[i], sigma[i]);
  fclose(fa);
  if (p.print_psi_diag && !p.restart_from_sigma) {
    /* printPsiDiag (mod_diag.c:439-444): every diagonalised state */
    double *all = malloc(nk * sbytes);
    if (!all) die("host allocation", NULL);
    check(ctx, fbse_download(ctx, all, d_psi, nk * sbytes), "download");
    write_states("psi-diag.dat", all, nk * stlen);
    free(all);
  }

  /* mod_output's selection (mod_output.c:63-120): every state, or those with
   * sigma_E <= sigmaECut */
  double *psi = malloc((size_t)(nk ? nk : 1) * sbytes);
  if (!psi) die("host allocation", NULL);
  long n_out = 0;
  for (long i = 0; i < nk; i++) {
    if (!p.get_all_states && !(sigma[i] <= p.sigma_e_cut)) continue;
    eval[n_out] = eval[i];
    sigma[n_out] = sigma[i];
    if (host_psi) memcpy(psi + n_out * stlen, host_psi + i * stlen, sbytes);
    else check(ctx, fbse_download(ctx, psi + n_out * stlen, (char *)d_psi + i * sbytes, sbytes), "download");
    n_out++;
  }
  printf("%ld eigenstates written\n", n_out);
  if (fbse_write_eval("eval.dat", eval, sigma, n_out)) die("cannot write", "eval.dat");
  if (fbse_write_psi("psi.dat", psi, n_out * stlen)) die("cannot write", "psi.dat");
  /* save_output (filter_mpi/save.c:446-503); its first line is a random tag */
  if (fbse_write_output("output.dat", (long)random(), natoms, xyz, ntypes, (const char *)names, nx, ny, nz, p.dx, p.dy,
                        p.dz, gx, gy, gz, xmin, ymin, zmin, p.ke_max, p.fermi_e, p.so, p.nl, p.use_spinors, nspin,
                        cplx, n_out, eval, sigma, psi))
    die("cannot write", "output.dat");
  check(ctx, fbse_free(ctx, d_psi), "free");
  if (p.print_cubes == 1)
    write_cubes(&p, psi, eval, sigma, n_out, nx, ny, nz, xmin, ymin, zmin, nspin, cplx, natoms, xyz, atype, names);
  if (p.calc_spin_ang_stat == 1) write_angular(ctx, &p, psi, eval, sigma, n_out, stlen, gx, gy, gz);
  fbse_destroy(ctx);
  return 0;
}
