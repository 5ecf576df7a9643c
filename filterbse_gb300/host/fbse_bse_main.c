/* fbse_bse: drop-in for the reference's bse executables: bse_cplx for
 * spinor filter output, bse_real for real one-component states (the singlet
 * exchange factor 2, real kernel files and optical files).
 *
 * Reads input.par and the filter's output.dat from the working directory
 * (bse_cplx/read.c, save.c), picks the quasiparticle basis as
 * get_qp_basis_indices does (bse_cplx/basis.c:7-254), and runs the BSE stage
 * on one GPU through libfbse_gpu: Coulomb potentials (init.c), direct and
 * exchange kernels (coulomb.c), the BSE eigensolve with its expectation
 * values (mod_bse.c, bethe-salpeter.c), pair and exciton transition dipoles
 * (dipole.c, optical.c), magnetic dipoles and rotational strengths.  Writes
 * BSEeval.par, direct-0.dat, exchange-0.dat, h0.dat, bsRE/IM.dat,
 * HBSmatRE/IM.dat, BSEcoeffRE/IM.dat, exciton.dat, OS0.dat, OS.dat, M0.dat,
 * M.dat, rs0.dat, rs.dat and bs-coeff-<j>.dat in the reference's formats; coulombDone = 1 reads the kernels back from direct.dat /
 * exchange.dat instead of computing them, calcCoulombOnly stops after the
 * kernels.  Errors go to stderr with EXIT_FAILURE. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/fbse.h"
#include "fbse_dropin.h"

#define AUTOEV 27.2114 /* bse_cplx/fd.h */

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

typedef struct {
  long ngrid, nspinngrid, mn, natoms, ntypes, nx, ny, nz;
  int nspin, complex_idx, so, nl;
  double ke_max, fermi_e, dx, dy, dz, xmin, ymin, zmin;
  double *eval, *sigma;
  long psi_pos; /* file offset of psitot */
} output_dat;

static int expect(int got, int want) { return got == want ? 0 : -1; }

/* the header and eigenvalues of output.dat (filter_mpi/save.c:446-503) */
static void read_output(const char *path, output_dat *o)
{
  FILE *f = fopen(path, "rb");
  if (!f) die("cannot open", path);
  long tag, lv;
  double d[8];
  int bad = 0;
  bad |= expect(fscanf(f, "%ld", &tag), 1);
  bad |= expect(fscanf(f, "%ld %ld", &o->ngrid, &o->nspinngrid), 2);
  bad |= expect(fscanf(f, "%ld", &o->mn), 1);
  bad |= expect(fscanf(f, "%ld %ld", &o->natoms, &o->ntypes), 2);
  for (long j = 0; j < o->ntypes && !bad; j++) bad |= expect(fscanf(f, "%ld", &lv), 1);
  bad |= expect(fscanf(f, "%d", &o->nspin), 1);
  bad |= expect(fscanf(f, "%d", &o->complex_idx), 1);
  bad |= expect(fscanf(f, "%lg %lg", &o->ke_max, &o->fermi_e), 2);
  int lr, spin, cplx;
  bad |= expect(fscanf(f, "%d %d %d %d %d", &o->so, &o->nl, &lr, &spin, &cplx), 5);
  for (long j = 0; j < o->natoms && !bad; j++) bad |= expect(fscanf(f, "%lg %lg %lg", &d[0], &d[1], &d[2]), 3);
  bad |= expect(fscanf(f, "%lg %lg %lg %lg %lg %lg %lg %lg", &o->dx, &o->dy, &o->dz, &d[3], &d[4], &d[5], &d[6],
                       &d[7]),
                8);
  bad |= expect(fscanf(f, "%lg %lg %lg %lg %lg %lg", &o->xmin, &d[0], &o->ymin, &d[1], &o->zmin, &d[2]), 6);
  bad |= expect(fscanf(f, "%ld %ld %ld", &o->nx, &o->ny, &o->nz), 3);
  bad |= expect(fscanf(f, "%lg %lg %lg", &d[0], &d[1], &d[2]), 3);
  if (bad || o->nx * o->ny * o->nz != o->ngrid) die("malformed header in", path);
  /* "%ld" of ngrid is followed directly by binary data: skip whitespace, then
   * exactly the digits of ngrid, so that a first binary byte that happens to
   * look like a digit is not swallowed */
  char want[32];
  snprintf(want, sizeof want, "%ld", o->ngrid);
  int ch;
  do ch = fgetc(f); while (ch == ' ' || ch == '\n' || ch == '\r' || ch == '\t');
  for (size_t k = 0; k < strlen(want); k++) {
    if (ch != want[k]) die("malformed grid size in", path);
    if (k + 1 < strlen(want)) ch = fgetc(f);
  }
  /* skip the grid coordinates (the BSE builds x = xmin + j dx, bse_cplx/read.c:398-409) */
  if (fseek(f, (o->nx + o->ny + o->nz) * (long)sizeof(double), SEEK_CUR)) die("truncated", path);
  o->eval = malloc(o->mn * sizeof(double));
  o->sigma = malloc(o->mn * sizeof(double));
  if (fread(o->eval, sizeof(double), o->mn, f) != (size_t)o->mn ||
      fread(o->sigma, sizeof(double), o->mn, f) != (size_t)o->mn)
    die("truncated eigenvalues in", path);
  o->psi_pos = ftell(f);
  fclose(f);
}

/* one part (0: re, 1: im) of an n x n complex row-major matrix as text rows */
static void write_matrices(fbse_ctx *ctx, void *d_dir, void *d_exc, void *d_coef, const double *eqp, long nh,
                           long ne, long lumo, int real)
{ /* the matrix files of the solve, from the device kernels and coefficients */
  const long n = nh * ne;
  const size_t bytes = (size_t)n * n * 2 * sizeof(double);
  double *dm = malloc(bytes), *xm = malloc(bytes), *cm = malloc(bytes);
  if (!dm || !xm || !cm) die("host allocation", NULL);
  check(ctx, fbse_download(ctx, dm, d_dir, bytes), "download");
  check(ctx, fbse_download(ctx, xm, d_exc, bytes), "download");
  check(ctx, fbse_download(ctx, cm, d_coef, bytes), "download");
  if (fbse_write_bse_matrices(dm, xm, cm, eqp, nh, ne, lumo, real)) die("cannot write", "the BSE matrix files");
  free(dm);
  free(xm);
  free(cm);
}

/* calcSpinAngStat (bse_cplx/main.c:160-195): the quasiparticle spin and
 * angular-momentum matrices (sx/sy/sz.dat, lx/ly/lz/lsqr/ls.dat,
 * angular.c:116-129, 200-211, 436-460, 562-586) and the exciton statistics
 * (spins.dat, orbital.dat, couple.dat, angular.c:789-791, 949-950, 1034) */
static void write_ang_stats(fbse_ctx *ctx, void *d_psi, const double *gx, const double *gy, const double *gz,
                            long nh, long ne, long lumo, const double *coeff)
{
  const long n = nh * nh + ne * ne, nx = nh * ne;
  double *sm = malloc(n * 6 * sizeof(double)), *lm = malloc(n * 6 * sizeof(double));
  double *l2 = malloc(n * 2 * sizeof(double)), *ls = malloc(n * 2 * sizeof(double));
  double *sp = malloc(nx * 6 * sizeof(double)), *st = malloc(nx * 2 * sizeof(double));
  double *orb = malloc(nx * 6 * sizeof(double)), *ot = malloc(nx * 2 * sizeof(double));
  double *lst = malloc(nx * 2 * sizeof(double));
  if (!sm || !lm || !l2 || !ls || !sp || !st || !orb || !ot || !lst) die("host allocation", NULL);
  check(ctx, fbse_bse_qp_ang_mom(ctx, d_psi, gx, gy, gz, nh, ne, lumo, sm, lm, l2, ls), "angular momenta");
  const char *sn[3] = {"sx.dat", "sy.dat", "sz.dat"}, *ln[3] = {"lx.dat", "ly.dat", "lz.dat"};
  for (int d = 0; d < 3; d++) {
    FILE *fs = fopen(sn[d], "w"), *fl = fopen(ln[d], "w");
    if (!fs || !fl) die("cannot write", sn[d]);
    for (int blk = 0; blk < 2; blk++) {
      const long cnt = blk ? ne : nh, off = blk ? nh * nh : 0, base = blk ? lumo : 0;
      for (long i = 0; i < cnt; i++)
        for (long j = 0; j < cnt; j++) {
          const long k = off + i * cnt + j;
          fprintf(fs, "%ld %ld % .10g % .10g\n", base + i, base + j, sm[6 * k + 2 * d], sm[6 * k + 2 * d + 1]);
          fprintf(fl, "%ld\t%ld\t%lf\t%lf\n", base + i, base + j, lm[6 * k + 2 * d], lm[6 * k + 2 * d + 1]);
        }
    }
    fclose(fs);
    fclose(fl);
  }
  FILE *fq = fopen("lsqr.dat", "w"), *fls = fopen("ls.dat", "w");
  if (!fq || !fls) die("cannot write", "lsqr.dat / ls.dat");
  for (int blk = 0; blk < 2; blk++) {
    const long cnt = blk ? ne : nh, off = blk ? nh * nh : 0, base = blk ? lumo : 0;
    for (long i = 0; i < cnt; i++)
      for (long j = 0; j < cnt; j++) {
        const long k = off + i * cnt + j;
        fprintf(fq, "%ld\t%ld\t%lf\t%lf\n", base + i, base + j, l2[2 * k], l2[2 * k + 1]);
        fprintf(fls, "%ld\t%ld\t%lf\t%lf\n", base + i, base + j, ls[2 * k], ls[2 * k + 1]);
      }
  }
  fclose(fq);
  fclose(fls);
  if (fbse_xton_ang_stats(nh, ne, coeff, sm, lm, l2, ls, sp, st, orb, ot, lst)) die("host allocation", NULL);
  FILE *fsp = fopen("spins.dat", "w"), *fo = fopen("orbital.dat", "w"), *fc = fopen("couple.dat", "w");
  if (!fsp || !fo || !fc) die("cannot write", "spins.dat / orbital.dat / couple.dat");
  for (long j = 0; j < nx; j++) {
    fprintf(fsp, "%ld\t%-10.5lg\t%-10.5lg\t%-10.5lg\t%-10.5lg\t%-10.5lg\t%-10.5lg\t", j, sp[6 * j], sp[6 * j + 1],
            sp[6 * j + 2], sp[6 * j + 3], sp[6 * j + 4], sp[6 * j + 5]);
    fprintf(fsp, "%-10.5lg\t (%-10.5lg)\n", 1.5 + 2.0 * st[2 * j], 2.0 * st[2 * j + 1]);
    fprintf(fo, "%ld\t%-10.5lf\t%-10.5lf\t%-10.5lf\t", j, orb[6 * j], orb[6 * j + 2], orb[6 * j + 4]);
    fprintf(fo, "%-10.5lf\t (%-10.5lf)\n", ot[2 * j], ot[2 * j + 1]);
    fprintf(fc, "%ld\t%-10.5lf\t (%-10.5lf)\n", j, lst[2 * j], lst[2 * j + 1]);
  }
  fclose(fsp);
  fclose(fo);
  fclose(fc);
  free(sm); free(lm); free(l2); free(ls); free(sp); free(st); free(orb); free(ot); free(lst);
}

/* Im(mu . conj(m)) of two complex 3-vectors stored (re, im) x 3 */
static double im_dot_conj(const double *mu, const double *m)
{
  double r = 0.0;
  for (int d = 0; d < 3; d++) r += mu[2 * d + 1] * m[2 * d] - mu[2 * d] * m[2 * d + 1];
  return r;
}


/* load_coulomb_mat (bse_cplx/coulomb.c:742-817): fills mat[ibs][jbs] from the
 * lines of path; the file is complete when the largest a, b reach the last
 * electron and the largest i, j the last hole (mod_kernel.c:56-80) */
static void load_kernel_file(const char *path, double *mat, long nh, long ne, long lumo, int real)
{
  const long nx = nh * ne;
  FILE *f = fopen(path, "r");
  if (!f) die("could not open file", path);
  long a, b, i, j, ibs, jbs, amax = 0, bmax = 0, imax = 0, jmax = 0, cnt = 0;
  double re, im = 0.0;
  while (cnt < nx * nx && (real ? fscanf(f, "%ld %ld %ld %ld %ld %ld %lg", &a, &b, &i, &j, &ibs, &jbs, &re) == 7
                                : fscanf(f, "%ld %ld %ld %ld %ld %ld %lg %lg", &a, &b, &i, &j, &ibs, &jbs, &re, &im) == 8)) {
    if (ibs < 0 || ibs >= nx || jbs < 0 || jbs >= nx) die("pair index out of range in", path);
    mat[2 * (ibs * nx + jbs)] = re;
    mat[2 * (ibs * nx + jbs) + 1] = im;
    if (a > amax) amax = a;
    if (b > bmax) bmax = b;
    if (i > imax) imax = i;
    if (j > jmax) jmax = j;
    cnt++;
  }
  fclose(f);
  const long el_max = lumo + ne - 1, ho_max = nh - 1;
  if (!(amax == el_max && bmax == el_max && imax == ho_max && jmax == ho_max))
    die("matrix elements not done in", path);
}

int main(void)
{
  char err[512];
  fbse_bse_params p;
  if (fbse_read_bse_params("input.par", &p, err, sizeof err)) die(err, NULL);
  output_dat o;
  read_output("output.dat", &o);
  /* complex spinors: bse_cplx; real one-component states: bse_real */
  const int real = (o.complex_idx == 1 && o.nspin == 1);
  if (!real && !(o.complex_idx == 2 && o.nspin == 2))
    die("output.dat holds neither complex spinors (bse_cplx) nor real one-component states (bse_real)", NULL);

  /* get_qp_basis_indices (bse_cplx/basis.c:7-254) */
  long *sel = malloc((o.mn ? o.mn : 1) * sizeof(long)), nh = 0, ne = 0;
  fbse_qp_basis(o.eval, o.sigma, o.mn, p.sigma_e_cut, p.fermi_e, p.max_hole_states, p.max_elec_states, sel, &nh,
                &ne);
  if (nh < 1 || ne < 1) die("no converged hole or electron states below/above fermiEnergy", NULL);
  const long nqp = nh + ne, lumo = nh, nx = nh * ne;
  double *eqp = malloc(nqp * sizeof(double));
  FILE *fe = fopen("BSEeval.par", "w");
  for (long i = 0; i < nqp; i++) {
    eqp[i] = o.eval[sel[i]];
    if (fe) fprintf(fe, "%ld % .12f %g\n", i, eqp[i], o.sigma[sel[i]]);
  }
  if (fe) fclose(fe);
  printf("fbse_bse: %ld holes, %ld electrons, %ld excitons; gap %.6g Ha\n", nh, ne, nx, eqp[lumo] - eqp[lumo - 1]);

  /* the basis states (get_qp_basis, basis.c:258-300): as stored (flen
   * doubles each), and as complex states (stlen doubles) for the dipoles */
  const long flen = o.complex_idx * o.nspinngrid, stlen = 2 * o.nspinngrid;
  double *file_psi = malloc((size_t)nqp * flen * sizeof(double));
  FILE *f = fopen("output.dat", "rb");
  if (!f || !file_psi) die("cannot read states from", "output.dat");
  for (long i = 0; i < nqp; i++) {
    if (fseek(f, o.psi_pos + sel[i] * flen * (long)sizeof(double), SEEK_SET) ||
        fread(file_psi + i * flen, sizeof(double), flen, f) != (size_t)flen)
      die("truncated states in", "output.dat");
  }
  fclose(f);
  double *psi_host = file_psi;
  if (real) {
    psi_host = calloc((size_t)nqp * stlen, sizeof(double));
    if (!psi_host) die("host allocation", NULL);
    for (size_t k = 0; k < (size_t)nqp * flen; k++) psi_host[2 * k] = file_psi[k];
  }

  /* context: the grid only (no potential / projectors are used by the BSE) */
  fbse_grid_desc gd;
  memset(&gd, 0, sizeof gd);
  gd.nx = o.nx; gd.ny = o.ny; gd.nz = o.nz;
  gd.dx = o.dx; gd.dy = o.dy; gd.dz = o.dz;
  gd.ke_max = o.ke_max;
  gd.nspin = o.nspin;
  gd.is_complex = 1;
  double *zero = calloc(o.ngrid, sizeof(double));
  fbse_ctx *ctx = NULL;
  check(ctx, fbse_create(&ctx, &gd, zero, NULL, p.precision ? FBSE_MIXED : FBSE_FP64), "fbse_create");
  double *gx = malloc(o.nx * sizeof(double)), *gy = malloc(o.ny * sizeof(double)), *gz = malloc(o.nz * sizeof(double));
  for (long j = 0; j < o.nx; j++) gx[j] = o.xmin + j * o.dx;
  for (long j = 0; j < o.ny; j++) gy[j] = o.ymin + j * o.dy;
  for (long j = 0; j < o.nz; j++) gz[j] = o.zmin + j * o.dz;

  void *d_psi, *d_bare, *d_scr, *d_dir, *d_exc, *d_coef;
  check(ctx, fbse_alloc(ctx, &d_psi, (size_t)nqp * stlen * sizeof(double)), "alloc");
  check(ctx, fbse_alloc(ctx, &d_bare, o.ngrid * 2 * sizeof(double)), "alloc");
  check(ctx, fbse_alloc(ctx, &d_scr, o.ngrid * 2 * sizeof(double)), "alloc");
  check(ctx, fbse_alloc(ctx, &d_dir, (size_t)nx * nx * 2 * sizeof(double)), "alloc");
  check(ctx, fbse_alloc(ctx, &d_exc, (size_t)nx * nx * 2 * sizeof(double)), "alloc");
  check(ctx, fbse_alloc(ctx, &d_coef, (size_t)nx * nx * 2 * sizeof(double)), "alloc");
  check(ctx, fbse_upload(ctx, d_psi, psi_host, (size_t)nqp * stlen * sizeof(double)), "upload");
  double *zeros = calloc((size_t)nx * nx * 2, sizeof(double));
  check(ctx, fbse_upload(ctx, d_dir, zeros, (size_t)nx * nx * 2 * sizeof(double)), "upload");
  check(ctx, fbse_upload(ctx, d_exc, zeros, (size_t)nx * nx * 2 * sizeof(double)), "upload");

  check(ctx, fbse_bse_potentials(ctx, gx, gy, gz, o.xmin, o.ymin, o.zmin, p.eps_x, p.eps_y, p.eps_z, d_bare, d_scr),
        "Coulomb potentials");
  {
    const size_t mbytes = (size_t)nx * nx * 2 * sizeof(double);
    double *hd = calloc((size_t)nx * nx * 2, sizeof(double)), *hx = calloc((size_t)nx * nx * 2, sizeof(double));
    if (!hd || !hx) die("host allocation", NULL);
    if (p.coulomb_done) {
      /* coulombDone = 1: the kernels from direct.dat / exchange.dat (mod_kernel.c:56-80) */
      load_kernel_file("direct.dat", hd, nh, ne, lumo, real);
      load_kernel_file("exchange.dat", hx, nh, ne, lumo, real);
      check(ctx, fbse_upload(ctx, d_dir, hd, mbytes), "upload");
      check(ctx, fbse_upload(ctx, d_exc, hx, mbytes), "upload");
      printf("kernels loaded from direct.dat and exchange.dat\n");
    } else if (real) {
      /* bse_real: real kernels from the real states, as complex matrices for the solve */
      void *d_pr, *d_dr, *d_xr;
      const size_t rb = (size_t)nx * nx * sizeof(double);
      check(ctx, fbse_alloc(ctx, &d_pr, (size_t)nqp * flen * sizeof(double)), "alloc");
      check(ctx, fbse_alloc(ctx, &d_dr, rb), "alloc");
      check(ctx, fbse_alloc(ctx, &d_xr, rb), "alloc");
      check(ctx, fbse_upload(ctx, d_pr, file_psi, (size_t)nqp * flen * sizeof(double)), "upload");
      check(ctx, fbse_bse_kernel_real(ctx, d_pr, nh, ne, lumo, d_bare, d_scr, d_dr, d_xr), "BSE kernels");
      double *rr = malloc(rb);
      if (!rr) die("host allocation", NULL);
      check(ctx, fbse_download(ctx, rr, d_dr, rb), "download");
      for (long k = 0; k < nx * nx; k++) hd[2 * k] = rr[k];
      check(ctx, fbse_download(ctx, rr, d_xr, rb), "download");
      for (long k = 0; k < nx * nx; k++) hx[2 * k] = rr[k];
      free(rr);
      fbse_free(ctx, d_pr);
      fbse_free(ctx, d_dr);
      fbse_free(ctx, d_xr);
      check(ctx, fbse_upload(ctx, d_dir, hd, mbytes), "upload");
      check(ctx, fbse_upload(ctx, d_exc, hx, mbytes), "upload");
      if (fbse_write_kernel_files(hd, hx, nh, ne, lumo, 1)) die("cannot write", "direct-0.dat / exchange-0.dat");
    } else {
      /* restartCoulomb = 1 continues an interrupted CPU run in the reference;
       * here the whole kernel is recomputed, which gives the same matrices */
      check(ctx, fbse_bse_kernel(ctx, d_psi, nh, ne, lumo, d_bare, d_scr, d_dir, d_exc), "BSE kernels");
      check(ctx, fbse_download(ctx, hd, d_dir, mbytes), "download");
      check(ctx, fbse_download(ctx, hx, d_exc, mbytes), "download");
      if (fbse_write_kernel_files(hd, hx, nh, ne, lumo, 0)) die("cannot write", "direct-0.dat / exchange-0.dat");
    }
    free(hd);
    free(hx);
    if (p.calc_coulomb_only) { /* mod_kernel.c:84-93 */
      printf("calcCoulombOnly: stopping after the kernels\n");
      fbse_destroy(ctx);
      return 0;
    }
  }
  double *ene = malloc(nx * sizeof(double)), *hx = malloc(nx * sizeof(double)), *dx = malloc(nx * sizeof(double));
  double *xx = malloc(nx * sizeof(double)), *h0x = malloc(nx * sizeof(double));
  check(ctx, fbse_bse_solve(ctx, eqp, nqp, nh, ne, lumo, d_dir, d_exc, ene, d_coef, hx, dx, xx, h0x), "BSE solve");
  write_matrices(ctx, d_dir, d_exc, d_coef, eqp, nh, ne, lumo, real);

  FILE *px = fopen("exciton.dat", "w"); /* bethe-salpeter.c:337-346 */
  if (!px) die("cannot write", "exciton.dat");
  fprintf(px, "#n \t E_n \t <H> \t <H_dir> \t <H_exc> \t <H_0> \t E_B (eV)\n");
  for (long i = 0; i < nx; i++)
    fprintf(px, "%ld % .12f % .12f % .12f  % .12f  % .12f  % .12f\n", i, ene[i], hx[i], dx[i], xx[i], h0x[i],
            (ene[i] - h0x[i]) * AUTOEV);
  fclose(px);

  double *mu = malloc((size_t)nx * 6 * sizeof(double)), *mx = malloc((size_t)nx * 6 * sizeof(double));
  check(ctx, fbse_bse_dipoles(ctx, d_psi, gx, gy, gz, nh, ne, lumo, mu), "transition dipoles");
  FILE *p0 = fopen("OS0.dat", "w"); /* dipole.c:61, 137-152 */
  if (!p0) die("cannot write", "OS0.dat");
  if (real) /* bse_real/dipole.c:61, 142-144: real components */
    fprintf(p0, "i  a   sqrt(mu2)     Ea-Ei \t  f_osc       mu_x        mu_y       mu_z\n");
  else
    fprintf(p0, "i  a   sqrt(mu2)     Ea-Ei \t  f_osc       mu_x.re     mu_x.im     mu_y.re     mu_y.im     mu_z.re     mu_z.im\n");
  for (long i = 0; i < nh; i++)
    for (long a = lumo; a < lumo + ne; a++) {
      const double *m = mu + (i * ne + (a - lumo)) * 6;
      const double e = eqp[a] - eqp[i];
      const double m2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2] + m[3] * m[3] + m[4] * m[4] + m[5] * m[5];
      if (real)
        fprintf(p0, "%ld % ld  %.8f %.12f % .8f % .8f % .8f % .8f\n", i, a, sqrt(m2), e, (2.0 / 3.0) * e * m2, m[0],
                m[2], m[4]);
      else
        fprintf(p0, "%ld % ld  %.8f %.12f % .8f % .8f % .8f % .8f % .8f % .8f % .8f\n", i, a, sqrt(m2), e,
                (2.0 / 3.0) * e * m2, m[0], m[1], m[2], m[3], m[4], m[5]);
    }
  fclose(p0);
  /* magnetic transition dipoles and rotational strengths of the pairs
   * (calc_mag_dipole, dipole.c:297-311, a-major; calc_rotational_strength,
   * dipole.c:333-370, i-major) */
  double *mg = malloc((size_t)nx * 6 * sizeof(double)), *mgx = malloc((size_t)nx * 6 * sizeof(double));
  check(ctx, fbse_bse_mag_dipoles(ctx, d_psi, gx, gy, gz, nh, ne, lumo, mg), "magnetic dipoles");
  FILE *pm0 = fopen("M0.dat", "w");
  if (!pm0) die("cannot write", "M0.dat");
  for (long a = lumo; a < lumo + ne; a++)
    for (long i = 0; i < nh; i++) {
      const double *m = mg + (i * ne + (a - lumo)) * 6;
      const double e = eqp[a] - eqp[i];
      const double ms = m[0] * m[0] + m[1] * m[1] + m[2] * m[2] + m[3] * m[3] + m[4] * m[4] + m[5] * m[5];
      fprintf(pm0, "%3ld %3ld  %+.8f %+.12f %+.8f %+.8f %+.8f %+.8f %+.8f %+.8f %+.8f\n", i, a, sqrt(ms), e,
              (4.0 / 3.0) * e * ms, m[0], m[1], m[2], m[3], m[4], m[5]);
    }
  fclose(pm0);
  FILE *pr0 = fopen("rs0.dat", "w");
  if (!pr0) die("cannot write", "rs0.dat");
  for (long i = 0; i < nh; i++)
    for (long a = lumo; a < lumo + ne; a++) {
      const long q = (i * ne + (a - lumo)) * 6;
      fprintf(pr0, "%ld %ld %.12f %.12g\n", i, a, eqp[a] - eqp[i], im_dot_conj(mu + q, mg + q));
    }
  fclose(pr0);
  check(ctx, fbse_bse_optical(ctx, d_coef, mu, nh, ne, mx), "exciton dipoles");
  check(ctx, fbse_bse_optical(ctx, d_coef, mg, nh, ne, mgx), "exciton magnetic dipoles");
  FILE *po = fopen("OS.dat", "w"); /* optical.c:72-75 */
  if (!po) die("cannot write", "OS.dat");
  for (long j = 0; j < nx; j++) {
    const double *m = mx + j * 6;
    const double os = m[0] * m[0] + m[1] * m[1] + m[2] * m[2] + m[3] * m[3] + m[4] * m[4] + m[5] * m[5];
    if (real) /* bse_real/optical.c:72-75: real parts */
      fprintf(po, "%ld % .8f % .8f % .8f % .12f % .12f % .12f\n", j, sqrt(os), ene[j], (2.0 / 3.0) * ene[j] * os, m[0],
              m[2], m[4]);
    else
      fprintf(po, "%ld % .8f % .8f % .8f % .12f % .12f % .12f % .12f % .12f % .12f\n", j, sqrt(os), ene[j],
              (2.0 / 3.0) * ene[j] * os, m[0], m[1], m[2], m[3], m[4], m[5]);
  }
  fclose(po);
  if (!real && fbse_write_qp_spins("qp_spins.dat", psi_host, eqp, nqp, o.ngrid, o.dx * o.dy * o.dz))
    die("cannot write", "qp_spins.dat");
  /* M.dat, rs.dat and bs-coeff-<j>.dat for j < 10 (optical.c:29-95) */
  FILE *pm = fopen("M.dat", "w"), *prs = fopen("rs.dat", "w");
  if (!pm || !prs) die("cannot write", "M.dat / rs.dat");
  for (long j = 0; j < nx; j++) {
    const double *m = mgx + j * 6;
    const double mos = m[0] * m[0] + m[1] * m[1] + m[2] * m[2] + m[3] * m[3] + m[4] * m[4] + m[5] * m[5];
    fprintf(pm, "%ld % .8f % .8f % .8f % .12f % .12f % .12f % .12f % .12f % .12f\n", j, sqrt(mos), ene[j],
            (4.0 / 3.0) * ene[j] * mos, m[0], m[1], m[2], m[3], m[4], m[5]);
    fprintf(prs, "%ld %.8f % .16f\n", j, ene[j], im_dot_conj(mx + j * 6, m));
  }
  fclose(pm);
  fclose(prs);
  {
    const long ncoef = nx < 10 ? nx : 10;
    double *cf = malloc((size_t)nx * nx * 2 * sizeof(double));
    if (!cf) die("host allocation", NULL);
    check(ctx, fbse_download(ctx, cf, d_coef, (size_t)nx * nx * 2 * sizeof(double)), "download");
    for (long j = 0; j < ncoef; j++) {
      char path[64];
      snprintf(path, sizeof path, "bs-coeff-%ld.dat", j);
      FILE *pc = fopen(path, "w");
      if (!pc) die("cannot write", path);
      for (long a = lumo, ibs = 0; a < lumo + ne; a++)
        for (long i = 0; i < nh; i++, ibs++) {
          const double *c = cf + 2 * (ibs * nx + j);
          fprintf(pc, "%ld %ld %.12lg %lg\n", i, a, eqp[a] - eqp[i], c[0] * c[0] + c[1] * c[1]);
        }
      fclose(pc);
    }
    if (p.calc_spin_ang_stat) {
      if (real)
        printf("calcSpinAngStat: the spin / angular statistics need spinor states; skipped\n");
      else
        write_ang_stats(ctx, d_psi, gx, gy, gz, nh, ne, lumo, cf);
    }
    free(cf);
  }
  printf("lowest exciton %.12f Ha, binding %.6f eV\n", ene[0], (ene[0] - h0x[0]) * AUTOEV);
  fbse_destroy(ctx);
  return 0;
}
