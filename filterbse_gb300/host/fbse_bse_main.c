/* fbse_bse: drop-in for the reference's bse executable (bse_cplx).
 *
 * Reads input.par and the filter's output.dat from the working directory
 * (bse_cplx/read.c, save.c), picks the quasiparticle basis as
 * get_qp_basis_indices does (bse_cplx/basis.c:7-254), and runs the BSE stage
 * on one GPU through libfbse_gpu: Coulomb potentials (init.c), direct and
 * exchange kernels (coulomb.c), the BSE eigensolve with its expectation
 * values (mod_bse.c, bethe-salpeter.c), pair and exciton transition dipoles
 * (dipole.c, optical.c).  Writes BSEeval.par, exciton.dat, OS0.dat and OS.dat
 * in the reference's formats.  Errors go to stderr with EXIT_FAILURE. */
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

int main(void)
{
  char err[512];
  fbse_bse_params p;
  if (fbse_read_bse_params("input.par", &p, err, sizeof err)) die(err, NULL);
  output_dat o;
  read_output("output.dat", &o);
  if (o.complex_idx != 2 || o.nspin != 2) die("the complex BSE needs spinor filter output (bse_cplx)", NULL);

  /* get_qp_basis_indices (bse_cplx/basis.c:7-254) */
  long *hole = malloc(o.mn * sizeof(long)), *elec = malloc(o.mn * sizeof(long)), nh = 0, ne = 0;
  for (long i = 0; i < o.mn; i++) {
    if (o.sigma[i] < p.sigma_e_cut && o.eval[i] < p.fermi_e) hole[nh++] = i;
    if (o.sigma[i] < p.sigma_e_cut && o.eval[i] > p.fermi_e) elec[ne++] = i;
  }
  if (nh < 1 || ne < 1) die("no converged hole or electron states below/above fermiEnergy", NULL);
  long h0 = 0;
  if (p.max_hole_states != -1 && nh > p.max_hole_states) {
    h0 = nh - p.max_hole_states; /* keep the holes closest to the gap */
    nh = p.max_hole_states;
  }
  if (p.max_elec_states != -1 && ne > p.max_elec_states) ne = p.max_elec_states;
  const long nqp = nh + ne, lumo = nh, nx = nh * ne;
  double *eqp = malloc(nqp * sizeof(double));
  long *sel = malloc(nqp * sizeof(long));
  for (long i = 0; i < nh; i++) sel[i] = hole[h0 + i];
  for (long i = 0; i < ne; i++) sel[nh + i] = elec[i];
  FILE *fe = fopen("BSEeval.par", "w");
  for (long i = 0; i < nqp; i++) {
    eqp[i] = o.eval[sel[i]];
    if (fe) fprintf(fe, "%ld % .12f %g\n", i, eqp[i], o.sigma[sel[i]]);
  }
  if (fe) fclose(fe);
  printf("fbse_bse: %ld holes, %ld electrons, %ld excitons; gap %.6g Ha\n", nh, ne, nx, eqp[lumo] - eqp[lumo - 1]);

  /* the basis states (get_qp_basis, basis.c:258-300) */
  const long stlen = 2 * o.nspinngrid; /* doubles per complex spinor state */
  double *psi_host = malloc((size_t)nqp * stlen * sizeof(double));
  FILE *f = fopen("output.dat", "rb");
  if (!f || !psi_host) die("cannot read states from", "output.dat");
  for (long i = 0; i < nqp; i++) {
    if (fseek(f, o.psi_pos + sel[i] * stlen * (long)sizeof(double), SEEK_SET) ||
        fread(psi_host + i * stlen, sizeof(double), stlen, f) != (size_t)stlen)
      die("truncated states in", "output.dat");
  }
  fclose(f);

  /* context: the grid only (no potential / projectors are used by the BSE) */
  fbse_grid_desc gd;
  memset(&gd, 0, sizeof gd);
  gd.nx = o.nx; gd.ny = o.ny; gd.nz = o.nz;
  gd.dx = o.dx; gd.dy = o.dy; gd.dz = o.dz;
  gd.ke_max = o.ke_max;
  gd.nspin = 2;
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
  check(ctx, fbse_bse_kernel(ctx, d_psi, nh, ne, lumo, d_bare, d_scr, d_dir, d_exc), "BSE kernels");
  double *ene = malloc(nx * sizeof(double)), *hx = malloc(nx * sizeof(double)), *dx = malloc(nx * sizeof(double));
  double *xx = malloc(nx * sizeof(double)), *h0x = malloc(nx * sizeof(double));
  check(ctx, fbse_bse_solve(ctx, eqp, nqp, nh, ne, lumo, d_dir, d_exc, ene, d_coef, hx, dx, xx, h0x), "BSE solve");

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
  fprintf(p0, "i  a   sqrt(mu2)     Ea-Ei \t  f_osc       mu_x.re     mu_x.im     mu_y.re     mu_y.im     mu_z.re     mu_z.im\n");
  for (long i = 0; i < nh; i++)
    for (long a = lumo; a < lumo + ne; a++) {
      const double *m = mu + (i * ne + (a - lumo)) * 6;
      const double e = eqp[a] - eqp[i];
      const double m2 = m[0] * m[0] + m[1] * m[1] + m[2] * m[2] + m[3] * m[3] + m[4] * m[4] + m[5] * m[5];
      fprintf(p0, "%ld % ld  %.8f %.12f % .8f % .8f % .8f % .8f % .8f % .8f % .8f\n", i, a, sqrt(m2), e,
              (2.0 / 3.0) * e * m2, m[0], m[1], m[2], m[3], m[4], m[5]);
    }
  fclose(p0);
  check(ctx, fbse_bse_optical(ctx, d_coef, mu, nh, ne, mx), "exciton dipoles");
  FILE *po = fopen("OS.dat", "w"); /* optical.c:72-75 */
  if (!po) die("cannot write", "OS.dat");
  for (long j = 0; j < nx; j++) {
    const double *m = mx + j * 6;
    const double os = m[0] * m[0] + m[1] * m[1] + m[2] * m[2] + m[3] * m[3] + m[4] * m[4] + m[5] * m[5];
    fprintf(po, "%ld % .8f % .8f % .8f % .12f % .12f % .12f % .12f % .12f % .12f\n", j, sqrt(os), ene[j],
            (2.0 / 3.0) * ene[j] * os, m[0], m[1], m[2], m[3], m[4], m[5]);
  }
  fclose(po);
  printf("lowest exciton %.12f Ha, binding %.6f eV\n", ene[0], (ene[0] - h0x[0]) * AUTOEV);
  fbse_destroy(ctx);
  return 0;
}
