/*
 * fbse_oracle.c -- CPU restatement of FilterBSE's filter hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the reference restatement that the
 * CUDA path is compared against; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  Nothing in filterbse_gb300/ links or calls it.
 *
 * Every function restates one reference function in plain FP64 C, in the
 * reference's own loop order (so that sums round the same way), and cites the
 * reference file:line it follows (paths relative to the FilterBSE tree).  The
 * restatement is pinned against the reference's own compiled functions
 * (oracle/_ref, built by oracle/ref_build/Makefile) and against the golden
 * vectors under tests/golden/ by tests/test_oracle_pin.py.
 *
 * Data model (filter_mpi/fd.h:333-337, 382-398):
 *   complex arrays are interleaved (re, im) doubles; a spinor is the spin-up
 *   block of ngrid values followed by the spin-down block; grid index
 *   jxyz = nx*(ny*jz + jy) + jx.
 *   The projector table is passed as structure-of-arrays:
 *     nl[a]                      points of atom a
 *     jxyz[a*npts + g]           grid index
 *     y1[(a*npts + g)*6 + 2m+c]  Y_1m (c=0 re, 1 im), m = 0..2
 *     proj[(a*npts + g)*nproj+p] SO radial projector (already * sqrt(SO_par))
 *     nlp[(a*npts + g)*nproj+p]  NL radial projector
 *     sgn[a*nproj + p]           sign of the NL channel
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846
#define ORC_EPSDX 1.0e-20

/* ------------------------------------------------------------------------- */
/* Random numbers: L'Ecuyer two-generator combination with a Bays-Durham     */
/* shuffle table, with process-wide state, following filter_mpi/rand.c:22-62 */
/* ------------------------------------------------------------------------- */
static long g_s2 = 123456789; /* second generator; rand.c:26 initial value */
static long g_y = 0;
static long g_tab[32];

double orc_ran(long *seed)
{
  const long m1 = 2147483563, m2 = 2147483399;
  const long a1 = 40014, a2 = 40692, q1 = 53668, q2 = 52774, r1 = 12211, r2 = 3791;
  const long mm1 = m1 - 1, div = 1 + mm1 / 32;
  const double scale = 1.0 / (double)m1, top = 1.0 - 1.2e-7;
  long k;
  if (*seed <= 0) { /* (re)initialise: rand.c:31-42 */
    *seed = (-(*seed) < 1) ? 1 : -(*seed);
    g_s2 = *seed;
    for (long j = 32 + 7; j >= 0; j--) {
      k = *seed / q1;
      *seed = a1 * (*seed - k * q1) - k * r1;
      if (*seed < 0) *seed += m1;
      if (j < 32) g_tab[j] = *seed;
    }
    g_y = g_tab[0];
  }
  k = *seed / q1; /* rand.c:44-50 */
  *seed = a1 * (*seed - k * q1) - k * r1;
  if (*seed < 0) *seed += m1;
  k = g_s2 / q2;
  g_s2 = a2 * (g_s2 - k * q2) - k * r2;
  if (g_s2 < 0) g_s2 += m2;
  long j = g_y / div; /* rand.c:52-58 */
  g_y = g_tab[j] - g_s2;
  g_tab[j] = *seed;
  if (g_y < 1) g_y += mm1;
  double t = scale * (double)g_y;
  return (t > top) ? top : t;
}

/* Fills n draws and returns the updated seed (used for the seed-sequence pin). */
long orc_ran_fill(long seed, long n, double *out)
{
  for (long i = 0; i < n; i++) {
    double v = orc_ran(&seed);
    if (out) out[i] = v;
  }
  return seed;
}

/* init_psi (filter_mpi/init.c:1256-1307): values U[-1,1] over the grid in
 * jz, jy, jx order (two draws per point when complex), then normalise the
 * block to 1 with dv (norm.c:10-35, 42-79).  psi is interleaved complex.
 * Returns the updated seed. */
long orc_init_psi(double *psi, long seed, long ngrid, int is_complex, double dv)
{
  for (long j = 0; j < ngrid; j++) {
    psi[2 * j] = -1.0 + 2.0 * orc_ran(&seed);
    psi[2 * j + 1] = is_complex ? (-1.0 + 2.0 * orc_ran(&seed)) : 0.0;
  }
  double nrm = 0.0;
  for (long j = 0; j < ngrid; j++) nrm += psi[2 * j] * psi[2 * j] + psi[2 * j + 1] * psi[2 * j + 1];
  nrm = sqrt(nrm * dv);
  for (long j = 0; j < ngrid; j++) { psi[2 * j] /= nrm; psi[2 * j + 1] /= nrm; }
  return seed;
}

/* ------------------------------------------------------------------------- */
/* Newton interpolation: Leja-type sample points and divided differences     */
/* ------------------------------------------------------------------------- */

/* samp_points_ashkenazy (filter_mpi/coeff.c:227-293) with a zero imaginary
 * range: 32*ncheby candidates on [min,max] (the last eighth is the imaginary
 * segment, which collapses to 0), greedy maximisation of the summed log
 * distance.  Writes ncheby points (re, im) and returns the capacity estimate. */
double orc_samp_points(long ncheby, double mn, double mx, double *pre, double *pim)
{
  long nc3 = 32 * ncheby, imfrac = nc3 / 8;
  double range = 0.0, minim = range * mn, maxim = range * mx;
  double dsre = (mx - mn) / (double)(nc3 - 1 - imfrac);
  double dsim = (maxim - minim) / (double)(imfrac - 1);
  double *sre = calloc(nc3, sizeof(double)), *sim = calloc(nc3, sizeof(double));
  double *acc = calloc(nc3, sizeof(double));
  for (long j = 0; j < nc3 - imfrac; j++) sre[j] = mn + (double)j * dsre;
  for (long j = nc3 - imfrac; j < nc3; j++) sim[j] = minim + (double)(j - nc3 + imfrac) * dsim;
  pre[0] = sre[0];
  pim[0] = sim[0];
  for (long k = 0; k < nc3; k++) {
    double d = (sre[k] - pre[0]) * (sre[k] - pre[0]) + (sim[k] - pim[0]) * (sim[k] - pim[0]);
    acc[k] = (d < 1.0e-10) ? -1.0e30 : log(d);
  }
  for (long j = 1; j < ncheby; j++) {
    long best = 0;
    double fbest = -2.0e30;
    for (long k = 0; k < nc3; k++)
      if (acc[k] > fbest) { fbest = acc[k]; best = k; }
    pre[j] = sre[best];
    pim[j] = sim[best];
    for (long k = 0; k < nc3; k++) {
      double d = (sre[k] - pre[j]) * (sre[k] - pre[j]) + (sim[k] - pim[j]) * (sim[k] - pim[j]);
      if (d < 1.0e-10) acc[k] = -1.0e30;
      else acc[k] += log(d);
    }
  }
  double fk = 1.0;
  for (long j = 0; j < ncheby; j++) fk *= pre[j] * pre[j] + pim[j] * pim[j];
  fk = pow(sqrt(fk), 1.0 / (double)ncheby);
  free(sre);
  free(sim);
  free(acc);
  return fk;
}

/* gen_newton_coeff (filter_mpi/coeff.c:8-118): divided differences of the
 * Gaussian filter f(x) = sqrt(dt/pi) exp(-dt (x-E_t)^2) at the unscaled nodes
 * x = (z+2)/scale + Vmin, scale = 4/dE.  an is [m][ncheby] (re, im). */
void orc_newton_coeff(long ncheby, long m, const double *samp, const double *targets,
                      double vmin, double de, double dt, double *an)
{
  double scale = 4.0 / de;
  double pref = sqrt(dt / ORC_PI);
  for (long ie = 0; ie < m; ie++) {
    double *a = an + 2 * ncheby * ie;
    double x = (samp[0] + 2.0) / scale + vmin;
    a[0] = pref * exp(-(x - targets[ie]) * (x - targets[ie]) * dt);
    a[1] = 0.0;
    x = (samp[1] + 2.0) / scale + vmin;
    a[2] = (pref * exp(-(x - targets[ie]) * (x - targets[ie]) * dt) - a[0]) / (samp[1] - samp[0]);
    a[3] = (-a[1]) / (samp[1] - samp[0]);
    for (long j = 2; j < ncheby; j++) {
      double res = 1.0, sre = 0.0, sim = 0.0;
      for (long i = 1; i < j; i++) {
        res *= (samp[j] - samp[i - 1]);
        sre += a[2 * i] * res;
        sim += a[2 * i + 1] * res;
      }
      res *= (samp[j] - samp[j - 1]);
      x = (samp[j] + 2.0) / scale + vmin;
      a[2 * j] = (pref * exp(-(x - targets[ie]) * (x - targets[ie]) * dt) - a[0] - sre) / res;
      a[2 * j + 1] = (-a[1] - sim) / res;
    }
  }
}

/* ------------------------------------------------------------------------- */
/* Grid, k^2 table, energy targets                                          */
/* ------------------------------------------------------------------------- */

/* init_kvec (filter_mpi/init.c:1383-1394) followed by the per-axis 0.5 k^2/N
 * scaling of build_grid_ksqr (init.c:318-336). */
void orc_axis_ksqr(long n, double dk, double ngrid_1, double *k2)
{
  long npos = (n % 2 == 0) ? n / 2 : (n - 1) / 2;
  for (long j = 0; j < n; j++) k2[j] = 0.0;
  for (long j = 1; j <= npos; j++) {
    double v = (double)j * dk * 1.0;
    k2[j] = v;
    k2[n - j] = -v;
  }
  for (long j = 1; j < n; j++) k2[j] *= 0.5 * k2[j] * ngrid_1;
}

/* ksqr table (filter_mpi/init.c:338-351): x + y + z, capped at KE_max/N. */
void orc_ksqr(long nx, long ny, long nz, double dkx, double dky, double dkz, double ke_max, double *ksqr)
{
  double nx_1 = 1.0 / (double)nx, ny_1 = 1.0 / (double)ny, nz_1 = 1.0 / (double)nz;
  double ng_1 = nx_1 * ny_1 * nz_1;
  double *kx = malloc(nx * sizeof(double)), *ky = malloc(ny * sizeof(double)), *kz = malloc(nz * sizeof(double));
  orc_axis_ksqr(nx, dkx, ng_1, kx);
  orc_axis_ksqr(ny, dky, ng_1, ky);
  orc_axis_ksqr(nz, dkz, ng_1, kz);
  double kemax = ke_max * (ny_1 * nx_1 * nz_1);
  for (long jz = 0; jz < nz; jz++)
    for (long jy = 0; jy < ny; jy++)
      for (long jx = 0; jx < nx; jx++) {
        double v = kx[jx] + ky[jy] + kz[jz];
        ksqr[nx * (ny * jz + jy) + jx] = (v > kemax) ? kemax : v;
      }
  free(kx);
  free(ky);
  free(kz);
}

/* ------------------------------------------------------------------------- */
/* Local potential on the grid                                              */
/* ------------------------------------------------------------------------- */

/* interpolate (filter_mpi/interpolate.c:5-49) for short-ranged tables: linear
 * interpolation in a table of n rows (r_i, v_i); 0 beyond the table. */
static double orc_interp(double r, double dr, const double *vr, const double *pot, long n)
{
  long i = (long)(r / dr);
  if (i > n - 2) return 0.0;
  double a = 1.0 * (pot[i + 1] - pot[i]) / (vr[i + 1] - vr[i]);
  double b = 1.0 * pot[i] - vr[i] * a;
  return a * r + b;
}

/* build_local_pot (filter_mpi/init.c:481-703, non-interpolated, no strain,
 * no LR, no LSD): V(r) = sum over atoms of the atom type's radial table.
 * tables: type t has rows [toff[t], toff[t]+tlen[t]) in tr/tv, spacing tdr[t]. */
void orc_local_pot(long nx, long ny, long nz, const double *gx, const double *gy, const double *gz,
                   long natoms, const double *rx, const double *ry, const double *rz, const long *atype,
                   const double *tr, const double *tv, const long *toff, const long *tlen, const double *tdr,
                   double *pot)
{
  for (long jz = 0; jz < nz; jz++)
    for (long jy = 0; jy < ny; jy++)
      for (long jx = 0; jx < nx; jx++) {
        double sum = 0.0;
        for (long a = 0; a < natoms; a++) {
          double dx = gx[jx] - rx[a], dy = gy[jy] - ry[a], dz = gz[jz] - rz[a];
          double d = sqrt(dx * dx + dy * dy + dz * dz);
          long t = atype[a];
          sum += orc_interp(d, tdr[t], tr + toff[t], tv + toff[t], tlen[t]);
        }
        pot[nx * (ny * jz + jy) + jx] = sum;
      }
}

/* ------------------------------------------------------------------------- */
/* Projector radial functions (the eigensolve itself is done by the caller) */
/* ------------------------------------------------------------------------- */

static double orc_bessel1(double x, double x1)
{ /* calcBessel, filter_mpi/projectors.c:8 */
  return (x < 1e-10) ? 0.0 : (sin(x) * (x1 * x1) - cos(x) * x1);
}

/* The k-space integral matrix of gen_SO_projectors / gen_nlc_projectors
 * (filter_mpi/projectors.c:27-45, 117-135).  kind 0: SO Gaussian width 0.7;
 * kind 1: NL lam1 exp(-r^2) + lam2 exp(-(r-1.5)^2).  A is N x N row-major. */
void orc_proj_matrix(long N, double dx, double rcut, int kind, double lam1, double lam2, double *A)
{
  double kmax = 1.5 * ORC_PI / dx, dk = kmax / (double)N, dr = rcut / (double)N;
  /* The integrand factors are tabulated once; each product is then formed in
   * the reference's left-to-right order ((((r^2 J_i) w) J_j) dr), so the
   * sums round exactly as the inline evaluation does. */
  double *J = malloc((size_t)N * N * sizeof(double)), *w = malloc(N * sizeof(double));
  for (long i = 0; i < N; i++) {
    double ki = (double)i * dk;
    for (long rp = 1; rp < N; rp++) {
      double r = (double)rp * dr;
      J[i * N + rp] = orc_bessel1(ki * r, (1.00 / (ki * r + 1e-10)));
    }
  }
  for (long rp = 1; rp < N; rp++) {
    double r = (double)rp * dr;
    w[rp] = (kind == 0) ? exp(-1.0 * ((r / 0.7) * (r / 0.7)))
                        : (lam1 * exp(-1.0 * ((r / 1.0) * (r / 1.0))) + lam2 * exp(-(((r - 1.5) / 1.0) * ((r - 1.5) / 1.0))));
  }
  for (long i = 0; i < N; i++) {
    for (long j = 0; j <= i; j++) {
      double sum = 0.0;
      for (long rp = 1; rp < N; rp++) {
        double r = (double)rp * dr;
        sum += ((r * r) * J[i * N + rp] * w[rp] * J[j * N + rp] * dr);
      }
      A[i * N + j] = sum;
      A[j * N + i] = sum;
    }
  }
  free(J);
  free(w);
}

/* Radial projector on the r grid from eigenvector vec with eigenvalue |w|
 * (filter_mpi/projectors.c:62-78, 197-216). */
void orc_proj_radial(long N, double dx, double rcut, const double *vec, double w, double *out)
{
  double kmax = 1.5 * ORC_PI / dx, dk = kmax / (double)N, dr = rcut / (double)N;
  double pre = (2.00 / ORC_PI) * sqrt(w);
  for (long rp = 0; rp < N; rp++) {
    double r = (double)rp * dr, sum = 0.0;
    for (long kp = 0; kp < N; kp++) {
      double k = (double)kp * dk;
      sum += k * k * orc_bessel1(k * r, 1 / (k * r + 1e-10)) * vec[kp] * dk;
    }
    out[rp] = sum * pre;
  }
}

/* init_NL_projectors (filter_mpi/init.c:848-1135 of the reference tree;
 * loop body init.c:508-589): for each projector atom collect grid points with
 * r^2 < R_NLcut2 in jz, jy, jx order and store Y_1m, the SO radial projectors
 * scaled by sqrt(SO_par) and the NL radial projectors.  so_tab is [nproj][N],
 * nl_tab is [atom][nproj][N] (zeros for atoms without NL).  Returns the
 * number of points written per atom in nl[]. */
void orc_nlc_table(long nx, long ny, long nz, const double *gx, const double *gy, const double *gz,
                   long nat, const double *rx, const double *ry, const double *rz, const double *so_par,
                   double rcut2, long npts, long nproj, long N, const double *so_tab, const double *nl_tab,
                   long *nl, int *jxyz, double *y1, double *proj, double *nlp)
{
  double tmp1 = 0.5 * sqrt(3.0 / ORC_PI), tmp2 = 0.5 * sqrt(3.0 / (2.0 * ORC_PI));
  double drp = sqrt(rcut2) / (double)N;
  double *vr = malloc(N * sizeof(double));
  for (long i = 0; i < N; i++) vr[i] = (double)i * drp;
  for (long a = 0; a < nat; a++) {
    long cnt = 0;
    for (long jz = 0; jz < nz; jz++) {
      double dz = gz[jz] - rz[a], dzeps = dz + ORC_EPSDX;
      for (long jy = 0; jy < ny; jy++) {
        double dy = gy[jy] - ry[a], dyeps = dy + ORC_EPSDX;
        for (long jx = 0; jx < nx; jx++) {
          double dx = gx[jx] - rx[a], dxeps = dx + ORC_EPSDX;
          double dr2 = dx * dx + dy * dy + dz * dz;
          if (!(dr2 < rcut2)) continue;
          long e = a * npts + cnt;
          if (cnt >= npts) { cnt++; continue; }
          jxyz[e] = (int)(nx * (ny * jz + jy) + jx);
          double r_1 = 1.0 / sqrt(dx * dx + dy * dy + dzeps * dzeps);
          y1[e * 6 + 2] = tmp1 * dzeps * r_1;
          y1[e * 6 + 3] = 0.0;
          r_1 = 1.0 / sqrt(dxeps * dxeps + dy * dy + dz * dz);
          y1[e * 6 + 4] = -tmp2 * dxeps * r_1;
          y1[e * 6 + 0] = tmp2 * dxeps * r_1;
          r_1 = 1.0 / sqrt(dx * dx + dyeps * dyeps + dz * dz);
          y1[e * 6 + 5] = -tmp2 * dyeps * r_1;
          y1[e * 6 + 1] = -tmp2 * dyeps * r_1;
          for (long p = 0; p < nproj; p++) {
            proj[e * nproj + p] = orc_interp(sqrt(dr2), drp, vr, so_tab + N * p, N) * sqrt(so_par[a]);
            nlp[e * nproj + p] = orc_interp(sqrt(dr2), drp, vr, nl_tab + (a * nproj + p) * N, N);
          }
          cnt++;
        }
      }
    }
    nl[a] = cnt;
  }
  free(vr);
}

/* ------------------------------------------------------------------------- */
/* Potential part of H: SO + NL projectors + local potential                */
/* ------------------------------------------------------------------------- */

/* def_LS (filter_mpi/hamiltonian.c:312-442): L.S in the flattened (s, m)
 * basis j = 3 s + m, stored LS[j' * 6 + j] (re, im). */
void orc_def_LS(double *LS)
{
  double h = sqrt(0.5);
  /* L_x, L_y, L_z for l = 1 in the m = -1, 0, +1 ordering and S = sigma/2 */
  double Lre[3][3][3] = {{{0, h, 0}, {h, 0, h}, {0, h, 0}},
                         {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}},
                         {{-1, 0, 0}, {0, 0, 0}, {0, 0, 1}}};
  double Lim[3][3][3] = {{{0, 0, 0}, {0, 0, 0}, {0, 0, 0}},
                         {{0, h, 0}, {-h, 0, h}, {0, -h, 0}},
                         {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}};
  double Sre[3][2][2] = {{{0, 0.5}, {0.5, 0}}, {{0, 0}, {0, 0}}, {{0.5, 0}, {0, -0.5}}};
  double Sim[3][2][2] = {{{0, 0}, {0, 0}}, {{0, -0.5}, {0.5, 0}}, {{0, 0}, {0, 0}}};
  for (int jp = 0; jp < 6; jp++) {
    int sp = jp / 3, mp = jp % 3;
    for (int j = 0; j < 6; j++) {
      int s = j / 3, m = j % 3;
      double re = 0.0, im = 0.0;
      for (int c = 0; c < 3; c++) {
        re += Lre[c][m][mp] * Sre[c][s][sp] - Lim[c][m][mp] * Sim[c][s][sp];
        im += Lre[c][m][mp] * Sim[c][s][sp] + Lim[c][m][mp] * Sre[c][s][sp];
      }
      LS[2 * (jp * 6 + j)] = re;
      LS[2 * (jp * 6 + j) + 1] = im;
    }
  }
}

/* p_spin_orbit_proj_pot (filter_mpi/phamiltonian.c:140-312, k = 0):
 * out += sum_atoms sum_p sum_{j',j} b_p Y_m LS[j',j] dv <b_p Y_m'|psi_s'>. */
void orc_apply_so(double *out, const double *psi, long ngrid, long nat, const long *nl, long npts, long nproj,
                  const int *jxyz, const double *y1, const double *proj, const double *LS, double dv)
{
  for (long a = 0; a < nat; a++) {
    for (long p = 0; p < nproj; p++) {
      for (int jp = 0; jp < 6; jp++) {
        int sp = jp / 3, mp = jp % 3;
        double pre = 0.0, pim = 0.0;
        for (long g = 0; g < nl[a]; g++) {
          long e = a * npts + g;
          long r = jxyz[e] + ngrid * sp;
          double yr = y1[e * 6 + 2 * mp], yi = y1[e * 6 + 2 * mp + 1], b = proj[e * nproj + p];
          pre += b * (psi[2 * r] * yr + psi[2 * r + 1] * yi);
          pim += b * (psi[2 * r + 1] * yr - psi[2 * r] * yi);
        }
        pre *= dv;
        pim *= dv;
        for (int j = 0; j < 6; j++) {
          double lr = LS[2 * (jp * 6 + j)], li = LS[2 * (jp * 6 + j) + 1];
          if (lr == 0.0 && li == 0.0) continue;
          int s = j / 3, m = j % 3;
          double qr = lr * pre - li * pim, qi = lr * pim + li * pre;
          for (long g = 0; g < nl[a]; g++) {
            long e = a * npts + g;
            long r = jxyz[e] + ngrid * s;
            double yr = y1[e * 6 + 2 * m], yi = y1[e * 6 + 2 * m + 1], b = proj[e * nproj + p];
            out[2 * r] += b * (yr * qr - yi * qi);
            out[2 * r + 1] += b * (yr * qi + yi * qr);
          }
        }
      }
    }
  }
}

/* p_nonlocal_proj_pot (filter_mpi/phamiltonian.c:316-444, k = 0): block
 * diagonal in spin, sign per (atom, projector). */
void orc_apply_nl(double *out, const double *psi, long ngrid, int nspin, long nat, const long *nl, long npts,
                  long nproj, const int *jxyz, const double *y1, const double *nlp, const int *sgn, double dv)
{
  for (long a = 0; a < nat; a++) {
    for (long p = 0; p < nproj; p++) {
      for (int s = 0; s < nspin; s++) {
        for (int m = 0; m < 3; m++) {
          double pre = 0.0, pim = 0.0;
          for (long g = 0; g < nl[a]; g++) {
            long e = a * npts + g;
            long r = jxyz[e] + ngrid * s;
            double yr = y1[e * 6 + 2 * m], yi = y1[e * 6 + 2 * m + 1], b = nlp[e * nproj + p];
            pre += b * (psi[2 * r] * yr + psi[2 * r + 1] * yi);
            pim += b * (psi[2 * r + 1] * yr - psi[2 * r] * yi);
          }
          int sg = sgn[a * nproj + p];
          pre *= sg * dv;
          pim *= sg * dv;
          for (long g = 0; g < nl[a]; g++) {
            long e = a * npts + g;
            long r = jxyz[e] + ngrid * s;
            double yr = y1[e * 6 + 2 * m], yi = y1[e * 6 + 2 * m + 1], b = nlp[e * nproj + p];
            out[2 * r] += b * (yr * pre - yi * pim);
            out[2 * r + 1] += b * (yr * pim + yi * pre);
          }
        }
      }
    }
  }
}

/* local part of p_potential (filter_mpi/phamiltonian.c:121-132):
 * out += V psi over the spinor (V repeated for each spin block). */
void orc_apply_vloc(double *out, const double *psi, const double *pot, long ngrid, int nspin, int is_complex)
{
  for (long j = 0; j < nspin * ngrid; j++) {
    double v = pot[j % ngrid];
    out[2 * j] += v * psi[2 * j];
    if (is_complex) out[2 * j + 1] += v * psi[2 * j + 1];
  }
}

/* p_hnorm's scale-and-shift (filter_mpi/filter.c:401-407). */
void orc_hnorm_shift(double *hpsi, const double *psi, long n, double de_1, double vmin, double zn)
{
  double c = 2.0 + zn + vmin * de_1;
  for (long j = 0; j < n; j++) {
    hpsi[2 * j] = de_1 * hpsi[2 * j] - c * psi[2 * j];
    hpsi[2 * j + 1] = de_1 * hpsi[2 * j + 1] - c * psi[2 * j + 1];
  }
}
