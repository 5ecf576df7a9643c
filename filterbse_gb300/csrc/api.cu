// C-ABI entry points of libfbse_gpu (declared in include/fbse.h).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "fbse_internal.cuh"

namespace fbse {

std::atomic<long> g_launches{0};

int set_err(fbse_ctx *c, int code, const std::string &msg)
{
  if (c) c->err = msg;
  return code;
}

int check_dev_status(fbse_ctx *c)
{
  int h[4] = {0, 0, 0, 0};
  if (!c->dstatus) return FBSE_OK;
  if (d2h(c->stream, h, c->dstatus, sizeof(h)) != cudaSuccess) return set_err(c, FBSE_ERR_CUDA, "status read");
  if (h[0]) {
    cudaMemsetAsync(c->dstatus, 0, sizeof(h), c->stream);
    return set_err(c, FBSE_ERR_NOCONV, "a kernel's bounded wait for its staged data timed out");
  }
  return FBSE_OK;
}

int ensure(fbse_ctx *c, void **p, size_t *have, size_t need)
{
  if (*have >= need && *p) return FBSE_OK;
  if (*p) {
    cudaStreamSynchronize(c->stream);
    cudaFree(*p);
    *p = nullptr;
    *have = 0;
  }
  if (need == 0) return FBSE_OK;
  if (cudaMalloc(p, need) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return set_err(c, FBSE_ERR_OOM, "device allocation of " + std::to_string(need) + " bytes failed");
  }
  *have = need;
  return FBSE_OK;
}

int newton_filter(fbse_ctx *c, const double *zn, const double *an, long ncheby, long m, double vmin, double de,
                  const double *psi0, long nstart, double *filtered);
int normalize_all(fbse_ctx *c, double *psitot, long n, double *norms);
int energy_all(fbse_ctx *c, const double *psitot, long n, double *ene, double *sigma);
int energy_range(fbse_ctx *c, long seed, long max_iter, double *emin, double *emax, long *iters);
int ortho_diag_sigma(fbse_ctx *c, double *psitot, long n, long *n_kept, double *eval, double *sigma);
int gram_slab(fbse_ctx *c, const double *A, long na, const double *B, long nb, long off, long len, double *out_host);
int rotate_slab(fbse_ctx *c, const double *A, long na, const double *C_host, long k, long off, long len, double *out);

// per-axis 0.5 k^2 / N exactly as init_kvec + build_grid_ksqr
// (filter_mpi/init.c:1383-1394, 318-336)
static void axis_k2(long n, double dk, double ngrid_1, std::vector<double> &k)
{
  k.assign(n, 0.0);
  long npos = (n % 2 == 0) ? n / 2 : (n - 1) / 2;
  for (long j = 1; j <= npos; j++) {
    double v = (double)j * dk * 1.0;
    k[j] = v;
    k[n - j] = -v;
  }
  for (long j = 1; j < n; j++) k[j] *= 0.5 * k[j] * ngrid_1;
}

template <typename D, typename S> static int upload(fbse_ctx *c, D **dst, const S *src, size_t n)
{
  std::vector<D> tmp(n);
  for (size_t i = 0; i < n; i++) tmp[i] = (D)src[i];
  FBSE_CUDA(c, cudaMalloc(dst, n * sizeof(D) + 16));
  FBSE_CUDA(c, cudaMemcpy(*dst, tmp.data(), n * sizeof(D), cudaMemcpyHostToDevice));
  return FBSE_OK;
}

// plane-major projector table of the projector-fused plane passes (hpsi_fused.cuh),
// built from the point-major table (covered points cj in increasing grid index,
// entries cb[k] .. cb[k+1]-1 of point k in increasing atom order, per entry
// its atom pa, Y_1m py[(m nent + e) 2 + re/im] and radial values ps / pn
// [q nent + e]).  Per plane z: the atoms whose spheres meet it (slots), its
// entries ordered by (layer = rank of the atom among the point's atoms, slot,
// grid point), the layer offsets, and segments of at most kSegMax entries of
// one (layer, slot) for the gather; per atom its segments in plane order.
// Leaves fz_ok = 0 (the separate kernels then run) when the grid, the
// precision or the table does not fit the kernel.
static int build_plane_table(fbse_ctx *c, const std::vector<int> &cj, const std::vector<int> &cb,
                             const std::vector<int> &pa, const std::vector<double> &py, const std::vector<double> &ps,
                             const std::vector<double> &pn, size_t nent)
{
  ProjDev &p = c->proj;
  p.fz_ok = 0;
  const long NX = kPipeN;
  if (c->precision != FBSE_MIXED || c->nx != NX || c->ny != NX || nent == 0)
    return FBSE_OK;
  for (size_t k = 0; k < nent; k++) {
    const double y0 = py[2 * k], y1 = py[2 * k + 1];
    if (py[(nent + k) * 2 + 1] != 0.0 || py[(2 * nent + k) * 2] != -y0 || py[(2 * nent + k) * 2 + 1] != y1)
      return FBSE_OK;
  }
  const long nz = c->nz, nxy = NX * NX;
  const int kPA = kPipePlaneAtoms, kML = kPipeMaxLayers, kSM = kPipeSegMax;
  std::vector<unsigned> ent;
  std::vector<float> fy[3], fso(nent * p.nproj), fnl(nent * p.nproj);
  std::vector<int> lay(nz * (kML + 1), 0), atoms(nz * kPA, -1), natoms(nz, 0), seg_beg, plane_seg(nz + 1, 0), seg_atom;
  ent.reserve(nent);
  for (auto &v : fy) v.reserve(nent);
  struct Item { int layer, slot, j, e; };
  size_t k = 0;
  for (long z = 0; z < nz; z++) {
    size_t k1 = k;
    while (k1 < cj.size() && cj[k1] / nxy == z) k1++;
    std::vector<int> at;
    for (int e = cb[k]; e < cb[k1]; e++) at.push_back(pa[e]);
    std::sort(at.begin(), at.end());
    at.erase(std::unique(at.begin(), at.end()), at.end());
    if ((int)at.size() > kPA) return FBSE_OK;
    natoms[z] = (int)at.size();
    for (size_t s = 0; s < at.size(); s++) atoms[z * kPA + s] = at[s];
    std::vector<Item> it;
    for (size_t q = k; q < k1; q++)
      for (int e = cb[q]; e < cb[q + 1]; e++) {
        if (e - cb[q] >= kML) return FBSE_OK;
        const int s = (int)(std::lower_bound(at.begin(), at.end(), pa[e]) - at.begin());
        it.push_back({e - cb[q], s, cj[q], e});
      }
    std::sort(it.begin(), it.end(), [](const Item &x, const Item &y) {
      return x.layer != y.layer ? x.layer < y.layer : x.slot != y.slot ? x.slot < y.slot : x.j < y.j;
    });
    plane_seg[z] = (int)seg_beg.size();
    const int base = (int)ent.size();
    for (int L = 0; L <= kML; L++) {
      size_t i = 0;
      while (i < it.size() && it[i].layer < L) i++;
      lay[z * (kML + 1) + L] = base + (int)i;
    }
    for (size_t i = 0; i < it.size(); i++) {
      const Item &x = it[i];
      const bool start = i == 0 || x.layer != it[i - 1].layer || x.slot != it[i - 1].slot ||
                         (int)ent.size() - seg_beg.back() >= kSM;
      if (start) {
        seg_beg.push_back((int)ent.size());
        seg_atom.push_back(at[x.slot]);
      }
      const int xy = x.j % (int)nxy;
      ent.push_back((unsigned)(xy % NX) | ((unsigned)(xy / NX) << 7) | ((unsigned)x.slot << 16));
      fy[0].push_back((float)py[2 * x.e]);
      fy[1].push_back((float)py[2 * x.e + 1]);
      fy[2].push_back((float)py[(nent + x.e) * 2]);
      const size_t o = ent.size() - 1;
      for (int q = 0; q < p.nproj; q++) {
        fso[q * nent + o] = (float)ps[q * nent + x.e];
        fnl[q * nent + o] = (float)pn[q * nent + x.e];
      }
    }
    k = k1;
  }
  plane_seg[nz] = (int)seg_beg.size();
  const long nseg = (long)seg_beg.size();
  seg_beg.push_back((int)ent.size());
  // atom -> segments (stable counting sort keeps plane order)
  std::vector<int> aseg_beg(p.nat + 1, 0), aseg(nseg ? nseg : 1, 0);
  for (long s = 0; s < nseg; s++) aseg_beg[seg_atom[s] + 1]++;
  for (long a = 0; a < p.nat; a++) aseg_beg[a + 1] += aseg_beg[a];
  {
    std::vector<int> fill(aseg_beg.begin(), aseg_beg.end() - 1);
    for (long s = 0; s < nseg; s++) aseg[fill[seg_atom[s]]++] = (int)s;
  }
  std::vector<float> fyall;
  fyall.reserve(3 * nent);
  for (auto &v : fy) fyall.insert(fyall.end(), v.begin(), v.end());
  int rc;
  if ((rc = upload(c, &p.fz_ent, ent.data(), ent.size()))) return rc;
  if ((rc = upload(c, &p.fz_y, fyall.data(), fyall.size()))) return rc;
  if ((rc = upload(c, &p.fz_so, fso.data(), fso.size()))) return rc;
  if ((rc = upload(c, &p.fz_nl, fnl.data(), fnl.size()))) return rc;
  if ((rc = upload(c, &p.fz_lay, lay.data(), lay.size()))) return rc;
  if ((rc = upload(c, &p.fz_atoms, atoms.data(), atoms.size()))) return rc;
  if ((rc = upload(c, &p.fz_natoms, natoms.data(), natoms.size()))) return rc;
  if ((rc = upload(c, &p.fz_seg_beg, seg_beg.data(), seg_beg.size()))) return rc;
  if ((rc = upload(c, &p.fz_plane_seg, plane_seg.data(), plane_seg.size()))) return rc;
  if ((rc = upload(c, &p.fz_aseg_beg, aseg_beg.data(), aseg_beg.size()))) return rc;
  if ((rc = upload(c, &p.fz_aseg, aseg.data(), aseg.size()))) return rc;
  p.fz_nent = (long)nent;
  p.fz_nseg = nseg;
  p.fz_ok = 1;
  return FBSE_OK;
}

static void def_LS(double *ls)
{  // def_LS (filter_mpi/hamiltonian.c:312-442): L.S in the flattened (s, m) basis
  const double h = std::sqrt(0.5);
  const double Lre[3][3][3] = {{{0, h, 0}, {h, 0, h}, {0, h, 0}}, {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}},
                               {{-1, 0, 0}, {0, 0, 0}, {0, 0, 1}}};
  const double Lim[3][3][3] = {{{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, {{0, h, 0}, {-h, 0, h}, {0, -h, 0}},
                               {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}};
  const double Sre[3][2][2] = {{{0, 0.5}, {0.5, 0}}, {{0, 0}, {0, 0}}, {{0.5, 0}, {0, -0.5}}};
  const double Sim[3][2][2] = {{{0, 0}, {0, 0}}, {{0, -0.5}, {0.5, 0}}, {{0, 0}, {0, 0}}};
  for (int jp = 0; jp < 6; jp++)
    for (int j = 0; j < 6; j++) {
      int sp = jp / 3, mp = jp % 3, s = j / 3, m = j % 3;
      double re = 0, im = 0;
      for (int k = 0; k < 3; k++) {
        re += Lre[k][m][mp] * Sre[k][s][sp] - Lim[k][m][mp] * Sim[k][s][sp];
        im += Lre[k][m][mp] * Sim[k][s][sp] + Lim[k][m][mp] * Sre[k][s][sp];
      }
      ls[2 * (jp * 6 + j)] = re;
      ls[2 * (jp * 6 + j) + 1] = im;
    }
}

static int create(fbse_ctx *c, const fbse_grid_desc *g, const double *pot, const fbse_proj_desc *pj)
{
  if (g->nx < 1 || g->ny < 1 || g->nz < 1) return set_err(c, FBSE_ERR_ARG, "grid sizes must be positive");
  if (g->nspin != 1 && g->nspin != 2) return set_err(c, FBSE_ERR_ARG, "nspin must be 1 or 2");
  if (g->so && (g->nspin != 2 || !g->is_complex))
    return set_err(c, FBSE_ERR_ARG, "spin-orbit requires complex spinors (read.c:914-921)");
  if (g->nspin == 2 && !g->is_complex) return set_err(c, FBSE_ERR_ARG, "spinors must be complex");
  if ((g->so || g->nl) && !pj) return set_err(c, FBSE_ERR_ARG, "projector table required when SO or NL is on");
  if (!pot) return set_err(c, FBSE_ERR_ARG, "local potential required");
  if ((double)g->nx * g->ny * g->nz > 2147483647.0) return set_err(c, FBSE_ERR_UNSUPPORTED, "grid too large");
  c->nx = g->nx; c->ny = g->ny; c->nz = g->nz;
  c->ngrid = g->nx * g->ny * g->nz;
  c->nspin = g->nspin; c->is_complex = g->is_complex ? 1 : 0; c->so = g->so ? 1 : 0; c->nl = g->nl ? 1 : 0;
  c->dx = g->dx; c->dy = g->dy; c->dz = g->dz;
  c->dv = g->dx * g->dy * g->dz;
  c->ke_max = g->ke_max;
  const double nx_1 = 1.0 / (double)g->nx, ny_1 = 1.0 / (double)g->ny, nz_1 = 1.0 / (double)g->nz;
  const double ng_1 = nx_1 * ny_1 * nz_1;
  c->kemax_scaled = g->ke_max * (ny_1 * nx_1 * nz_1);
  FBSE_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  FBSE_CUDA(c, cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
  for (int k = 0; k < fbse_ctx::kSide; k++) {
    FBSE_CUDA(c, cudaStreamCreateWithFlags(&c->side[k], cudaStreamNonBlocking));
    FBSE_CUDA(c, cudaEventCreateWithFlags(&c->ev_join[k], cudaEventDisableTiming));
  }
  FBSE_CUDA(c, cudaMalloc(&c->dstatus, 4 * sizeof(int)));
  FBSE_CUDA(c, cudaMemset(c->dstatus, 0, 4 * sizeof(int)));
  int rc;
  if ((rc = plan_axis(c, c->ax[0], (int)g->nx))) return rc;
  if ((rc = plan_axis(c, c->ax[1], (int)g->ny))) return rc;
  if ((rc = plan_axis(c, c->ax[2], (int)g->nz))) return rc;
  // reciprocal spacing: box = n d (even n) or (n - 1) d (odd n)  (init.c:65-80)
  const long ns[3] = {g->nx, g->ny, g->nz};
  const double ds[3] = {g->dx, g->dy, g->dz};
  double **dst[3] = {&c->k2x, &c->k2y, &c->k2z};
  float **dstf[3] = {&c->k2xf, &c->k2yf, &c->k2zf};
  const double dkin[3] = {g->dkx, g->dky, g->dkz};
  for (int a = 0; a < 3; a++) {
    const double box = (ns[a] % 2 == 0) ? (double)ns[a] * ds[a] : (double)(ns[a] - 1) * ds[a];
    const double dk = dkin[a] > 0 ? dkin[a] : 6.28318530717958647692 / box;
    c->dk[a] = dk;
    std::vector<double> k;
    axis_k2(ns[a], dk, ng_1, k);
    if ((rc = upload(c, dst[a], k.data(), k.size()))) return rc;
    if ((rc = upload(c, dstf[a], k.data(), k.size()))) return rc;
  }
  if ((rc = upload(c, &c->pot64, pot, c->ngrid))) return rc;
  if ((rc = upload(c, &c->pot32, pot, c->ngrid))) return rc;
  c->vpot_min = 1e300; c->vpot_max = -1e300;
  for (long i = 0; i < c->ngrid; i++) {
    c->vpot_min = std::fmin(c->vpot_min, pot[i]);
    c->vpot_max = std::fmax(c->vpot_max, pot[i]);
  }
  if ((g->so || g->nl) && pj) {
    ProjDev &p = c->proj;
    if (pj->n_atoms < 0 || pj->npts < 1 || pj->nproj < 1 || pj->nproj > 5)
      return set_err(c, FBSE_ERR_ARG, "projector table: n_atoms >= 0, npts >= 1, 1 <= nproj <= 5");
    p.nat = pj->n_atoms; p.npts = pj->npts; p.nproj = pj->nproj; p.so = c->so; p.nl = c->nl;
    const size_t ne = (size_t)p.nat * p.npts;
    std::vector<int> cnt(p.nat > 0 ? p.nat : 1);
    for (long a = 0; a < p.nat; a++) {
      if (pj->nl[a] < 0 || pj->nl[a] > p.npts) return set_err(c, FBSE_ERR_ARG, "projector table: nl[a] > npts");
      cnt[a] = (int)pj->nl[a];
      for (long e = 0; e < pj->nl[a]; e++) {
        const int j = pj->jxyz[a * p.npts + e];
        if (j < 0 || j >= c->ngrid) return set_err(c, FBSE_ERR_ARG, "projector table: grid index out of range");
      }
    }
    // entries beyond nl[a] are never read; zero-fill copies keep them finite.
    // Device layout is structure-of-arrays so that a warp reading 32
    // consecutive entries issues one coalesced load per quantity:
    //   y1[(m*ne + i)*2 + {re, im}],  so/nl[p*ne + i]   (i = a*npts + e)
    std::vector<int> jx(ne, 0);
    std::vector<double> y1(ne * 6, 0.0), so(ne * p.nproj, 0.0), nlr(ne * p.nproj, 0.0);
    for (long a = 0; a < p.nat; a++)
      for (long e = 0; e < pj->nl[a]; e++) {
        const size_t i = a * p.npts + e;
        jx[i] = pj->jxyz[i];
        for (int m = 0; m < 3; m++)
          for (int k = 0; k < 2; k++) y1[(m * ne + i) * 2 + k] = pj->y1[i * 6 + 2 * m + k];
        for (int k = 0; k < p.nproj; k++) {
          so[k * ne + i] = pj->so_proj ? pj->so_proj[i * p.nproj + k] : 0.0;
          nlr[k * ne + i] = pj->nl_proj ? pj->nl_proj[i * p.nproj + k] : 0.0;
        }
      }
    std::vector<int> sg((size_t)(p.nat > 0 ? p.nat : 1) * p.nproj, 0);
    if (pj->nl_sign)
      for (size_t i = 0; i < (size_t)p.nat * p.nproj; i++) sg[i] = pj->nl_sign[i];
    double ls[72];
    if (pj->LS) std::memcpy(ls, pj->LS, sizeof(ls));
    else def_LS(ls);
    if ((rc = upload(c, &p.nl_cnt, cnt.data(), cnt.size()))) return rc;
    if ((rc = upload(c, &p.jxyz, jx.data(), jx.size() ? jx.size() : 1))) return rc;
    if ((rc = upload(c, &p.y1, y1.data(), y1.size()))) return rc;
    if ((rc = upload(c, &p.sop, so.data(), so.size()))) return rc;
    if ((rc = upload(c, &p.nlp, nlr.data(), nlr.size()))) return rc;
    if ((rc = upload(c, &p.y1f, y1.data(), y1.size()))) return rc;
    if ((rc = upload(c, &p.sopf, so.data(), so.size()))) return rc;
    if ((rc = upload(c, &p.nlpf, nlr.data(), nlr.size()))) return rc;
    if ((rc = upload(c, &p.sgn, sg.data(), sg.size()))) return rc;
    // point-major copy (counting sort by grid index; entries of one point in
    // increasing atom order because atoms are visited in order)
    {
      size_t nent = 0;
      for (long a = 0; a < p.nat; a++) nent += (size_t)pj->nl[a];
      if (nent > 2147483647u) return set_err(c, FBSE_ERR_UNSUPPORTED, "projector table too large");
      std::vector<int> start((size_t)c->ngrid + 1, 0);
      for (long a = 0; a < p.nat; a++)
        for (long e = 0; e < pj->nl[a]; e++) start[(size_t)pj->jxyz[a * p.npts + e] + 1]++;
      std::vector<int> cj, cb;
      for (long j = 0; j < c->ngrid; j++)
        if (start[j + 1]) cj.push_back((int)j);
      for (long j = 0; j < c->ngrid; j++) start[j + 1] += start[j];  // start[j] = first entry of point j
      for (size_t k = 0; k < cj.size(); k++) cb.push_back(start[cj[k]]);
      cb.push_back((int)nent);
      std::vector<int> pa(nent ? nent : 1, 0);
      std::vector<double> py((nent ? nent : 1) * 6, 0.0), ps((nent ? nent : 1) * p.nproj, 0.0),
          pn((nent ? nent : 1) * p.nproj, 0.0);
      for (long a = 0; a < p.nat; a++)
        for (long e = 0; e < pj->nl[a]; e++) {
          const size_t i = a * p.npts + e;
          const size_t k = (size_t)start[pj->jxyz[i]]++;
          pa[k] = (int)a;
          for (int m = 0; m < 3; m++)
            for (int q = 0; q < 2; q++) py[(m * nent + k) * 2 + q] = y1[(m * ne + i) * 2 + q];
          for (int q = 0; q < p.nproj; q++) {
            ps[q * nent + k] = so[q * ne + i];
            pn[q * nent + k] = nlr[q * ne + i];
          }
        }
      p.ncov = (long)cj.size();
      p.nent = (long)nent;
      // chunks of consecutive covered points for the scatter: at most
      // kScatterChunkPoints points and kScatterChunkAtoms distinct atoms each;
      // per chunk its atoms, per entry the atom's slot in its chunk
      std::vector<int> chb, cha;
      std::vector<unsigned char> slot(nent ? nent : 1, 0);
      {
        long k = 0;
        while (k < p.ncov) {
          std::vector<int> atoms;
          const long k0 = k;
          while (k < p.ncov && k - k0 < kScatterChunkPoints) {
            std::vector<int> add;
            for (int e = cb[k]; e < cb[k + 1]; e++)
              if (std::find(atoms.begin(), atoms.end(), pa[e]) == atoms.end() &&
                  std::find(add.begin(), add.end(), pa[e]) == add.end())
                add.push_back(pa[e]);
            if ((long)(atoms.size() + add.size()) > kScatterChunkAtoms) break;
            atoms.insert(atoms.end(), add.begin(), add.end());
            for (int e = cb[k]; e < cb[k + 1]; e++)
              slot[e] = (unsigned char)(std::find(atoms.begin(), atoms.end(), pa[e]) - atoms.begin());
            k++;
          }
          if (k == k0) return set_err(c, FBSE_ERR_UNSUPPORTED, "projector table: a point lies in too many spheres");
          chb.push_back((int)k0);
          atoms.resize(kScatterChunkAtoms, -1);
          cha.insert(cha.end(), atoms.begin(), atoms.end());
        }
        chb.push_back((int)p.ncov);
      }
      p.nchunk = (long)chb.size() - 1;
      if (cha.empty()) cha.assign(kScatterChunkAtoms, -1);
      if ((rc = upload(c, &p.chunk_beg, chb.data(), chb.size()))) return rc;
      if ((rc = upload(c, &p.chunk_atoms, cha.data(), cha.size()))) return rc;
      if ((rc = upload(c, &p.pe_slot, slot.data(), slot.size()))) return rc;
      if (cj.empty()) cj.push_back(0);
      if ((rc = upload(c, &p.cov_j, cj.data(), cj.size()))) return rc;
      if ((rc = upload(c, &p.cov_beg, cb.data(), cb.size()))) return rc;
      if ((rc = upload(c, &p.pe_atom, pa.data(), pa.size()))) return rc;
      if ((rc = upload(c, &p.pe_y1, py.data(), py.size()))) return rc;
      if ((rc = upload(c, &p.pe_sop, ps.data(), ps.size()))) return rc;
      if ((rc = upload(c, &p.pe_nlp, pn.data(), pn.size()))) return rc;
      if ((rc = upload(c, &p.pe_y1f, py.data(), py.size()))) return rc;
      if ((rc = upload(c, &p.pe_sopf, ps.data(), ps.size()))) return rc;
      if ((rc = upload(c, &p.pe_nlpf, pn.data(), pn.size()))) return rc;
      if ((rc = build_plane_table(c, cj, cb, pa, py, ps, pn, nent))) return rc;
    }
    FBSE_CUDA(c, cudaMalloc(&p.LS, 36 * sizeof(double2)));
    FBSE_CUDA(c, cudaMemcpy(p.LS, ls, 36 * sizeof(double2), cudaMemcpyHostToDevice));
  }
  return FBSE_OK;
}

}  // namespace fbse

using namespace fbse;

extern "C" {

int fbse_version(void) { return FBSE_ABI_VERSION; }

long fbse_launch_count(void) { return g_launches.load(); }

const char *fbse_last_error(const fbse_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int fbse_create(fbse_ctx **out, const fbse_grid_desc *grid, const double *pot_local, const fbse_proj_desc *proj,
                int precision)
{
  if (!out || !grid) return FBSE_ERR_ARG;
  *out = nullptr;
  if (precision != FBSE_FP64 && precision != FBSE_MIXED) return FBSE_ERR_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return FBSE_ERR_CUDA;
  }
  fbse_ctx *c = new fbse_ctx();
  c->precision = precision;
  int rc = create(c, grid, pot_local, proj);
  // pageable uploads may still be in flight after cudaMemcpy returns; the
  // context's non-blocking stream must not see them half done
  if (rc == FBSE_OK && cudaDeviceSynchronize() != cudaSuccess)
    rc = set_err(c, FBSE_ERR_CUDA, std::string("fbse_create: ") + cudaGetErrorString(cudaGetLastError()));
  *out = c;  // returned even on failure so fbse_last_error can explain
  return rc;
}

void fbse_destroy(fbse_ctx *c)
{
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (int a = 0; a < 3; a++) free_axis(c->ax[a]);
  void *bufs[] = {c->dstatus, c->k2x, c->k2y, c->k2z, c->k2xf, c->k2yf, c->k2zf, c->pot64, c->pot32, c->wk, c->coef, c->tmp, c->red,
                  c->proj.nl_cnt, c->proj.jxyz, c->proj.y1, c->proj.sop, c->proj.nlp, c->proj.sgn, c->proj.LS,
                  c->proj.y1f, c->proj.sopf, c->proj.nlpf, c->proj.cov_j, c->proj.cov_beg, c->proj.pe_atom,
                  c->proj.pe_y1, c->proj.pe_sop, c->proj.pe_nlp, c->proj.pe_y1f, c->proj.pe_sopf, c->proj.pe_nlpf,
                  c->proj.chunk_beg, c->proj.chunk_atoms, c->proj.pe_slot, c->proj.fz_ent, c->proj.fz_y,
                  c->proj.fz_so, c->proj.fz_nl, c->proj.fz_lay, c->proj.fz_atoms, c->proj.fz_natoms,
                  c->proj.fz_seg_beg, c->proj.fz_plane_seg, c->proj.fz_aseg_beg, c->proj.fz_aseg};
  for (void *b : bufs)
    if (b) cudaFree(b);
  for (void *b : c->cache)
    if (b) cudaFree(b);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  for (int k = 0; k < fbse_ctx::kSide; k++) {
    if (c->side[k]) cudaStreamSynchronize(c->side[k]);
    if (c->ev_join[k]) cudaEventDestroy(c->ev_join[k]);
    if (c->side[k]) cudaStreamDestroy(c->side[k]);
  }
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int fbse_alloc(fbse_ctx *c, void **dptr, size_t bytes)
{
  if (!c || !dptr) return FBSE_ERR_ARG;
  if (cudaMalloc(dptr, bytes ? bytes : 1) != cudaSuccess) {
    cudaGetLastError();
    return set_err(c, FBSE_ERR_OOM, "fbse_alloc of " + std::to_string(bytes) + " bytes failed");
  }
  return FBSE_OK;
}

int fbse_free(fbse_ctx *c, void *dptr)
{
  if (!c) return FBSE_ERR_ARG;
  cudaStreamSynchronize(c->stream);
  FBSE_CUDA(c, cudaFree(dptr));
  return FBSE_OK;
}

int fbse_upload(fbse_ctx *c, void *dst, const void *src, size_t bytes)
{
  if (!c) return FBSE_ERR_ARG;
  FBSE_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
  FBSE_CUDA(c, cudaStreamSynchronize(c->stream));
  return FBSE_OK;
}

int fbse_download(fbse_ctx *c, void *dst, const void *src, size_t bytes)
{
  if (!c) return FBSE_ERR_ARG;
  FBSE_CUDA(c, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
  FBSE_CUDA(c, cudaStreamSynchronize(c->stream));
  return FBSE_OK;
}

int fbse_sync(fbse_ctx *c)
{
  if (!c) return FBSE_ERR_ARG;
  FBSE_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_dev_status(c);
}

void *fbse_stream(fbse_ctx *c) { return c ? (void *)c->stream : nullptr; }

int fbse_get_tuning(fbse_ctx *c, fbse_tuning *t)
{
  if (!c || !t) return c ? set_err(c, FBSE_ERR_ARG, "fbse_get_tuning: null") : FBSE_ERR_ARG;
  *t = c->tune;
  return FBSE_OK;
}

int fbse_set_tuning(fbse_ctx *c, const fbse_tuning *t)
{
  if (!c || !t) return c ? set_err(c, FBSE_ERR_ARG, "fbse_set_tuning: null") : FBSE_ERR_ARG;
  auto pow2_in = [](long v, long hi) { return v == 0 || (v >= 1 && v <= hi && (v & (v - 1)) == 0); };
  if (t->fft_kernels < 0 || t->fft_kernels > 2 || t->fft_plane_cluster < 0 || t->fft_plane_cluster > 1 ||
      t->fft_chunk_blocks < 0 || !(pow2_in(t->scatter_states, 8) || t->scatter_states == 18 || t->scatter_states == 20) ||
      !pow2_in(t->gather_points, 4) ||
      (t->newton_ring != 0 && (t->newton_ring < 8 || t->newton_ring > 128)) || t->bse_simt < 0 || t->bse_simt > 1 ||
      !(t->tc_image_bytes >= 0) || !(t->ritz_cut >= 0 && t->ritz_cut < 1) || t->ritz_hpsi < 0 ||
      t->ritz_hpsi > 2 || t->hpsi_fused < 0 || t->hpsi_fused > 1 || t->hpsi_streams < 0 || t->hpsi_streams > 4)
    return set_err(c, FBSE_ERR_ARG, "fbse_set_tuning: a field is out of range");
  c->tune = *t;
  c->tuned.clear();  // earlier decisions may rest on the old fixed choices
  return FBSE_OK;
}

long fbse_tuning_report(fbse_ctx *c, char *buf, long n)
{
  if (!c) return -1;
  std::string j = "[";
  for (size_t i = 0; i < c->tuned.size(); i++) {
    const TuneRecord &r = c->tuned[i];
    j += (i ? ", " : "") + std::string("{\"kernel\": \"") + r.kernel + "\", \"problem\": \"" + r.problem +
         "\", \"candidates\": {";
    for (size_t k = 0; k < r.cand.size(); k++) {
      char b[64];
      snprintf(b, sizeof b, "%s\"%ld\": %.2f", k ? ", " : "", r.cand[k].first, r.cand[k].second);
      j += b;
    }
    j += "}, \"choice\": " + std::to_string(r.choice) + "}";
  }
  j += "]";
  if (buf && n > 0) {
    const size_t m = std::min<size_t>((size_t)n - 1, j.size());
    std::memcpy(buf, j.data(), m);
    buf[m] = 0;
  }
  return (long)j.size();
}

int fbse_hpsi(fbse_ctx *c, const void *in, void *out, long nstates)
{
  if (!c || !in || !out || nstates < 1) return c ? set_err(c, FBSE_ERR_ARG, "fbse_hpsi: bad arguments") : FBSE_ERR_ARG;
  if (in == out) return set_err(c, FBSE_ERR_ARG, "fbse_hpsi: input and output must differ");
  if (c->precision == FBSE_MIXED)
    return hpsi_apply<float>(c, (const float2 *)in, (float2 *)out, nstates, 1.0, 0.0);
  return hpsi_apply<double>(c, (const double2 *)in, (double2 *)out, nstates, 1.0, 0.0);
}

int fbse_hnorm(fbse_ctx *c, const void *in, void *out, long nstates, double vmin, double de, double zn)
{
  if (!c || !in || !out || nstates < 1 || !(de > 0))
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_hnorm: bad arguments") : FBSE_ERR_ARG;
  if (in == out) return set_err(c, FBSE_ERR_ARG, "fbse_hnorm: input and output must differ");
  const double de_1 = 4.0 / de;
  const double b = -(2.0 + zn + vmin * de_1);
  if (c->precision == FBSE_MIXED) return hpsi_apply<float>(c, (const float2 *)in, (float2 *)out, nstates, de_1, b);
  return hpsi_apply<double>(c, (const double2 *)in, (double2 *)out, nstates, de_1, b);
}

int fbse_newton_filter(fbse_ctx *c, const double *zn, const double *an, long ncheby, long m, double vmin,
                       double de, const double *psi0, long nstart, double *filtered)
{
  if (!c || !zn || !an || !psi0 || !filtered) return c ? set_err(c, FBSE_ERR_ARG, "fbse_newton_filter: null") : FBSE_ERR_ARG;
  return newton_filter(c, zn, an, ncheby, m, vmin, de, psi0, nstart, filtered);
}

int fbse_energy_range(fbse_ctx *c, long seed, long max_iter, double *emin, double *emax, long *iters)
{
  if (!c || !emin || !emax || max_iter < 1) return c ? set_err(c, FBSE_ERR_ARG, "fbse_energy_range: bad arguments") : FBSE_ERR_ARG;
  const int rc = energy_range(c, seed, max_iter, emin, emax, iters);
  return rc ? rc : check_dev_status(c);
}

int fbse_normalize_all(fbse_ctx *c, double *psitot, long n, double *norms)
{
  if (!c || !psitot) return c ? set_err(c, FBSE_ERR_ARG, "fbse_normalize_all: null") : FBSE_ERR_ARG;
  return normalize_all(c, psitot, n, norms);
}

int fbse_energy_all(fbse_ctx *c, const double *psitot, long n, double *ene)
{
  if (!c || !psitot || !ene) return c ? set_err(c, FBSE_ERR_ARG, "fbse_energy_all: null") : FBSE_ERR_ARG;
  return energy_all(c, psitot, n, ene, nullptr);
}

int fbse_sigma_e(fbse_ctx *c, const double *psitot, long n, double *eval, double *sigma)
{
  if (!c || !psitot || !eval || !sigma) return c ? set_err(c, FBSE_ERR_ARG, "fbse_sigma_e: null") : FBSE_ERR_ARG;
  const int rc = energy_all(c, psitot, n, eval, sigma);
  return rc ? rc : check_dev_status(c);
}

int fbse_gram(fbse_ctx *c, const double *A, long na, const double *B, long nb, long off, long len, double *out)
{
  if (!c || !A || !B || !out) return c ? set_err(c, FBSE_ERR_ARG, "fbse_gram: null") : FBSE_ERR_ARG;
  return gram_slab(c, A, na, B, nb, off, len, out);
}

int fbse_rotate(fbse_ctx *c, const double *A, long na, const double *coef, long k, long off, long len, double *out)
{
  if (!c || !A || !coef || !out) return c ? set_err(c, FBSE_ERR_ARG, "fbse_rotate: null") : FBSE_ERR_ARG;
  if (out == A) return set_err(c, FBSE_ERR_ARG, "fbse_rotate: out must not alias A");
  return rotate_slab(c, A, na, coef, k, off, len, out);
}

int fbse_ortho_diag_sigma(fbse_ctx *c, double *psitot, long n, long *n_kept, double *eval, double *sigma)
{
  if (!c || !psitot || !n_kept || !eval || !sigma || n < 1)
    return c ? set_err(c, FBSE_ERR_ARG, "fbse_ortho_diag_sigma: bad arguments") : FBSE_ERR_ARG;
  const int rc = ortho_diag_sigma(c, psitot, n, n_kept, eval, sigma);
  return rc ? rc : check_dev_status(c);
}

}  // extern "C"
