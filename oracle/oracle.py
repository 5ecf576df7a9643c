"""FP64 CPU oracle for FilterBSE's filter hot path (TEST INFRASTRUCTURE ONLY).

This module is the reference restatement the CUDA path is compared against.  Only tests/,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it;
the product package ``filterbse_gb300`` never does.

The loop-heavy pieces are a C restatement (``oracle/fbse_oracle.c``, built to
``oracle/liboracle.so``); the 3D FFT of the kinetic term uses numpy's FFT with
FFTW's conventions (forward e^{-i}, unnormalised backward), and the LAPACK
steps (SVD, symmetric/Hermitian eigensolves) use numpy.linalg.  Every routine
cites the reference function it restates (paths relative to the FilterBSE tree).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

PROJ_LEN = 1024  # filter_mpi/fd.h: PROJ_LEN
NPROJ = 5  # filter_mpi/read.c: ist->nproj default

_D = ctypes.POINTER(ctypes.c_double)
_L = ctypes.POINTER(ctypes.c_long)
_I = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the C restatement to oracle/liboracle.so (gcc, -O2, no -ffast-math,
    no contraction into fused multiply-adds: plain IEEE arithmetic on every host)."""
    src = os.path.join(_HERE, "fbse_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(src),
                                                                                     os.path.getmtime(__file__)):
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu99", "-ffp-contract=off", "-o", _LIB_PATH,
                               src, "-lm"])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _lib.orc_ran.restype = ctypes.c_double
        _lib.orc_ran_fill.restype = ctypes.c_long
        _lib.orc_ran_fill.argtypes = [ctypes.c_long, ctypes.c_long, _D]
        _lib.orc_init_psi.restype = ctypes.c_long
        _lib.orc_init_psi.argtypes = [_D, ctypes.c_long, ctypes.c_long, ctypes.c_int, ctypes.c_double]
        _lib.orc_samp_points.restype = ctypes.c_double
        _lib.orc_samp_points.argtypes = [ctypes.c_long, ctypes.c_double, ctypes.c_double, _D, _D]
        _lib.orc_newton_coeff.argtypes = [ctypes.c_long, ctypes.c_long, _D, _D, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_double, _D]
        _lib.orc_axis_ksqr.argtypes = [ctypes.c_long, ctypes.c_double, ctypes.c_double, _D]
        _lib.orc_ksqr.argtypes = [ctypes.c_long] * 3 + [ctypes.c_double] * 4 + [_D]
        _lib.orc_local_pot.argtypes = [ctypes.c_long] * 3 + [_D] * 3 + [ctypes.c_long, _D, _D, _D, _L,
                                                                         _D, _D, _L, _L, _D, _D]
        _lib.orc_proj_matrix.argtypes = [ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, _D]
        _lib.orc_proj_radial.argtypes = [ctypes.c_long, ctypes.c_double, ctypes.c_double, _D,
                                         ctypes.c_double, _D]
        _lib.orc_nlc_table.argtypes = ([ctypes.c_long] * 3 + [_D] * 3 + [ctypes.c_long, _D, _D, _D, _D,
                                       ctypes.c_double, ctypes.c_long, ctypes.c_long, ctypes.c_long, _D, _D,
                                       _L, _I, _D, _D, _D])
        _lib.orc_def_LS.argtypes = [_D]
        _lib.orc_apply_so.argtypes = [_D, _D, ctypes.c_long, ctypes.c_long, _L, ctypes.c_long, ctypes.c_long,
                                      _I, _D, _D, _D, ctypes.c_double]
        _lib.orc_apply_nl.argtypes = [_D, _D, ctypes.c_long, ctypes.c_int, ctypes.c_long, _L, ctypes.c_long,
                                      ctypes.c_long, _I, _D, _D, _I, ctypes.c_double]
        _lib.orc_apply_vloc.argtypes = [_D, _D, _D, ctypes.c_long, ctypes.c_int, ctypes.c_int]
        _lib.orc_hnorm_shift.argtypes = [_D, _D, ctypes.c_long] + [ctypes.c_double] * 3
    return _lib


def _p(a, t=_D):
    return a.ctypes.data_as(t)


# --------------------------------------------------------------------------
# Random starts, Newton coefficients
# --------------------------------------------------------------------------

def ran_fill(seed: int, n: int, out: bool = True):
    """n draws of ran_nrc (filter_mpi/rand.c:22-62); returns (values, new seed)."""
    buf = np.empty(n) if out else None
    s = lib().orc_ran_fill(seed, n, _p(buf) if out else None)
    return buf, s


def init_psi(seed: int, ngrid: int, is_complex: bool, dv: float):
    """init_psi (filter_mpi/init.c:1256-1307): one normalised random block."""
    psi = np.empty(2 * ngrid)
    s = lib().orc_init_psi(_p(psi), seed, ngrid, int(is_complex), dv)
    return psi.view(np.complex128), s


def init_filter_states(seed: int, n_filters: int, ngrid: int, nspin: int, is_complex: bool, dv: float):
    """init_filter_states (filter_mpi/init.c:1138-1255): n_filters random starts,
    each spin block drawn and normalised separately; returns ([n][nspin*ngrid], seeds)."""
    out = np.empty((n_filters, nspin * ngrid), np.complex128)
    seeds = []
    for j in range(n_filters):
        for s in range(nspin):
            seeds.append(seed)
            blk, seed = init_psi(seed, ngrid, is_complex, dv)
            out[j, s * ngrid:(s + 1) * ngrid] = blk
    return out, seeds, seed


def samp_points(ncheby: int):
    """samp_points_ashkenazy on [-2, 2] (filter_mpi/coeff.c:227-293)."""
    re = np.empty(ncheby)
    im = np.empty(ncheby)
    fk = lib().orc_samp_points(ncheby, -2.0, 2.0, _p(re), _p(im))
    return re, im, fk


def newton_coeff(zn, targets, vmin, de, dt):
    """gen_newton_coeff (filter_mpi/coeff.c:8-118); returns complex [m][ncheby]."""
    zn = np.ascontiguousarray(zn, np.float64)
    targets = np.ascontiguousarray(targets, np.float64)
    m, nc = len(targets), len(zn)
    an = np.empty(2 * m * nc)
    lib().orc_newton_coeff(nc, m, _p(zn), _p(targets), vmin, de, dt, _p(an))
    return an.view(np.complex128).reshape(m, nc)


def filter_dt(ncheby: int, de: float) -> float:
    """dt = (ncheby / (2.5 dE))^2 (filter_mpi/mod_filter.c:114)."""
    return (ncheby / (2.5 * de)) ** 2


def ene_targets(vbmin, vbmax, cbmin, cbmax, n_vb, n_cb):
    """set_ene_targets (filter_mpi/init.c:401-478)."""
    t = np.empty(n_vb + n_cb)
    d = (vbmax - vbmin) / n_vb
    for jx in range(n_vb):
        t[n_vb - jx - 1] = vbmax - jx * d
    d = (cbmax - cbmin) / n_cb
    for jx in range(n_vb, n_vb + n_cb):
        t[jx] = cbmin + (jx - n_vb) * d
    return t


# --------------------------------------------------------------------------
# Grid and system description
# --------------------------------------------------------------------------

@dataclass
class Grid:
    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    xmin: float
    ymin: float
    zmin: float
    ke_max: float = 20.0
    box_n: bool = False  # True: box = n d on every axis (older reference versions)

    @property
    def ngrid(self):
        return self.nx * self.ny * self.nz

    @property
    def dv(self):
        return self.dx * self.dy * self.dz

    def axes(self):
        """build_grid_ksqr's coordinates (filter_mpi/init.c:284-290): cumulative sums."""
        out = []
        for n, d, lo in ((self.nx, self.dx, self.xmin), (self.ny, self.dy, self.ymin), (self.nz, self.dz, self.zmin)):
            a = np.empty(n)
            v = lo
            for j in range(n):
                a[j] = v
                v += d
            out.append(a)
        return out

    def dk(self):
        """reciprocal spacing 2 pi / box (filter_mpi/init.c:65-80): box = n d (even), (n-1) d (odd)."""
        res = []
        for n, d in ((self.nx, self.dx), (self.ny, self.dy), (self.nz, self.dz)):
            box = n * d if (n % 2 == 0 or self.box_n) else (n - 1) * d
            res.append(2.0 * np.pi / box)
        return res

    def ksqr(self):
        k = np.empty(self.ngrid)
        dkx, dky, dkz = self.dk()
        lib().orc_ksqr(self.nx, self.ny, self.nz, dkx, dky, dkz, self.ke_max, _p(k))
        return k

    def axis_ksqr(self):
        ng_1 = (1.0 / self.nx) * (1.0 / self.ny) * (1.0 / self.nz)
        out = []
        for n, dk in zip((self.nx, self.ny, self.nz), self.dk()):
            a = np.empty(n)
            lib().orc_axis_ksqr(n, dk, ng_1, _p(a))
            out.append(a)
        return out


def reference_grid(coords: np.ndarray, d: float, n_in=(0, 0, 0), ke_max=20.0) -> Grid:
    """init_grid_params (filter_mpi/init.c:5-255, non-periodic): grow each axis to
    cover the dot plus 5 bohr each side, forced even when grown."""
    dims = []
    for ax in range(3):
        c = coords[:, ax]
        ext = np.sqrt(np.max((c[:, None] - c[None, :]) ** 2)) if len(c) > 1 else 0.0
        xd = np.rint(0.5 * ext + 5.0)
        lo, hi = -xd, xd - d
        ntmp = int((hi - lo) / d)
        n = n_in[ax]
        if ntmp > n:
            n = ntmp + (ntmp % 2)
        box = n * d if n % 2 == 0 else (n - 1) * d
        dims.append((n, -box / 2.0))
    return Grid(dims[0][0], dims[1][0], dims[2][0], d, d, d, dims[0][1], dims[1][1], dims[2][1], ke_max)


@dataclass
class Projectors:
    """Structure-of-arrays copy of the reference's nlc table (fd.h:382-398)."""
    nl: np.ndarray          # [nat] points per atom
    npts: int               # row stride (max points)
    jxyz: np.ndarray        # int32 [nat*npts]
    y1: np.ndarray          # [nat*npts*6] (re, im) x 3
    proj: np.ndarray        # [nat*npts*nproj] SO radial (scaled by sqrt(SO_par))
    nlp: np.ndarray         # [nat*npts*nproj] NL radial
    sgn: np.ndarray         # int32 [nat*nproj]
    nproj: int = NPROJ

    @property
    def nat(self):
        return len(self.nl)


@dataclass
class System:
    grid: Grid
    pot: np.ndarray               # [ngrid] local potential
    nspin: int = 1
    is_complex: bool = False
    so: bool = False
    nlflag: bool = False
    proj: Projectors | None = None
    LS: np.ndarray = field(default_factory=lambda: def_LS())

    @property
    def ngrid(self):
        return self.grid.ngrid


def def_LS():
    """def_LS (filter_mpi/hamiltonian.c:312-442) as complex [6][6] indexed [j'][j]."""
    ls = np.zeros(72)
    lib().orc_def_LS(_p(ls))
    return ls.view(np.complex128).reshape(6, 6)


def local_pot(grid: Grid, coords, atype, tables):
    """build_local_pot (filter_mpi/init.c:481-703) for short-ranged tables.
    tables: list per type of (r, v) arrays."""
    gx, gy, gz = grid.axes()
    rr = np.ascontiguousarray(coords[:, 0]), np.ascontiguousarray(coords[:, 1]), np.ascontiguousarray(coords[:, 2])
    tr = np.concatenate([np.asarray(t[0], np.float64) for t in tables])
    tv = np.concatenate([np.asarray(t[1], np.float64) for t in tables])
    tlen = np.array([len(t[0]) for t in tables], np.int64)
    toff = np.concatenate([[0], np.cumsum(tlen)[:-1]]).astype(np.int64)
    tdr = np.array([t[0][1] - t[0][0] for t in tables], np.float64)
    at = np.ascontiguousarray(atype, np.int64)
    pot = np.empty(grid.ngrid)
    lib().orc_local_pot(grid.nx, grid.ny, grid.nz, _p(gx), _p(gy), _p(gz), len(at), _p(rr[0]), _p(rr[1]),
                        _p(rr[2]), _p(at, _L), _p(tr), _p(tv), _p(toff, _L), _p(tlen, _L), _p(tdr), _p(pot))
    return pot


def so_radial(dx: float, rcut: float, nproj: int = NPROJ):
    """gen_SO_projectors (filter_mpi/projectors.c:12-84): the nproj leading
    eigenvectors of the k-space integral matrix mapped back to r.  [nproj][N]."""
    N = PROJ_LEN
    A = np.empty(N * N)
    lib().orc_proj_matrix(N, dx, rcut, 0, 0.0, 0.0, _p(A))
    w, v = np.linalg.eigh(A.reshape(N, N))
    out = np.empty((nproj, N))
    for p in range(nproj):
        vec = np.ascontiguousarray(v[:, N - p - 1])
        lib().orc_proj_radial(N, dx, rcut, _p(vec), float(w[N - p - 1]), _p(out[p]))
    return out


def nl_radial(dx: float, rcut: float, lam1: float, lam2: float, nproj: int = NPROJ):
    """gen_nlc_projectors (filter_mpi/projectors.c:87-228): the nproj eigenvectors
    of largest |eigenvalue|, signs = sign of the eigenvalue.  ([nproj][N], sgn)."""
    N = PROJ_LEN
    if lam1 == 0 and lam2 == 0:
        return np.zeros((nproj, N)), np.zeros(nproj, np.int32)
    A = np.empty(N * N)
    lib().orc_proj_matrix(N, dx, rcut, 1, lam1, lam2, _p(A))
    w, v = np.linalg.eigh(A.reshape(N, N))
    # insertion selection of the nproj largest |w| (projectors.c:166-186)
    eigs = [0.0] * nproj
    idx = [0] * nproj
    for i in range(N):
        if abs(w[i]) > eigs[nproj - 1]:
            for j in range(nproj - 1, -1, -1):
                if j == 0 or eigs[j - 1] > abs(w[i]):
                    eigs[j] = abs(w[i])
                    idx[j] = i
                    break
                eigs[j] = eigs[j - 1]
                idx[j] = idx[j - 1]
    out = np.empty((nproj, N))
    sgn = np.empty(nproj, np.int32)
    for p in range(nproj):
        sgn[p] = -1 if w[idx[p]] < 0 else 1
        vec = np.ascontiguousarray(v[:, idx[p]])
        lib().orc_proj_radial(N, dx, rcut, _p(vec), float(abs(w[idx[p]])), _p(out[p]))
    return out, sgn


def r_nlcut2(dx: float) -> float:
    """R_NLcut2 = 1.5 + 6 ln 10 + 3 dx (filter_mpi/read.c:908)."""
    return 1.5 + 6.0 * np.log(10.0) + 3.0 * dx


def nlc_table(grid: Grid, coords, so_par, so_tab, nl_tabs, nl_sgn, nproj=NPROJ) -> Projectors:
    """init_NL_projectors (filter_mpi/init.c:848-1060) over the projector atoms
    (coords rows), using the reference's EPSDX-shifted Y_1m; the points per
    atom are bounded by the largest sphere count (build_grid_ksqr,
    init.c:353-393)."""
    rc2 = r_nlcut2(grid.dx)
    gx, gy, gz = grid.axes()
    nat = len(coords)
    # count the maximum points per atom (build_grid_ksqr, init.c:353-393)
    npts = 0
    for a in range(nat):
        d2 = (gx[None, None, :] - coords[a, 0]) ** 2 + (gy[None, :, None] - coords[a, 1]) ** 2 + \
             (gz[:, None, None] - coords[a, 2]) ** 2
        npts = max(npts, int(np.count_nonzero(d2 < rc2)))
    npts = max(npts, 1)
    N = PROJ_LEN
    so_tab = np.ascontiguousarray(so_tab, np.float64).reshape(nproj, N)
    nl_tabs = np.ascontiguousarray(nl_tabs, np.float64).reshape(nat, nproj, N)
    nl = np.zeros(nat, np.int64)
    jxyz = np.zeros(nat * npts, np.int32)
    y1 = np.zeros(nat * npts * 6)
    proj = np.zeros(nat * npts * nproj)
    nlp = np.zeros(nat * npts * nproj)
    cx, cy, cz = (np.ascontiguousarray(coords[:, i]) for i in range(3))
    sp = np.ascontiguousarray(so_par, np.float64)
    lib().orc_nlc_table(grid.nx, grid.ny, grid.nz, _p(gx), _p(gy), _p(gz), nat, _p(cx), _p(cy), _p(cz), _p(sp),
                        rc2, npts, nproj, N, _p(so_tab), _p(nl_tabs), _p(nl, _L), _p(jxyz, _I), _p(y1), _p(proj),
                        _p(nlp))
    return Projectors(nl, npts, jxyz, y1, proj, nlp, np.ascontiguousarray(nl_sgn, np.int32).reshape(-1), nproj)


# --------------------------------------------------------------------------
# H psi
# --------------------------------------------------------------------------

def kinetic(psi: np.ndarray, sysm: System) -> np.ndarray:
    """kinetic (filter_mpi/hamiltonian.c:62-99) per spin block: FFTW forward,
    times ksqr (which already holds 1/N), FFTW backward (unnormalised)."""
    g = sysm.grid
    k = g.ksqr().reshape(g.nz, g.ny, g.nx)
    out = np.empty_like(psi)
    n = g.ngrid
    for s in range(sysm.nspin):
        blk = psi[s * n:(s + 1) * n].reshape(g.nz, g.ny, g.nx)
        f = np.fft.fftn(blk) * k
        out[s * n:(s + 1) * n] = (np.fft.ifftn(f) * n).reshape(-1)
    return out


def potential_add(out: np.ndarray, psi: np.ndarray, sysm: System):
    """p_potential (filter_mpi/phamiltonian.c:65-137): SO, then NL, then V_loc."""
    L = lib()
    o = out.view(np.float64)
    p = np.ascontiguousarray(psi).view(np.float64)
    n = sysm.ngrid
    pr = sysm.proj
    if sysm.so:
        ls = np.ascontiguousarray(sysm.LS).view(np.float64)
        L.orc_apply_so(_p(o), _p(p), n, pr.nat, _p(pr.nl, _L), pr.npts, pr.nproj, _p(pr.jxyz, _I), _p(pr.y1),
                       _p(pr.proj), _p(ls), sysm.grid.dv)
    if sysm.nlflag:
        L.orc_apply_nl(_p(o), _p(p), n, sysm.nspin, pr.nat, _p(pr.nl, _L), pr.npts, pr.nproj, _p(pr.jxyz, _I),
                       _p(pr.y1), _p(pr.nlp), _p(pr.sgn, _I), sysm.grid.dv)
    pot = np.ascontiguousarray(sysm.pot, np.float64)
    L.orc_apply_vloc(_p(o), _p(p), _p(pot), n, sysm.nspin, int(sysm.is_complex))


def hamiltonian(psi: np.ndarray, sysm: System) -> np.ndarray:
    """p_hamiltonian (filter_mpi/phamiltonian.c:10-60): H psi for one state
    (complex [nspin*ngrid]).  For real states the imaginary channel is left to
    the kinetic term only, exactly as the reference's real path does."""
    psi = np.ascontiguousarray(psi, np.complex128)
    out = kinetic(psi, sysm)
    potential_add(out, psi, sysm)
    return out


def hnorm(psi: np.ndarray, sysm: System, de_1: float, vmin: float, zn: float) -> np.ndarray:
    """p_hnorm (filter_mpi/filter.c:375-410)."""
    h = hamiltonian(psi, sysm)
    hv = h.view(np.float64)
    lib().orc_hnorm_shift(_p(hv), _p(np.ascontiguousarray(psi).view(np.float64)), len(psi), de_1, vmin, zn)
    return h


def filter_cycle(psi0: np.ndarray, sysm: System, an: np.ndarray, zn: np.ndarray, vmin: float, de: float):
    """filter_cycle (filter_mpi/filter.c:187-371): returns [m][nspin*ngrid] filtered
    states F_t = sum_j a_{t,j} prod_{i<j}(H_s - z_i) psi0 (complex storage; for
    real systems only the real part is meaningful, as in psi_rank)."""
    de_1 = 4.0 / de
    m, nc = an.shape
    psi = np.array(psi0, np.complex128)
    if not sysm.is_complex:
        psi = psi.real.astype(np.complex128)
    acc = an[:, 0:1] * psi[None, :]
    for jc in range(1, nc):
        psi = hnorm(psi, sysm, de_1, vmin, zn[jc - 1])
        acc += an[:, jc:jc + 1] * psi[None, :]
    if not sysm.is_complex:
        acc = acc.real.astype(np.complex128)
    return acc


def energy(psi: np.ndarray, sysm: System) -> float:
    """energy (filter_mpi/energy.c:6-57): dv sum Re(conj(psi) H psi)."""
    h = hamiltonian(psi, sysm)
    return float(np.sum(psi.real * h.real + psi.imag * h.imag) * sysm.grid.dv)


def normalize(psi: np.ndarray, dv: float) -> np.ndarray:
    """normalize (filter_mpi/norm.c:42-79)."""
    return psi / np.sqrt(np.sum(np.abs(psi) ** 2) * dv)


def energy_range(sysm: System, max_iter: int = 1500, seed: int = -874917403):
    """get_energy_range (filter_mpi/energy.c:169-379) with approxEnergyRange = 0:
    imaginary-time descent for E_min (tau = 0.05, halved-step on rises) and power
    iteration for E_max, then the blanket inflation (x1.2 / -0.2|E_min|) used
    when SO is on or no projectors are active.  Returns (Vmin, dE, Emin, Emax)."""
    n = sysm.ngrid
    dv = sysm.grid.dv
    phi = np.empty(sysm.nspin * n, np.complex128)
    for s in range(sysm.nspin):
        blk, seed = init_psi(seed, n, sysm.is_complex, dv)
        phi[s * n:(s + 1) * n] = blk
    tau = 0.05
    emin, old = 10.0, 0.0
    i = 0
    while abs((emin - old) / emin) > 1e-6 and i < max_iter:
        psi = phi.copy()
        h = hamiltonian(psi, sysm)
        phi = normalize(psi - tau * h, dv)
        old = emin
        emin = energy(phi, sysm)
        if i > 5 and (emin - old) > 0:
            tau -= 0.025
        i += 1
    psi = np.empty(sysm.nspin * n, np.complex128)
    for s in range(sysm.nspin):
        blk, seed = init_psi(seed, n, sysm.is_complex, dv)
        psi[s * n:(s + 1) * n] = blk
    emax, old = 0.1, 0.0
    i = 0
    while abs((emax - old) / emax) > 1e-6 and i < max_iter:
        psi = normalize(hamiltonian(psi, sysm), dv)
        old = emax
        emax = energy(psi, sysm)
        i += 1
    return inflate_range(sysm, emin, emax)


def nl_bounds(proj: "Projectors", dv: float):
    """The NL spectral-bound estimate of init_NL_projectors
    (filter_mpi/init.c:1095-1130): per (atom, projector, m) channel
    lam = sgn dv sum_points NL_proj^2 |Y_1m|^2; (min(0, lam...), max(0, lam...))."""
    lo = hi = 0.0
    for a in range(len(proj.nl)):
        sl = slice(a * proj.npts, a * proj.npts + int(proj.nl[a]))
        b2 = proj.nlp.reshape(-1, proj.nproj)[sl] ** 2
        y = proj.y1.reshape(-1, 3, 2)[sl]
        y2 = y[..., 0] ** 2 + y[..., 1] ** 2
        for q in range(proj.nproj):
            for m in range(3):
                lam = float(proj.sgn[a * proj.nproj + q]) * dv * float(np.sum(b2[:, q] * y2[:, m]))
                lo, hi = min(lo, lam), max(hi, lam)
    return lo, hi


def approx_energy_range(vmax_loc: float, ke_max: float, so: bool, nl: bool, lam_min: float, lam_max: float):
    """The approxEnergyRange branch of get_energy_range (filter_mpi/energy.c:302-335):
    [-0.8, Vmax + KE_max], + 3.5 on Emax with SO, the NL pads 1.15 lam."""
    emin, emax = -0.8, vmax_loc + ke_max
    if so:
        emax += 3.5
    if nl:
        emax += 1.15 * lam_max if lam_max > 0.0 else 0.0
        emin += 1.15 * lam_min if lam_min < 0.0 else 0.0
    return emin, emax


def inflate_range(sysm: System, emin: float, emax: float, nl_lambda_min: float = 0.0):
    """Range inflation of get_energy_range (filter_mpi/energy.c:338-369).
    NL-only jobs with a negative NL bound get the trimmed rule."""
    if sysm.nlflag and not sysm.so and nl_lambda_min < 0.0:
        emax_i = emax * 1.05
        emin_i = emin - 0.1 * abs(emin)
        weyl = 1.05 * (float(np.min(sysm.pot)) + nl_lambda_min)
        if emin_i > weyl:
            emin_i = weyl
    else:
        emax_i = emax * 1.2
        emin_i = emin - 0.2 * abs(emin)
    return emin_i, emax_i - emin_i, emin, emax


# --------------------------------------------------------------------------
# Orthogonalisation, subspace diagonalisation, sigma_E
# --------------------------------------------------------------------------

def ortho(psis: np.ndarray, is_complex: bool, eps: float = 1e-10, dv: float = 1.0):
    """ortho_real/ortho_cplx (filter_mpi/ortho.c:5-187) + normalize_all
    (mod_ortho.c:80): thin SVD of the (points x states) matrix, keep left
    vectors with s_i/s_0 >= 1e-10, normalise with dv.  psis: [n][npts]."""
    A = psis.T if is_complex else psis.real.T
    u, s, _ = np.linalg.svd(A, full_matrices=False)
    keep = int(np.sum(s / s[0] >= eps))
    return u[:, :keep].T.copy() / np.sqrt(dv), s


def diag(psis: np.ndarray, sysm: System):
    """diag_H (filter_mpi/Hmat.c:5-297): H_ij = dv <psi_i|H|psi_j>, eigh, rotate,
    then normalize_all (mod_diag.c).  Returns (evals, vectors [n][npts])."""
    dv = sysm.grid.dv
    H = np.array([hamiltonian(p if sysm.is_complex else p.real.astype(np.complex128), sysm) for p in psis])
    if not sysm.is_complex:
        M = (psis.real @ H.real.T) * dv
        M = 0.5 * (M + M.T)
    else:
        M = (psis.conj() @ H.T) * dv
        M = 0.5 * (M + M.conj().T)
    e, c = np.linalg.eigh(M)
    vec = c.T @ psis
    vec = np.array([normalize(v, dv) for v in vec])
    return e, vec


def sigma_e(psis: np.ndarray, sysm: System):
    """calc_sigma_E (filter_mpi/energy.c:383-539): sigma = sqrt|<H^2> - <H>^2|,
    computed here as the equal residual norm ||(H - E) psi|| for normalised psi
    (the reference's two-application form loses digits to cancellation)."""
    dv = sysm.grid.dv
    ev, sg = [], []
    for p in psis:
        p = p if sysm.is_complex else p.real.astype(np.complex128)
        h = hamiltonian(p, sysm)
        e = float(np.sum(p.real * h.real + p.imag * h.imag) * dv)
        r = h - e * p
        if not sysm.is_complex:
            r = r.real
        ev.append(e)
        sg.append(float(np.sqrt(np.sum(np.abs(r) ** 2) * dv)))
    return np.array(ev), np.array(sg)


# --------------------------------------------------------------------------
# Bethe-Salpeter stage (bse_cplx/)
# --------------------------------------------------------------------------

def bse_axes(grid: Grid):
    """The BSE stage's coordinates, x_j = xmin + j dx (bse_cplx/read.c:398-409)."""
    return [lo + np.arange(n) * d for n, d, lo in ((grid.nx, grid.dx, grid.xmin), (grid.ny, grid.dy, grid.ymin),
                                                   (grid.nz, grid.dz, grid.zmin))]


def bse_potentials(grid: Grid, eps=(6.0, 6.0, 6.0)):
    """init_elec_hole_kernel (bse_cplx/init.c:8-268): bare v(k) and screened
    W(k) on the grid, flat [ngrid] complex, including the 1/N."""
    from scipy.special import erf
    gx, gy, gz = bse_axes(grid)
    nx, ny, nz, N = grid.nx, grid.ny, grid.nz, grid.ngrid
    xm, ym, zm = abs(grid.xmin), abs(grid.ymin), abs(grid.zmin)
    if xm < ym and xm < zm:
        minr, boxl = xm, nx * grid.dx
    elif ym < zm and ym < xm:
        minr, boxl = ym, ny * grid.dy
    else:
        minr, boxl = zm, nz * grid.dz
    gamma = 7.0 / (2.0 * minr)
    ex, ey, ez = eps
    sqe_1 = 1.0 / np.sqrt(ex * ey * ez)
    sqrtaveps = np.sqrt((ex + ey + ez) / 3.0)
    gammaeps = gamma * sqrtaveps
    sqrk0 = gamma ** 2 * sqrtaveps ** 2

    def coul(r, g):  # calc_coulomb (init.c:271-291)
        out = np.empty_like(r)
        small = r < 1e-10
        out[small] = 2.0 * g / np.sqrt(np.pi)
        out[~small] = erf(g * r[~small]) / r[~small]
        return out

    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    x2, y2, z2 = X * X, Y * Y, Z * Z
    r2 = x2 + y2 + z2
    inside = r2 < boxl * boxl
    potr = np.where(inside, coul(np.sqrt(x2 + y2 + z2), gamma), 0.0)
    potrx = np.where(inside, sqe_1 * coul(np.sqrt(x2 / ex + y2 / ey + z2 / ez), gammaeps), 0.0)
    fb = np.fft.fftn(potr.astype(np.complex128))
    fs = np.fft.fftn(potrx.astype(np.complex128))
    dk = [2 * np.pi / (n * d) for n, d in ((nx, grid.dx), (ny, grid.dy), (nz, grid.dz))]

    def k2(n, d):
        m = np.arange(n)
        m = np.where(m <= n // 2, m, n - m)
        return (m * d) ** 2

    KZ, KY, KX = np.meshgrid(k2(nz, dk[2]), k2(ny, dk[1]), k2(nx, dk[0]), indexing="ij")
    JZ, JY, JX = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    alpha = np.pi * (JX + JY + JZ + N // 2).astype(np.float64)
    ph = np.cos(alpha) + 1j * np.sin(alpha)
    bare = fb * ph * grid.dv + 4 * np.pi / (KX + KY + KZ + gamma ** 2)
    ek = ex * KX + ey * KY + ez * KZ
    scr = fs * ph * grid.dv + 4 * np.pi * (1.0 - np.exp(-0.25 * ek / sqrk0)) / (ek + 1e-10)
    return (bare / N).reshape(-1), (scr / N).reshape(-1)


def hartree(rho: np.ndarray, potq: np.ndarray, grid: Grid):
    """hartree (bse_cplx/hartree.c:7-31): FFTW forward, times potq, backward."""
    shp = (grid.nz, grid.ny, grid.nx)
    f = np.fft.fftn(rho.reshape(shp)) * potq.reshape(shp)
    return (np.fft.ifftn(f) * grid.ngrid).reshape(-1)


def bse_kernels(psi_qp: np.ndarray, nh: int, ne: int, lumo: int, bare, scr, grid: Grid, nspin: int = 2):
    """calc_eh_kernel_cplx (bse_cplx/coulomb.c:20-738): direct and exchange,
    lower triangles ibs >= jbs as the reference fills them."""
    N = grid.ngrid
    dv = grid.dv

    def rho(x, y):
        return sum(np.conj(psi_qp[x, s * N:(s + 1) * N]) * psi_qp[y, s * N:(s + 1) * N] for s in range(nspin))

    nx = ne * nh
    D = np.zeros((nx, nx), np.complex128)
    X = np.zeros((nx, nx), np.complex128)
    for a in range(ne):
        for b in range(ne):
            h = hartree(rho(lumo + a, lumo + b), scr, grid)
            for i in range(nh):
                for j in range(nh):
                    ibs, jbs = a * nh + i, b * nh + j
                    if ibs < jbs:
                        continue
                    D[ibs, jbs] = np.sum(h * rho(j, i)) * dv
    for a in range(ne):
        for i in range(nh):
            h = hartree(rho(lumo + a, i), bare, grid)
            for b in range(ne):
                for j in range(nh):
                    ibs, jbs = a * nh + i, b * nh + j
                    if ibs < jbs:
                        continue
                    X[ibs, jbs] = -np.sum(h * rho(j, lumo + b)) * dv
    return D, X


def bse_kernels_real(psi_qp: np.ndarray, nh: int, ne: int, lumo: int, bare, scr, grid: Grid):
    """calc_eh_kernel_cplx of the real-valued BSE (bse_real/coulomb.c:20-705) for
    real one-component states [n_qp][ngrid]: rho products without conjugation,
    the real part of each convolution (bse_real/hartree.c:31), and the singlet
    factor 2 on the exchange (coulomb.c:568)."""
    N = grid.ngrid
    dv = grid.dv
    nx = ne * nh
    D = np.zeros((nx, nx))
    X = np.zeros((nx, nx))
    for a in range(ne):
        for b in range(ne):
            h = hartree(psi_qp[lumo + a] * psi_qp[lumo + b], scr, grid).real
            for i in range(nh):
                for j in range(nh):
                    ibs, jbs = a * nh + i, b * nh + j
                    if ibs >= jbs:
                        D[ibs, jbs] = np.sum(h * psi_qp[j] * psi_qp[i]) * dv
    for a in range(ne):
        for i in range(nh):
            h = hartree(psi_qp[lumo + a] * psi_qp[i], bare, grid).real
            for b in range(ne):
                for j in range(nh):
                    ibs, jbs = a * nh + i, b * nh + j
                    if ibs >= jbs:
                        X[ibs, jbs] = -2.0 * np.sum(h * psi_qp[j] * psi_qp[lumo + b]) * dv
    return D, X


def bse_solve(eval_qp, nh, ne, lumo, D, X):
    """build_h0_mat, build_BSE_mat, bethe_salpeter (bse_cplx/mod_bse.c:54-148,
    bethe-salpeter.c:7-350): returns (E, C, <H>, <Kd>, <Kx>, <h0>)."""
    n = nh * ne
    Df = np.tril(D) + np.conj(np.tril(D, -1)).T
    Xf = np.tril(X) + np.conj(np.tril(X, -1)).T
    Df[np.diag_indices(n)] = Df.diagonal().real
    Xf[np.diag_indices(n)] = Xf.diagonal().real
    h0 = np.zeros((n, n))
    for a in range(ne):
        for i in range(nh):
            h0[a * nh + i, a * nh + i] = eval_qp[lumo + a] - eval_qp[i]
    H = h0 - (Df + Xf)
    H[np.diag_indices(n)] = H.diagonal().real
    e, C = np.linalg.eigh(H)
    ex = lambda M: np.real(np.einsum("li,lk,ki->i", C.conj(), M, C))
    return e, C, ex(H), ex(Df), ex(Xf), ex(h0)


def bse_dipoles(psi_qp, nh, ne, lumo, grid: Grid, nspin=2):
    """calc_elec_dipole (bse_cplx/dipole.c:7-158): [nh*ne][3] complex."""
    gx, gy, gz = bse_axes(grid)
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    coords = [X.reshape(-1), Y.reshape(-1), Z.reshape(-1)]
    N = grid.ngrid
    mu = np.zeros((nh * ne, 3), np.complex128)
    for i in range(nh):
        for a in range(ne):
            t = sum(np.conj(psi_qp[i, s * N:(s + 1) * N]) * psi_qp[lumo + a, s * N:(s + 1) * N] for s in range(nspin))
            for d in range(3):
                mu[i * ne + a, d] = np.sum(t * coords[d]) * grid.dv
    return mu


def init_kvec(n, dk):
    """init_kvec (bse_cplx/ang_mom_operators.c:90-103) without the 1/N norm:
    k[j] = j dk, k[n-j] = -j dk for j = 1..n/2 in that order."""
    k = np.zeros(n)
    for j in range(1, n // 2 + 1):
        k[j] = j * dk
        k[n - j] = -j * dk
    return k


def bse_mag_dipoles(psi_qp, nh, ne, lumo, grid: Grid, nspin=2):
    """calc_mag_dipole (bse_cplx/dipole.c:160-331): m_ia = (dv/2) sum
    conj(psi_i) L'psi_a with L'psi = -(r x p psi), p_d psi = IFFT(k_d FFT psi)
    (l_operator / p_operator, ang_mom_operators.c:6-170; the two unnormalised
    FFTW transforms and the 1/N in k_d make numpy's fftn / ifftn pair)."""
    gx, gy, gz = bse_axes(grid)
    shp = (grid.nz, grid.ny, grid.nx)
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    KZ, KY, KX = np.meshgrid(init_kvec(grid.nz, 2 * np.pi / (grid.nz * grid.dz)),
                             init_kvec(grid.ny, 2 * np.pi / (grid.ny * grid.dy)),
                             init_kvec(grid.nx, 2 * np.pi / (grid.nx * grid.dx)), indexing="ij")
    N = grid.ngrid
    m = np.zeros((nh * ne, 3), np.complex128)
    for a in range(ne):
        L = []
        for s in range(nspin):
            f = np.fft.fftn(psi_qp[lumo + a, s * N:(s + 1) * N].reshape(shp))
            px, py, pz = (np.fft.ifftn(k * f) for k in (KX, KY, KZ))
            L.append([-(Y * pz - Z * py), -(Z * px - X * pz), -(X * py - Y * px)])
        for i in range(nh):
            for d in range(3):
                m[i * ne + a, d] = 0.5 * grid.dv * sum(
                    np.sum(np.conj(psi_qp[i, s * N:(s + 1) * N].reshape(shp)) * L[s][d]) for s in range(nspin))
    return m


def _l_prime(f, grid):
    """l_operator (bse_cplx/ang_mom_operators.c:6-52) on one spin block:
    L' f = -(r x p f), p_d f = IFFT(k_d FFT f) (p_operator, init_kvec)."""
    gx, gy, gz = bse_axes(grid)
    shp = (grid.nz, grid.ny, grid.nx)
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    KZ, KY, KX = np.meshgrid(init_kvec(grid.nz, 2 * np.pi / (grid.nz * grid.dz)),
                             init_kvec(grid.ny, 2 * np.pi / (grid.ny * grid.dy)),
                             init_kvec(grid.nx, 2 * np.pi / (grid.nx * grid.dx)), indexing="ij")
    F = np.fft.fftn(f.reshape(shp))
    px, py, pz = (np.fft.ifftn(k * F) for k in (KX, KY, KZ))
    return [(-(Y * pz - Z * py)).reshape(-1), (-(Z * px - X * pz)).reshape(-1), (-(X * py - Y * px)).reshape(-1)]


def bse_qp_ang_mom(psi_qp, nh, ne, lumo, grid: Grid):
    """calc_qp_spin_mtrx and calc_qp_ang_mom_mtrx (bse_cplx/angular.c:7-690)
    for spinor states: s, l [nh^2 + ne^2][3], l2, ls [nh^2 + ne^2] with the
    reference's per-block conventions (holes: -1/2 conj for spins, conj of the
    negated L' sums; electrons: the sums as they are)."""
    N, dv = grid.ngrid, grid.dv
    n = nh * nh + ne * ne
    S = np.zeros((n, 3), np.complex128)
    Lm = np.zeros((n, 3), np.complex128)
    L2 = np.zeros(n, np.complex128)
    LS = np.zeros(n, np.complex128)
    for blk, (cnt, s0, off) in enumerate(((nh, 0, 0), (ne, lumo, nh * nh))):
        for i in range(cnt):
            pi = psi_qp[s0 + i]
            iu, idn = pi[:N], pi[N:]
            lp = [_l_prime(iu, grid), _l_prime(idn, grid)]  # [spin][d]
            l2 = [sum(_l_prime(lp[sp][d], grid)[d] for d in range(3)) for sp in range(2)]
            for j in range(cnt):
                pj = psi_qp[s0 + j]
                ju, jd = pj[:N], pj[N:]
                c = np.conj
                sx = np.sum(c(jd) * iu) + np.sum(c(ju) * idn)
                sy = 1j * np.sum(c(jd) * iu) - 1j * np.sum(c(ju) * idn)
                sz = np.sum(c(ju) * iu) - np.sum(c(jd) * idn)
                sv = np.array([sx, sy, sz])
                k = off + i * cnt + j
                S[k] = 0.5 * sv * dv if blk else -0.5 * np.conj(sv) * dv
                if j < i:
                    continue
                r = np.array([np.sum(c(ju) * lp[0][d]) + np.sum(c(jd) * lp[1][d]) for d in range(3)])
                rl2 = np.sum(c(ju) * l2[0]) + np.sum(c(jd) * l2[1])
                rls = (np.sum(c(jd) * lp[0][0]) + np.sum(c(ju) * lp[1][0]) + 1j * np.sum(c(jd) * lp[0][1])
                       - 1j * np.sum(c(ju) * lp[1][1]) + np.sum(c(ju) * lp[0][2]) - np.sum(c(jd) * lp[1][2]))
                lv = r * dv if blk else -np.conj(r) * dv
                l2v = rl2 * dv if blk else np.conj(rl2) * dv
                lsv = 0.5 * rls * dv if blk else 0.5 * np.conj(rls) * dv
                kt = off + j * cnt + i
                Lm[k], Lm[kt] = lv, np.conj(lv)
                L2[k], L2[kt] = l2v, np.conj(l2v)
                LS[k], LS[kt] = lsv, np.conj(lsv)
    return S, Lm, L2, LS


def bse_electron_ls_as_written(psi_qp, nh, ne, lumo, grid: Grid):
    """The electron block of ldots as calc_qp_ang_mom_mtrx computes it
    (bse_cplx/angular.c:582-604): its L.S loop sets jsg = ngrid once and never
    advances it, so every term that should read the spin-down point jg reads
    the first spin-down point.  Upper triangle with the diagonal from the loop,
    strict lower triangle by conjugation (angular.c:614-631).  [ne^2] complex, row a, column b.
    Only for pinning the reference; bse_qp_ang_mom holds the L.S sums."""
    N, dv = grid.ngrid, grid.dv
    out = np.zeros(ne * ne, np.complex128)
    for a in range(ne):
        pa = psi_qp[lumo + a]
        Lx, Ly, Lz = (np.concatenate([u, d]) for u, d in zip(_l_prime(pa[:N], grid), _l_prime(pa[N:], grid)))
        for b in range(a, ne):
            pb = psi_qp[lumo + b]
            up, d0 = pb[:N], pb[N]
            c = np.conj
            ls = (c(d0) * np.sum(Lx[:N]) + np.sum(c(up)) * Lx[N] + 1j * c(d0) * np.sum(Ly[:N])
                  - 1j * np.sum(c(up)) * Ly[N] + np.sum(c(up) * Lz[:N]) - N * c(d0) * Lz[N])
            out[a * ne + b] = 0.5 * ls * dv
            if b > a:
                out[b * ne + a] = np.conj(out[a * ne + b])
    return out


def filter_angular_stats(psis, grid: Grid):
    """calc_angular_exp (filter_mpi/angular.c:4-165) for complex spinor states
    (rows of psitot, (re, im) interleaved, up block then down block): per
    state low_pass_filter on each block (angular.c:403-455: FFTW round trip
    with the mask kx^2 + ky^2 + kz^2 < (3 dkz)^2 on init_kvec's wave vectors,
    which carry 1/N), normalize (norm.c:41-78), apply_J_op / apply_L_op
    (angular.c:169-400: p_d = IFFT(k_d/N FFT), L = r x p with the centre at the
    origin, plus sigma/2) and the eight sums times dv (angular.c:127-157).
    Each state's own imaginary parts are read (angular.c:63 offsets the
    spin-up imaginary part of state i > 0 by i * nspinngrid).  [n, 8]"""
    N = grid.ngrid
    shp = (grid.nz, grid.ny, grid.nx)
    gx, gy, gz = grid.axes()
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    dkx, dky, dkz = grid.dk()
    kx, ky, kz = (init_kvec(n, dk) / N for n, dk in ((grid.nx, dkx), (grid.ny, dky), (grid.nz, dkz)))
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    mask = (KX ** 2 + KY ** 2 + KZ ** 2) < (3.0 * dkz) ** 2
    out = np.zeros((len(psis), 8))
    for i, row in enumerate(psis):
        z = np.asarray(row, np.float64).view(np.complex128)
        blocks = []
        for s in range(2):
            f = np.fft.fftn(z[s * N:(s + 1) * N].reshape(shp))
            blocks.append(np.fft.ifftn(np.where(mask, f, 0.0)) * N)  # FFTW's unnormalised backward
        nrm = np.sqrt(sum(np.sum(np.abs(b) ** 2) for b in blocks) * grid.dv)
        blocks = [b / nrm for b in blocks]
        J = []
        for b in blocks:
            F = np.fft.fftn(b)
            px, py, pz = (np.fft.ifftn(k * N * F) for k in (KX, KY, KZ))  # k carries 1/N; ifftn adds another
            J.append([Y * pz - Z * py, Z * px - X * pz, X * py - Y * px])
        u, d = blocks
        J[0][0] = J[0][0] + 0.5 * d
        J[1][0] = J[1][0] + 0.5 * u
        J[0][1] = J[0][1] - 0.5j * d
        J[1][1] = J[1][1] + 0.5j * u
        J[0][2] = J[0][2] + 0.5 * u
        J[1][2] = J[1][2] - 0.5 * d
        r = np.zeros(8)
        for s in range(2):
            for a in range(3):
                r[2 * a] += np.sum((np.conj(blocks[s]) * J[s][a]).real)
                r[2 * a + 1] += np.sum(np.abs(J[s][a]) ** 2)
            r[6] += sum(np.sum(np.abs(J[s][a]) ** 2) for a in range(3))
            r[7] += np.sum(np.abs(blocks[s]) ** 2)
        out[i] = r * grid.dv
    return out


def xton_ang_stats(C, S, Lm, L2, LS, nh, ne):
    """calc_xton_spin_mtrx and calc_xton_ang_mom_mtrx (bse_cplx/angular.c:692-1043):
    per exciton n: <S> (3), the spin sum of spins.dat, <L> (3), the orbital sum
    of orbital.dat and the L.S sum of couple.dat.  C[ibs][n], ibs = a*nh + i."""
    nx = nh * ne
    he = lambda i, j: i * nh + j            # hole pair index
    el = lambda a, b: nh * nh + a * ne + b  # electron pair index
    spin = np.zeros((nx, 3), np.complex128)
    stot = np.zeros(nx, np.complex128)
    orb = np.zeros((nx, 3), np.complex128)
    otot = np.zeros(nx, np.complex128)
    lstot = np.zeros(nx, np.complex128)
    for n in range(nx):
        c = C[:, n]
        for a in range(ne):
            for i in range(nh):
                ibs = a * nh + i
                st = sum(np.conj(c[b * nh + i]) * S[el(a, b)] for b in range(ne)) + \
                    sum(np.conj(c[a * nh + j]) * S[he(i, j)] for j in range(nh))
                lt = sum(np.conj(c[b * nh + i]) * Lm[el(a, b)] for b in range(ne)) + \
                    sum(np.conj(c[a * nh + j]) * Lm[he(i, j)] for j in range(nh))
                spin[n] += c[ibs] * st
                orb[n] += c[ibs] * lt
                for b in range(ne):
                    for j in range(nh):
                        ct = np.conj(c[b * nh + j]) * c[ibs]
                        stot[n] += ct * np.sum(S[el(a, b)] * S[he(i, j)])
                        o = 2.0 * np.sum(Lm[el(a, b)] * Lm[he(i, j)])
                        if i == j:
                            o += L2[el(a, b)]
                        if a == b:
                            o += L2[he(i, j)]
                        otot[n] += ct * o
                        x = np.sum(Lm[el(a, b)] * S[he(i, j)]) + np.sum(S[el(a, b)] * Lm[he(i, j)])
                        if i == j:
                            x += LS[el(a, b)]
                        if a == b:
                            x += LS[he(i, j)]
                        lstot[n] += ct * x
    return spin, stot, orb, otot, lstot


def bse_optical(C, mu, nh, ne):
    """calc_optical_exc (bse_cplx/optical.c:36-80), electric part: exciton
    dipoles [n][3] and OS.dat's oscillator strengths need E: (2/3) E |mu|^2."""
    n = nh * ne
    out = np.zeros((n, 3), np.complex128)
    for a in range(ne):
        for i in range(nh):
            out += np.outer(C[a * nh + i, :], mu[i * ne + a])
    return out
