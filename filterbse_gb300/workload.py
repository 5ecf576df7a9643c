"""Synthetic nanocrystal workloads in the reference's own input model.

Builds what the reference reads from conf.par / pot*.par / SO_*.par and sets
up in mod_init / mod_pseudopot: a passivated zincblende CdSe sphere, the
grid of init_grid_params, the local potential of build_local_pot (on the GPU,
fbse_build_local_pot), the spin-orbit radial projectors of gen_SO_projectors
and the projector table of init_NL_projectors (on the GPU, fbse_build_nlc).  This is the input generator
(the counterpart of the reference's example scripts), not part of the
per-step hot path.

Recorded choices (the reference does not fix them):
  * lattice constant 6.08 A, zincblende, sphere centred on a Cd site; core
    atoms with fewer than two core neighbours are dropped (repeatedly);
  * one ligand per dangling bond along the bond: P1 at 0.55 of the bond from
    Cd, P2 at 0.25 from Se (the 2.2 nm CdSe example places them at 2.74 and
    1.24-1.49 bohr of a 4.97 bohr bond);
  * local potentials: the reference's shipped II-VI tables (potCd, potSe,
    potP1, potP2) -- the workload's form-factor parameters are not published,
    and the shipped tables stand in for them;
  * spin-orbit: SO_par = 0.01 for Cd and Se, NL parameters 0 (no NL term).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

ANG = 1.889726125  # bohr per angstrom (filter_mpi/fd.h ANGTOBOHR)
PROJ_LEN = 1024
NPROJ = 5
_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
POT_DIR = os.path.join(_ROOT, "tests", "golden", "cdse22")


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

    @property
    def ngrid(self):
        return self.nx * self.ny * self.nz

    @property
    def dv(self):
        return self.dx * self.dy * self.dz

    def axes(self):
        out = []
        for n, d, lo in ((self.nx, self.dx, self.xmin), (self.ny, self.dy, self.ymin), (self.nz, self.dz, self.zmin)):
            a = np.empty(n)
            v = lo
            for j in range(n):  # cumulative sums as build_grid_ksqr (init.c:284-290)
                a[j] = v
                v += d
            out.append(a)
        return out

    def dk(self):
        return tuple(2.0 * np.pi / (n * d if n % 2 == 0 else (n - 1) * d)
                     for n, d in ((self.nx, self.dx), (self.ny, self.dy), (self.nz, self.dz)))


@dataclass
class ProjTable:
    nl: np.ndarray
    npts: int
    jxyz: np.ndarray
    y1: np.ndarray
    proj: np.ndarray
    nlp: np.ndarray
    sgn: np.ndarray
    nproj: int = NPROJ


@dataclass
class Dot:
    types: list
    coords: np.ndarray  # bohr, centred
    grid: Grid
    pot: np.ndarray
    proj: ProjTable | None
    nspin: int
    is_complex: bool
    so: bool
    nl: bool

    @property
    def n_core(self):
        return sum(1 for t in self.types if not t.startswith("P"))


MATERIALS = {
    # cation, anion, lattice constant (A), directory of the local-potential tables
    "CdSe": ("Cd", "Se", 6.08, os.path.join(_ROOT, "tests", "golden", "cdse22")),
    "InP": ("In", "P", 5.87, os.path.join(_ROOT, "tests", "golden", "inp")),
}


def zincblende_dot(radius_ang: float, a_ang: float = 6.08, cation: str = "Cd", anion: str = "Se"):
    """Passivated zincblende sphere (CdSe by default); returns (types, coords
    in bohr), core first.  Ligands: P1 on the cation's dangling bonds, P2 on
    the anion's (the passivation model of the reference's CdSe and InP
    examples)."""
    a = a_ang * ANG
    R = radius_ang * ANG
    n = int(np.ceil(R / a)) + 2
    fcc = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    cells = np.array([[i, j, k] for i in range(-n, n + 1) for j in range(-n, n + 1) for k in range(-n, n + 1)], float)
    cd = (cells[:, None, :] + fcc[None]).reshape(-1, 3) * a
    se = cd + a * 0.25
    pos = np.vstack([cd, se])
    kind = np.array([0] * len(cd) + [1] * len(se))
    keep = np.linalg.norm(pos, axis=1) <= R
    pos, kind = pos[keep], kind[keep]
    bonds = a / 4.0 * np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], float)
    bl = np.linalg.norm(bonds[0])

    def neighbour_mask(pos, kind):
        from scipy.spatial import cKDTree
        tree = cKDTree(pos)
        has = np.zeros((len(pos), 4), bool)
        for b in range(4):
            sgn = np.where(kind == 0, 1.0, -1.0)[:, None]
            d, _ = tree.query(pos + sgn * bonds[b], distance_upper_bound=0.1)
            has[:, b] = np.isfinite(d)
        return has

    while True:
        has = neighbour_mask(pos, kind)
        ok = has.sum(axis=1) >= 2
        if ok.all():
            break
        pos, kind = pos[ok], kind[ok]
    has = neighbour_mask(pos, kind)
    lig_pos, lig_typ = [], []
    for i in range(len(pos)):
        sgn = 1.0 if kind[i] == 0 else -1.0
        for b in range(4):
            if not has[i, b]:
                frac = 0.55 if kind[i] == 0 else 0.25
                lig_pos.append(pos[i] + sgn * bonds[b] * frac)
                lig_typ.append("P1" if kind[i] == 0 else "P2")
    order = np.argsort(kind, kind="stable")
    types = [cation if k == 0 else anion for k in kind[order]] + lig_typ
    coords = np.vstack([pos[order], np.array(lig_pos).reshape(-1, 3)])
    coords = coords - coords.mean(axis=0)  # centerConf (read.c)
    return types, coords


def reference_grid(coords, d, ke_max=20.0, n_in=(0, 0, 0)) -> Grid:
    """init_grid_params (filter_mpi/init.c:5-255, non-periodic)."""
    dims = []
    for ax in range(3):
        c = coords[:, ax]
        ext = float(c.max() - c.min())
        xd = np.rint(0.5 * ext + 5.0)
        ntmp = int(((xd - d) - (-xd)) / d)
        n = n_in[ax]
        if ntmp > n:
            n = ntmp + (ntmp % 2)
        box = n * d if n % 2 == 0 else (n - 1) * d
        dims.append((n, -box / 2.0))
    return Grid(dims[0][0], dims[1][0], dims[2][0], d, d, d, dims[0][1], dims[1][1], dims[2][1], ke_max)


def read_table(path):
    t = np.loadtxt(path)
    return t[:, 0].copy(), t[:, 1].copy()


def local_pot(grid: Grid, types, coords, pot_dir=POT_DIR) -> np.ndarray:
    """Local potential on the GPU (fbse_build_local_pot).  Ligand tables
    (potP1 / potP2) come from the II-VI directory for every material."""
    from . import load
    uniq = sorted(set(types), key=types.index)
    tabs = [read_table(os.path.join(POT_DIR if t in ("P1", "P2") else pot_dir, f"pot{t}.par")) for t in uniq]
    tr = np.concatenate([t[0] for t in tabs])
    tv = np.concatenate([t[1] for t in tabs])
    tlen = np.array([len(t[0]) for t in tabs], np.int64)
    toff = np.concatenate([[0], np.cumsum(tlen)[:-1]]).astype(np.int64)
    at = np.array([uniq.index(t) for t in types], np.int32)
    gx, gy, gz = grid.axes()
    xyz = np.ascontiguousarray(coords, np.float64)
    pot = np.empty(grid.ngrid)
    D = ctypes.POINTER(ctypes.c_double)
    Lp = ctypes.POINTER(ctypes.c_long)
    L = load()
    L.fbse_build_local_pot.argtypes = [ctypes.c_long] * 3 + [D] * 3 + [ctypes.c_long, D,
                                                                     ctypes.POINTER(ctypes.c_int), ctypes.c_int, D, D,
                                                                     Lp, Lp, D]
    rc = L.fbse_build_local_pot(grid.nx, grid.ny, grid.nz, gx.ctypes.data_as(D), gy.ctypes.data_as(D),
                                gz.ctypes.data_as(D), len(at), xyz.ctypes.data_as(D),
                                at.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(uniq), tr.ctypes.data_as(D),
                                tv.ctypes.data_as(D), toff.ctypes.data_as(Lp), tlen.ctypes.data_as(Lp),
                                pot.ctypes.data_as(D))
    if rc:
        raise RuntimeError(f"fbse_build_local_pot failed ({rc})")
    return pot


def r_nlcut2(dx):
    return 1.5 + 6.0 * np.log(10.0) + 3.0 * dx  # read.c:908


def so_radial(dx, rcut, nproj=NPROJ):
    """gen_SO_projectors (filter_mpi/projectors.c:12-84) in numpy: the leading
    eigenvectors of the k-space matrix of the Gaussian (width 0.7) radial SO
    shape, transformed back to r on PROJ_LEN points."""
    N = PROJ_LEN
    dk = 1.5 * np.pi / dx / N
    dr = rcut / N
    k = np.arange(N) * dk
    r = np.arange(N) * dr
    kr = k[:, None] * r[None, :]
    x1 = 1.0 / (kr + 1e-10)
    J = np.where(kr < 1e-10, 0.0, np.sin(kr) * x1 * x1 - np.cos(kr) * x1)
    w = np.exp(-(r / 0.7) ** 2) * r * r * dr
    w[0] = 0.0
    A = (J * w[None, :]) @ J.T
    ev, vec = np.linalg.eigh(A)
    out = np.empty((nproj, N))
    for p in range(nproj):
        lam = ev[N - p - 1]
        out[p] = (2.0 / np.pi) * np.sqrt(lam) * ((k * k * dk)[None, :] * J.T * vec[:, N - p - 1][None, :]).sum(axis=1)
    return out


def nlc_table(grid: Grid, coords, so_par, so_tab, nproj=NPROJ) -> ProjTable:
    """init_NL_projectors (filter_mpi/init.c, body 508-589) on the GPU
    (fbse_build_nlc): grid points with r^2 < R_NLcut2 in jz, jy, jx order,
    Y_1m with the reference's EPSDX shifts, SO radial interpolated and scaled
    by sqrt(SO_par); no NL channels."""
    from . import build_nlc
    nl, npts, jx, y1, pj, nlp = build_nlc(grid.axes(), coords, so_par, so_tab, None, nproj, r_nlcut2(grid.dx))
    return ProjTable(nl.astype(np.int64), npts, jx, y1, pj, nlp, np.zeros(len(coords) * nproj, np.int32), nproj)


def cdse_dot(radius_ang: float, d: float = 0.5, ke_max: float = 20.0, spinor: bool = True, so_par: float = 0.01,
             grid_n=(0, 0, 0), material: str = "CdSe") -> Dot:
    cat, an, a_ang, pdir = MATERIALS[material]
    types, coords = zincblende_dot(radius_ang, a_ang, cat, an)
    grid = reference_grid(coords, d, ke_max, grid_n)
    pot = local_pot(grid, types, coords, pdir)
    proj = None
    if spinor:
        core = [i for i, t in enumerate(types) if not t.startswith("P")]
        tab = so_radial(d, np.sqrt(r_nlcut2(d)))
        proj = nlc_table(grid, coords[core], np.full(len(core), so_par), tab)
    return Dot(types, coords, grid, pot, proj, 2 if spinor else 1, spinor, spinor, False)


def smooth_size(n: int) -> int:
    """The smallest m >= n whose prime factors are all at most 7 (the radices
    the FFT kernels keep in registers)."""
    m = n
    while True:
        r = m
        for p in (2, 3, 5, 7):
            while r % p == 0:
                r //= p
        if r == 1:
            return m
        m += 1


def uneven_dots(n: int = 24, seed: int = 20261206, d_min_nm: float = 2.0, d_max_nm: float = 4.0, d: float = 0.5,
                ke_max: float = 10.0, max_grid: int = 160, smooth: bool = True):
    """The multi-dot workload: n passivated zincblende dots, CdSe and InP
    alternating, diameters uniform in [d_min_nm, d_max_nm] from a seeded
    generator, each on its own grid by the reference's grid rule (capped at
    max_grid points per axis, a recorded choice: the rule gives 104^3-190^3 for
    2-4 nm, the stated workload 64^3-160^3).  smooth: each axis grows to the
    next size with prime factors <= 7 (the rule's size is a minimum; the rule
    gives sizes such as 116 = 4 x 29 and 148 = 4 x 37, whose large prime radix
    takes the slow direct-DFT pass; the extra points are vacuum), a recorded
    choice.  Returns [(material, diameter_nm, Dot)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        mat = "CdSe" if i % 2 == 0 else "InP"
        dia = float(rng.uniform(d_min_nm, d_max_nm))
        cat, an, a_ang, pdir = MATERIALS[mat]
        types, coords = zincblende_dot(5.0 * dia, a_ang, cat, an)
        g = reference_grid(coords, d, ke_max)
        if max(g.nx, g.ny, g.nz) > max_grid:
            n_ = max_grid
            g = Grid(n_, n_, n_, d, d, d, -n_ * d / 2, -n_ * d / 2, -n_ * d / 2, ke_max)
        elif smooth:
            ns_ = [smooth_size(v) for v in (g.nx, g.ny, g.nz)]
            if ns_ != [g.nx, g.ny, g.nz]:
                g = reference_grid(coords, d, ke_max, n_in=tuple(ns_))
        pot = local_pot(g, types, coords, pdir)
        core = [k for k, t in enumerate(types) if not t.startswith("P")]
        tab = so_radial(d, np.sqrt(r_nlcut2(d)))
        proj = nlc_table(g, coords[core], np.full(len(core), 0.01), tab)
        out.append((mat, dia, Dot(types, coords, g, pot, proj, 2, True, True, False)))
    return out
