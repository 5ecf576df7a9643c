"""Small test systems for the parity tests, built with the oracle (test-only).

tiny_cluster(): a handful of atoms from the 2.2 nm CdSe example (golden
fixture) on a small grid with awkward axis lengths, local potential from the
reference's II-VI tables, and optionally a projector table.
"""
import os

import numpy as np

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def read_conf(path):
    with open(path) as f:
        n = int(f.readline().split()[0])
        at, xyz = [], []
        for _ in range(n):
            p = f.readline().split()
            at.append(p[0])
            xyz.append([float(p[1]), float(p[2]), float(p[3])])
    xyz = np.array(xyz)
    return at, xyz - xyz.mean(axis=0)  # centerConf (read.c:1135-1148)


def read_pot(path):
    d = np.loadtxt(path)
    return d[:, 0].copy(), d[:, 1].copy()


def cdse_tables(types):
    return [read_pot(os.path.join(GOLD, "cdse22", f"pot{t}.par")) for t in types]


def tiny_cluster(nx=24, ny=21, nz=22, d=0.8, natoms=12, nspin=1, is_complex=False, so=False, nl=False,
                 ke_max=10.0, seed=7):
    atyp, xyz = read_conf(os.path.join(GOLD, "cdse22", "conf.par"))
    order = np.argsort(np.sum(xyz ** 2, axis=1))[:natoms]
    atyp = [atyp[i] for i in order]
    xyz = xyz[order]
    types = sorted(set(atyp), key=atyp.index)
    tidx = np.array([types.index(a) for a in atyp])
    g = O.Grid(nx, ny, nz, d, d, d, -nx * d / 2, -ny * d / 2, -nz * d / 2, ke_max)
    pot = O.local_pot(g, xyz, tidx, cdse_tables(types))
    sysm = O.System(g, pot, nspin=nspin, is_complex=is_complex, so=so, nlflag=nl)
    if so or nl:
        core = [i for i, a in enumerate(atyp) if not a.startswith("P")]
        rng = np.random.default_rng(seed)
        rc = np.sqrt(O.r_nlcut2(d))
        so_tab = synthetic_radial(rc, rng, 0.3)
        nat = len(core)
        nl_tabs = np.stack([synthetic_radial(rc, rng, 0.5) for _ in core])
        sgn = rng.choice([-1, 1], size=(nat, O.NPROJ)).astype(np.int32)
        so_par = rng.uniform(0.2, 1.0, nat)
        sysm.proj = O.nlc_table(g, xyz[core], so_par, so_tab, nl_tabs, sgn)
    return sysm


def synthetic_radial(rc, rng, amp):
    """A smooth radial table [nproj][PROJ_LEN] (stands in for the projector
    generator where only the application kernels are under test)."""
    r = np.linspace(0, rc, O.PROJ_LEN, endpoint=False)
    out = []
    for p in range(O.NPROJ):
        w = rng.uniform(0.5, 1.5)
        out.append(amp * rng.uniform(0.5, 1.0) * np.exp(-(r / w) ** 2) * np.cos(p * r / rc * np.pi))
    return np.array(out)


def random_states(n, sysm, rng, real=None):
    real = (not sysm.is_complex) if real is None else real
    L = sysm.nspin * sysm.ngrid
    a = rng.uniform(-1, 1, (n, L))
    if real:
        return a.astype(np.complex128)
    return a + 1j * rng.uniform(-1, 1, (n, L))
