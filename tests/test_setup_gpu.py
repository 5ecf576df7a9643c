"""The setup kernels on the GPU against the oracle: the local potential
(build_local_pot, filter_mpi/init.c:481-703) and the projector table
(init_NL_projectors, filter_mpi/init.c:848-1135).  Both are evaluated without
fused multiply-adds, so the table matches the oracle's plain IEEE evaluation
bit for bit; the potential sums the atoms in the same order."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import GOLD, cdse_tables, read_conf

pytestmark = pytest.mark.gpu

D = ctypes.POINTER(ctypes.c_double)


@pytest.mark.parametrize("shape,nat,box", [((24, 22, 20), 3, 3.0), ((37, 41, 29), 9, 6.0), ((64, 64, 64), 40, 12.0)])
def test_projector_table_matches_oracle(fbse, cuda, shape, nat, box):
    nx, ny, nz = shape
    g = O.Grid(nx, ny, nz, 0.5, 0.5, 0.5, -nx * 0.25, -ny * 0.25 + 0.1, -nz * 0.25 - 0.07)
    rng = np.random.default_rng(nat)
    xyz = rng.uniform(-box, box, (nat, 3))
    xyz[0] = [g.xmin - 1.0, 0.0, 0.0]  # a sphere cut by the grid edge
    so_par = rng.uniform(0.1, 1.0, nat)
    so_tab = rng.normal(size=(5, 1024))
    nl_tab = rng.normal(size=(nat, 5, 1024))
    sgn = rng.choice([-1, 1], size=(nat, 5)).astype(np.int32)
    ref = O.nlc_table(g, xyz, so_par, so_tab, nl_tab, sgn)
    nl, npts, jx, y1, sp, nlp = fbse.build_nlc(g.axes(), xyz, so_par, so_tab, nl_tab, 5, O.r_nlcut2(g.dx))
    assert npts == ref.npts
    assert np.array_equal(nl, ref.nl)
    assert np.array_equal(jx, ref.jxyz)
    assert np.array_equal(y1, ref.y1)
    assert np.array_equal(sp, ref.proj)
    assert np.array_equal(nlp, ref.nlp)


def test_projector_table_without_tables_and_atoms(fbse, cuda):
    g = O.Grid(16, 16, 16, 0.5, 0.5, 0.5, -4.0, -4.0, -4.0)
    nl, npts, jx, y1, sp, nlp = fbse.build_nlc(g.axes(), np.array([[0.1, 0.2, -0.3]]), None, None, None, 5,
                                               O.r_nlcut2(g.dx))
    assert nl[0] == npts > 100 and not sp.any() and not nlp.any()
    nl, npts, jx, y1, sp, nlp = fbse.build_nlc(g.axes(), np.zeros((0, 3)), None, None, None, 5, O.r_nlcut2(g.dx))
    assert len(nl) == 0 and npts == 1


def _local_pot(fbse, g, xyz, tidx, tables):
    L = fbse.load()
    L.fbse_build_local_pot.argtypes = [ctypes.c_long] * 3 + [D] * 3 + [ctypes.c_long, D, ctypes.POINTER(ctypes.c_int),
                                                                       ctypes.c_int, D, D,
                                                                       ctypes.POINTER(ctypes.c_long),
                                                                       ctypes.POINTER(ctypes.c_long), D]
    gx, gy, gz = (np.ascontiguousarray(a) for a in g.axes())
    tr = np.concatenate([t[0] for t in tables])
    tv = np.concatenate([t[1] for t in tables])
    tl = np.array([len(t[0]) for t in tables], np.int64)
    to = np.concatenate([[0], np.cumsum(tl)[:-1]]).astype(np.int64)
    R = np.ascontiguousarray(xyz, np.float64)
    at = np.ascontiguousarray(tidx, np.int32)
    pot = np.empty(g.ngrid)
    rc = L.fbse_build_local_pot(g.nx, g.ny, g.nz, gx.ctypes.data_as(D), gy.ctypes.data_as(D), gz.ctypes.data_as(D),
                                len(R), R.ctypes.data_as(D), at.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                len(tables), tr.ctypes.data_as(D), tv.ctypes.data_as(D),
                                to.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                                tl.ctypes.data_as(ctypes.POINTER(ctypes.c_long)), pot.ctypes.data_as(D))
    assert rc == 0
    return pot


def test_local_potential_matches_oracle_and_reference_cube(fbse, cuda):
    """fbse_build_local_pot on the 2.2 nm CdSe example: against the oracle on
    the whole grid, and against the reference's own localPot.cube sample."""
    lines = open(os.path.join(GOLD, "cdse22", "localPot_sample.txt")).read().splitlines()
    hdr = [l[1:].split() for l in lines if l.startswith("#")][2:6]
    xmin, ymin, zmin = float(hdr[0][1]), float(hdr[0][2]), float(hdr[0][3])
    nx, ny, nz = int(hdr[1][0]), int(hdr[2][0]), int(hdr[3][0])
    d = float(hdr[1][1])
    vals = np.array([l.split() for l in lines if not l.startswith("#")], float)
    atyp, xyz = read_conf(os.path.join(GOLD, "cdse22", "conf.par"))
    types = sorted(set(atyp), key=atyp.index)
    tidx = np.array([types.index(a) for a in atyp])
    g = O.Grid(nx, ny, nz, d, d, d, xmin, ymin, zmin, 10.0)
    tables = cdse_tables(types)
    got = _local_pot(fbse, g, xyz, tidx, tables)
    want = O.local_pot(g, xyz, tidx, tables)
    assert np.max(np.abs(got - want)) < 1e-12 * np.max(np.abs(want))
    ci = vals[:, 0].astype(int)  # cube order: x outer, y, z inner
    ix, rem = np.divmod(ci, ny * nz)
    iy, iz = np.divmod(rem, nz)
    assert np.allclose(got[nx * (ny * iz + iy) + ix], vals[:, 1], rtol=1e-4, atol=6e-5)  # "%.5g" in the cube
