"""Pins the oracle's real-valued Bethe-Salpeter stage against the reference's
own bse_real/ code (compiled from where it lies into
oracle/_ref/libfbse_ref_bse_real.so with the project-written FFTW subset, the
LAPACK forwarders and one-rank MPI; CPU): the interactions, the real direct
and exchange kernels (singlet factor 2 on the exchange), the dsyev solve with
its exciton.dat, the electric and magnetic transition dipoles and the optical
outputs, on smooth seeded real one-component states."""
import ctypes
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.test_bse_gpu import qp_states
from tests.test_oracle_pin_bse import GRID, _grid_args, _p

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BSER_SO = os.path.join(ROOT, "oracle", "_ref", "libfbse_ref_bse_real.so")
D = ctypes.POINTER(ctypes.c_double)
AUTOEV = 27.2114  # bse_real/fd.h


@pytest.fixture(scope="module")
def rr():
    if not os.path.exists(REF_BSER_SO):
        pytest.skip("oracle/_ref not built (the reference tree is not mounted here)")
    L = ctypes.CDLL(REF_BSER_SO)
    gargs = [ctypes.c_long] * 3 + [ctypes.c_double] * 6 + [D] * 3
    L.ref_bser_potentials.argtypes = gargs + [ctypes.c_double] * 3 + [D, D]
    L.ref_bser_kernel.argtypes = [D] + [ctypes.c_long] * 3 + gargs + [D] * 4
    L.ref_bser_solve.argtypes = [D, D, D] + [ctypes.c_long] * 3 + [D, D]
    L.ref_bser_dipoles.argtypes = [D, D] + [ctypes.c_long] * 3 + gargs + [D, D]
    L.ref_bser_optical.argtypes = [D] * 5 + [ctypes.c_long] * 3
    L.ref_set_lapack.argtypes = [ctypes.c_char_p]
    here = os.path.dirname(os.path.dirname(np.__file__))
    lap = glob.glob(os.path.join(here, "numpy.libs", "libscipy_openblas64_*.so"))
    if not lap or not L.ref_set_lapack(lap[0].encode()):
        pytest.skip("numpy's ILP64 LAPACK is not available")
    return L


def real_states(g, n, seed):
    psi = qp_states(g, n, seed, nspin=1).real.copy()
    psi /= np.sqrt(np.sum(psi ** 2, axis=1) * g.dv)[:, None]
    return np.ascontiguousarray(psi)


def test_bse_real_potentials_match_reference(rr):
    """init_elec_hole_kernel (bse_real/init.c:8-283)"""
    keep, ga = _grid_args(GRID)
    bare = np.empty(GRID.ngrid, np.complex128)
    scr = np.empty(GRID.ngrid, np.complex128)
    rr.ref_bser_potentials(*ga, 5.5, 6.5, 7.0, _p(bare.view(np.float64)), _p(scr.view(np.float64)))
    mb, ms = O.bse_potentials(GRID, (5.5, 6.5, 7.0))
    assert np.max(np.abs(mb - bare)) < 1e-12 * np.max(np.abs(bare))
    assert np.max(np.abs(ms - scr)) < 1e-12 * np.max(np.abs(scr))


def _kernels(rr, psi, nh, ne, lumo):
    keep, ga = _grid_args(GRID)
    bare, scr = O.bse_potentials(GRID, (6.0, 6.0, 6.0))
    n = nh * ne
    dr = np.zeros((n, n))
    xr = np.zeros((n, n))
    rr.ref_bser_kernel(_p(psi), nh, ne, lumo, *ga, _p(bare.view(np.float64)), _p(scr.view(np.float64)), _p(dr),
                       _p(xr))
    return bare, scr, dr, xr


def test_bse_real_kernels_and_solve_match_reference(rr, tmp_path, monkeypatch):
    """calc_eh_kernel_cplx of bse_real (coulomb.c:20-705) at one rank: the
    lower triangles of the real direct and exchange kernels; then
    build_h0_mat / build_BSE_mat / bethe_salpeter (mod_bse.c:59-130,
    bethe-salpeter.c:7-250): exciton energies, coefficients (row n = exciton
    n, up to sign) and the columns of exciton.dat as the real stage prints
    them -- after its step 4 the "<H>" column holds <h0>_n, and the <H_dir>,
    <H_exc>, <H_0> columns are the diagonals of the kernels and of h0
    (bethe-salpeter.c:215-250)"""
    monkeypatch.chdir(tmp_path)
    nh, ne, lumo = 3, 3, 4
    psi = real_states(GRID, lumo + ne, 71)
    bare, scr, dr, xr = _kernels(rr, psi, nh, ne, lumo)
    dm, xm = O.bse_kernels_real(psi, nh, ne, lumo, bare, scr, GRID)
    low = np.tril(np.ones(dm.shape, bool))
    scale = max(np.max(np.abs(dm)), np.max(np.abs(xm)))
    assert np.max(np.abs(dm - dr)[low]) < 1e-14 * scale
    assert np.max(np.abs(xm - xr)[low]) < 1e-14 * scale

    rng = np.random.default_rng(9)
    ev = np.sort(np.concatenate([rng.uniform(-0.30, -0.20, lumo), rng.uniform(-0.05, 0.05, ne)]))
    n = nh * ne
    xe = np.zeros(n)
    cf = np.zeros((n, n))
    # the reference's solve symmetrises its kernel arrays in place: hand it copies
    rr.ref_bser_solve(_p(dr.copy()), _p(xr.copy()), _p(ev), nh, ne, lumo, _p(xe), _p(cf))
    e, C, eh, ed, ex, e0 = O.bse_solve(ev, nh, ne, lumo, dr.astype(np.complex128), xr.astype(np.complex128))
    assert np.max(np.abs(xe - e)) < 1e-13
    gaps = np.diff(e)
    for j in range(n):
        if (j == 0 or gaps[j - 1] > 1e-8) and (j == n - 1 or gaps[j] > 1e-8):
            assert abs(abs(np.dot(cf[j], C[:, j].real)) - 1.0) < 1e-10
    rows = np.loadtxt(tmp_path / "exciton.dat")
    assert rows.shape == (n, 7)
    h0 = np.array([ev[lumo + b // nh] - ev[b % nh] for b in range(n)])  # pair ibs = a nh + i
    Df = np.tril(dr) + np.tril(dr, -1).T
    Xf = np.tril(xr) + np.tril(xr, -1).T
    for col, want in ((1, e), (2, e0), (3, np.diag(Df)), (4, np.diag(Xf)), (5, h0), (6, (e - h0) * AUTOEV)):
        assert np.allclose(rows[:, col], want, atol=1e-10), col


def test_bse_real_dipoles_and_optical_match_reference(rr, tmp_path, monkeypatch):
    """calc_elec_dipole / calc_mag_dipole of bse_real (dipole.c:7-331) against
    the oracle on the real states taken as complex one-component states, and
    calc_optical_exc (optical.c:6-100) on the reference's own coefficients:
    OS.dat's |mu|, E, (2/3) E |mu|^2 and mu, M.dat's |m|"""
    monkeypatch.chdir(tmp_path)
    nh, ne, lumo = 3, 2, 4
    psi = real_states(GRID, lumo + ne, 73)
    ev = np.linspace(-0.3, 0.0, lumo + ne)
    keep, ga = _grid_args(GRID)
    n = nh * ne
    mu = np.zeros((n, 3), np.complex128)
    m = np.zeros((n, 3), np.complex128)
    rr.ref_bser_dipoles(_p(psi), _p(ev), nh, ne, lumo, *ga, _p(mu.view(np.float64)), _p(m.view(np.float64)))
    pc = psi.astype(np.complex128)
    mine_mu = O.bse_dipoles(pc, nh, ne, lumo, GRID, nspin=1)
    mine_m = O.bse_mag_dipoles(pc, nh, ne, lumo, GRID, nspin=1)
    assert np.max(np.abs(mine_mu - mu)) < 1e-12 * np.max(np.abs(mine_mu))
    assert np.max(np.abs(mine_m - m)) < 1e-12 * np.max(np.abs(mine_m))

    _, _, dr, xr = _kernels(rr, psi, nh, ne, lumo)
    xe = np.zeros(n)
    cf = np.zeros((n, n))
    rr.ref_bser_solve(_p(dr.copy()), _p(xr.copy()), _p(ev), nh, ne, lumo, _p(xe), _p(cf))
    rr.ref_bser_optical(_p(cf), _p(xe), _p(ev), _p(mu.view(np.float64)), _p(m.view(np.float64)), nh, ne, lumo)
    os_rows = np.loadtxt(tmp_path / "OS.dat")
    m_rows = np.loadtxt(tmp_path / "M.dat")
    C = cf.T.astype(np.complex128)  # column n = exciton n
    mx = O.bse_optical(C, mu, nh, ne)
    mm = O.bse_optical(C, m, nh, ne)
    osc = np.sum(np.abs(mx) ** 2, axis=1)
    assert os_rows.shape == (n, 7) and m_rows.shape == (n, 10)
    assert np.allclose(os_rows[:, 1], np.sqrt(osc), atol=2e-8)
    assert np.allclose(os_rows[:, 2], xe, atol=2e-8)
    assert np.allclose(os_rows[:, 3], 2.0 / 3.0 * xe * osc, atol=2e-8)
    assert np.allclose(os_rows[:, 4:7], mx.real, atol=2e-12)
    assert np.allclose(m_rows[:, 1], np.sqrt(np.sum(np.abs(mm) ** 2, axis=1)), atol=2e-8)


def test_bse_real_kernel_files_match_reference(rr, tmp_path, monkeypatch):
    """direct-0.dat / exchange-0.dat of the real stage (bse_real/coulomb.c:352,
    583: one value per element) against the library's host
    fbse_write_kernel_files (real = 1) on the reference's own kernels"""
    import filterbse_gb300 as F
    monkeypatch.chdir(tmp_path)
    nh, ne, lumo = 3, 2, 4
    psi = real_states(GRID, lumo + ne, 89)
    _, _, dr, xr = _kernels(rr, psi, nh, ne, lumo)
    mine = tmp_path / "mine"
    mine.mkdir()
    monkeypatch.chdir(mine)
    L = F.load()
    L.fbse_write_kernel_files.argtypes = [D, D] + [ctypes.c_long] * 3 + [ctypes.c_int]
    pairs = [np.ascontiguousarray(np.stack([m, np.zeros_like(m)], axis=-1)) for m in (dr, xr)]
    assert L.fbse_write_kernel_files(_p(pairs[0]), _p(pairs[1]), nh, ne, lumo, 1) == 0
    for name in ("direct-0.dat", "exchange-0.dat"):
        assert (mine / name).read_bytes() == (tmp_path / name).read_bytes(), name


def test_bse_real_matrix_files_match_reference(rr, tmp_path, monkeypatch):
    """h0.dat, bs.dat, HBSmat.dat and BSEcoeff.dat of the real stage
    (bse_real/mod_bse.c:59-130, bethe-salpeter.c:70-114; BSEcoeff row n =
    exciton n) against the library's host fbse_write_bse_matrices (real = 1)
    on the same kernels and the reference's own eigenvectors, byte for byte"""
    import filterbse_gb300 as F
    monkeypatch.chdir(tmp_path)
    nh, ne, lumo = 3, 2, 4
    psi = real_states(GRID, lumo + ne, 101)
    _, _, dr, xr = _kernels(rr, psi, nh, ne, lumo)
    ev = np.ascontiguousarray(np.linspace(-0.3, 0.02, lumo + ne))
    n = nh * ne
    xe = np.zeros(n)
    cf = np.zeros((n, n))
    rr.ref_bser_solve(_p(dr.copy()), _p(xr.copy()), _p(ev), nh, ne, lumo, _p(xe), _p(cf))
    full = [np.tril(m) + np.tril(m, -1).T for m in (dr, xr)]
    pairs = [np.ascontiguousarray(np.stack([m, np.zeros_like(m)], axis=-1)) for m in full + [cf.T]]
    mine = tmp_path / "mine"
    mine.mkdir()
    monkeypatch.chdir(mine)
    L = F.load()
    L.fbse_write_bse_matrices.argtypes = [D, D, D, D] + [ctypes.c_long] * 3 + [ctypes.c_int]
    assert L.fbse_write_bse_matrices(_p(pairs[0]), _p(pairs[1]), _p(pairs[2]), _p(ev), nh, ne, lumo, 1) == 0
    for name in ("h0.dat", "bs.dat", "HBSmat.dat", "BSEcoeff.dat"):
        assert (mine / name).read_bytes() == (tmp_path / name).read_bytes(), name
