"""Pins the oracle's Bethe-Salpeter stage against the reference's own BSE code
(bse_cplx/ compiled from where it lies into oracle/_ref/libfbse_ref_bse.so with
the project-written FFTW subset, LAPACKE forwarder and one-rank MPI; CPU):
the bare and screened interactions, the direct and exchange kernels, the BSE
solve with its exciton expectation values, the electric and magnetic
transition dipoles and the optical outputs (OS.dat, M.dat), on smooth seeded
spinor states."""
import ctypes
import glob
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.test_bse_gpu import qp_states

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_BSE_SO = os.path.join(ROOT, "oracle", "_ref", "libfbse_ref_bse.so")
D = ctypes.POINTER(ctypes.c_double)
GRID = O.Grid(14, 13, 12, 0.8, 0.8, 0.8, -5.6, -5.2, -4.8)


def _p(a):
    return np.ascontiguousarray(a).ctypes.data_as(D)


@pytest.fixture(scope="module")
def rb():
    if not os.path.exists(REF_BSE_SO):
        pytest.skip("oracle/_ref not built (the reference tree is not mounted here)")
    L = ctypes.CDLL(REF_BSE_SO)
    gargs = [ctypes.c_long] * 3 + [ctypes.c_double] * 6 + [D] * 3
    L.ref_bse_potentials.argtypes = gargs + [ctypes.c_double] * 3 + [D, D]
    L.ref_bse_kernel.argtypes = [D] + [ctypes.c_long] * 3 + gargs + [D] * 4
    L.ref_bse_solve.argtypes = [D, D, D] + [ctypes.c_long] * 3 + [D, D]
    L.ref_bse_dipoles.argtypes = [D, D] + [ctypes.c_long] * 3 + gargs + [D]
    L.ref_bse_mag_dipoles.argtypes = [D, D] + [ctypes.c_long] * 3 + gargs + [D]
    L.ref_bse_optical.argtypes = [D] * 5 + [ctypes.c_long] * 3
    L.ref_bse_qp_ang_mom.argtypes = [D] + [ctypes.c_long] * 3 + gargs + [D] * 4
    L.ref_bse_xton_ang.argtypes = [D] * 5 + [ctypes.c_long] * 3
    L.ref_set_lapack.argtypes = [ctypes.c_char_p]
    here = os.path.dirname(os.path.dirname(np.__file__))
    lap = glob.glob(os.path.join(here, "numpy.libs", "libscipy_openblas64_*.so"))
    if not lap or not L.ref_set_lapack(lap[0].encode()):
        pytest.skip("numpy's ILP64 LAPACK is not available")
    return L


def _grid_args(g):
    axes = [np.ascontiguousarray(a) for a in O.bse_axes(g)]
    return axes, [g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.xmin, g.ymin, g.zmin] + [_p(a) for a in axes]


@pytest.mark.parametrize("g", [GRID, O.Grid(12, 10, 13, 0.8, 0.8, 0.8, -4.8, -4.0, -5.2)])
def test_bse_potentials_match_reference(rb, g):
    """init_elec_hole_kernel (bse_cplx/init.c:8-268)"""
    keep, ga = _grid_args(g)
    eps = (6.1, 5.3, 7.2)
    bare = np.empty(g.ngrid, np.complex128)
    scr = np.empty(g.ngrid, np.complex128)
    rb.ref_bse_potentials(*ga, *eps, _p(bare.view(np.float64)), _p(scr.view(np.float64)))
    mb, ms = O.bse_potentials(g, eps)
    assert np.max(np.abs(mb - bare)) < 1e-12 * np.max(np.abs(bare))
    assert np.max(np.abs(ms - scr)) < 1e-12 * np.max(np.abs(scr))


def _kernels(rb, g, psi, nh, ne, lumo, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)  # the kernel files
    keep, ga = _grid_args(g)
    bare, scr = O.bse_potentials(g, (6.0, 6.0, 6.0))
    n = nh * ne
    dr = np.zeros((n, n), np.complex128)
    xr = np.zeros((n, n), np.complex128)
    rb.ref_bse_kernel(_p(psi.view(np.float64)), nh, ne, lumo, *ga, _p(bare.view(np.float64)),
                      _p(scr.view(np.float64)), _p(dr.view(np.float64)), _p(xr.view(np.float64)))
    return bare, scr, dr, xr


def test_bse_kernels_match_reference(rb, tmp_path, monkeypatch):
    """calc_eh_kernel_cplx (bse_cplx/coulomb.c:20-738) at one rank: the lower
    triangles (ibs >= jbs) of the screened direct and bare exchange kernels"""
    nh, ne, lumo = 3, 2, 4
    psi = np.ascontiguousarray(qp_states(GRID, lumo + ne, 41))
    bare, scr, dr, xr = _kernels(rb, GRID, psi, nh, ne, lumo, tmp_path, monkeypatch)
    dm, xm = O.bse_kernels(psi, nh, ne, lumo, bare, scr, GRID)
    low = np.tril(np.ones((nh * ne, nh * ne), bool))
    scale = max(np.max(np.abs(dm)), np.max(np.abs(xm)))
    print(f"\n[reference BSE kernels] max |K^d| {np.max(np.abs(dm)):.3e}, max |K^x| {np.max(np.abs(xm)):.3e}, "
          f"max dev {max(np.max(np.abs(dm - dr)[low]), np.max(np.abs(xm - xr)[low])):.1e}")
    assert np.max(np.abs(dm - dr)[low]) < 1e-12 * scale
    assert np.max(np.abs(xm - xr)[low]) < 1e-12 * scale


def test_bse_solve_matches_reference(rb, tmp_path, monkeypatch):
    """build_h0_mat, build_BSE_mat, bethe_salpeter (bse_cplx/mod_bse.c:54-148,
    bethe-salpeter.c:7-350): exciton energies, coefficients (up to phase,
    non-degenerate excitons) and the expectation values of exciton.dat"""
    nh, ne, lumo = 3, 2, 4
    psi = np.ascontiguousarray(qp_states(GRID, lumo + ne, 43))
    _, _, dr, xr = _kernels(rb, GRID, psi, nh, ne, lumo, tmp_path, monkeypatch)
    rng = np.random.default_rng(5)
    ev = np.sort(np.concatenate([rng.uniform(-0.30, -0.20, lumo), rng.uniform(-0.05, 0.05, ne)]))
    n = nh * ne
    xe = np.zeros(n)
    cf = np.zeros((n, n), np.complex128)
    # the reference's solve works in its kernel arrays: hand it copies
    rb.ref_bse_solve(_p(dr.copy().view(np.float64)), _p(xr.copy().view(np.float64)), _p(ev), nh, ne, lumo, _p(xe),
                     _p(cf.view(np.float64)))
    e, C, eh, ed, ex, e0 = O.bse_solve(ev, nh, ne, lumo, dr, xr)
    assert np.max(np.abs(xe - e)) < 1e-13
    gaps = np.diff(e)
    for j in range(n):
        if (j == 0 or gaps[j - 1] > 1e-8) and (j == n - 1 or gaps[j] > 1e-8):
            assert abs(abs(np.vdot(cf[:, j], C[:, j])) - 1.0) < 1e-10
    rows = np.loadtxt(tmp_path / "exciton.dat")
    assert rows.shape == (n, 7)
    # E_n, <H>, <H_dir>, <H_exc>, <H_0> ("% .12f", bethe-salpeter.c:337-346)
    for col, want in ((1, e), (2, eh), (3, ed), (4, ex), (5, e0)):
        assert np.allclose(rows[:, col], want, atol=1e-11), col


def test_bse_dipoles_match_reference(rb, tmp_path, monkeypatch):
    """calc_elec_dipole (bse_cplx/dipole.c:7-158): <i| r |a> for every hole /
    electron pair"""
    monkeypatch.chdir(tmp_path)
    nh, ne, lumo = 3, 2, 4
    psi = np.ascontiguousarray(qp_states(GRID, lumo + ne, 47))
    ev = np.linspace(-0.3, 0.0, lumo + ne)
    keep, ga = _grid_args(GRID)
    mu = np.zeros((nh * ne, 3), np.complex128)
    rb.ref_bse_dipoles(_p(psi.view(np.float64)), _p(ev), nh, ne, lumo, *ga, _p(mu.view(np.float64)))
    mine = O.bse_dipoles(psi, nh, ne, lumo, GRID)
    assert np.max(np.abs(mine - mu)) < 1e-12 * np.max(np.abs(mine))


def test_bse_mag_dipoles_and_optical_match_reference(rb, tmp_path, monkeypatch):
    """calc_mag_dipole (bse_cplx/dipole.c:160-331) against the oracle, and
    calc_optical_exc (optical.c:6-99) on the reference's own exciton
    coefficients: OS.dat's |mu|, E and (2/3) E |mu|^2 and M.dat's |m| from the
    oracle's exciton dipoles"""
    monkeypatch.chdir(tmp_path)
    nh, ne, lumo = 3, 2, 4
    psi = np.ascontiguousarray(qp_states(GRID, lumo + ne, 53))
    ev = np.linspace(-0.3, 0.0, lumo + ne)
    keep, ga = _grid_args(GRID)
    m = np.zeros((nh * ne, 3), np.complex128)
    rb.ref_bse_mag_dipoles(_p(psi.view(np.float64)), _p(ev), nh, ne, lumo, *ga, _p(m.view(np.float64)))
    mine_m = O.bse_mag_dipoles(psi, nh, ne, lumo, GRID)
    assert np.max(np.abs(mine_m - m)) < 1e-12 * np.max(np.abs(mine_m))
    mu = O.bse_dipoles(psi, nh, ne, lumo, GRID)
    _, _, dr, xr = _kernels(rb, GRID, psi, nh, ne, lumo, tmp_path, monkeypatch)
    e, C, *_ = O.bse_solve(ev, nh, ne, lumo, dr, xr)
    n = nh * ne
    rb.ref_bse_optical(_p(np.ascontiguousarray(C).view(np.float64)), _p(e), _p(ev),
                       _p(np.ascontiguousarray(mu).view(np.float64)), _p(np.ascontiguousarray(m).view(np.float64)),
                       nh, ne, lumo)
    os_rows = np.loadtxt(tmp_path / "OS.dat")
    m_rows = np.loadtxt(tmp_path / "M.dat")
    mx = O.bse_optical(C, mu, nh, ne)
    mm = O.bse_optical(C, m, nh, ne)
    osc = np.sum(np.abs(mx) ** 2, axis=1)
    assert os_rows.shape[0] == m_rows.shape[0] == n
    assert np.allclose(os_rows[:, 1], np.sqrt(osc), atol=2e-8)
    assert np.allclose(os_rows[:, 2], e, atol=2e-8)
    assert np.allclose(os_rows[:, 3], 2.0 / 3.0 * e * osc, atol=2e-8)
    assert np.allclose(m_rows[:, 1], np.sqrt(np.sum(np.abs(mm) ** 2, axis=1)), atol=2e-8)


def test_bse_spin_and_angular_matrices_match_reference(rb, tmp_path, monkeypatch):
    """calc_qp_spin_mtrx and calc_qp_ang_mom_mtrx (bse_cplx/angular.c:7-690)
    against the oracle's quasiparticle s, l, l^2 and l.s matrices; then
    calc_xton_spin_mtrx and calc_xton_ang_mom_mtrx (angular.c:692-1043) on the
    reference's matrices and the oracle's exciton coefficients: spins.dat,
    orbital.dat and couple.dat against the oracle's exciton sums to their
    printed digits.  The electron block of <L.S> is the reference's loop as
    written (its spin-down index stays at the first point), which the oracle
    restates separately; the library computes the L.S sums for both blocks."""
    monkeypatch.chdir(tmp_path)
    nh, ne, lumo = 3, 2, 4
    psi = np.ascontiguousarray(qp_states(GRID, lumo + ne, 67))
    keep, ga = _grid_args(GRID)
    nq = nh * nh + ne * ne
    s = np.zeros((nq, 3), np.complex128)
    l = np.zeros((nq, 3), np.complex128)
    l2 = np.zeros(nq, np.complex128)
    ls = np.zeros(nq, np.complex128)
    rb.ref_bse_qp_ang_mom(_p(psi.view(np.float64)), nh, ne, lumo, *ga, *[_p(a.view(np.float64)) for a in (s, l, l2, ls)])
    S, Lm, L2, LS = O.bse_qp_ang_mom(psi, nh, ne, lumo, GRID)
    hh = nh * nh
    for mine, ref in ((S, s), (Lm, l), (L2, l2), (LS[:hh], ls[:hh])):
        assert np.max(np.abs(mine - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))
    # the electron L.S loop (angular.c:582-604) never advances its spin-down
    # index: the reference's numbers are that loop as written, not the L.S sums
    quirk = O.bse_electron_ls_as_written(psi, nh, ne, lumo, GRID)
    assert np.max(np.abs(quirk - ls[hh:])) < 1e-12 * max(1.0, np.max(np.abs(quirk)))
    assert np.max(np.abs(LS[hh:] - ls[hh:])) > 1e-3
    ev = np.linspace(-0.3, 0.0, lumo + ne)
    _, _, dr, xr = _kernels(rb, GRID, psi, nh, ne, lumo, tmp_path, monkeypatch)
    e, C, *_ = O.bse_solve(ev, nh, ne, lumo, dr, xr)
    C = np.ascontiguousarray(C)
    rb.ref_bse_xton_ang(_p(C.view(np.float64)), *[_p(a.view(np.float64)) for a in (s, l, l2, ls)], nh, ne, lumo)
    # both sides on the reference's own matrices (its electron L.S included)
    spin, stot, orb, otot, lstot = O.xton_ang_stats(C, s, l, l2, ls, nh, ne)
    n = nh * ne
    def rows(name):  # "(imaginary part)" columns read as plain numbers
        return np.array([[float(t) for t in line.replace("(", " ").replace(")", " ").split()]
                         for line in open(tmp_path / name)])

    sp, ob, cp = rows("spins.dat"), rows("orbital.dat"), rows("couple.dat")
    assert sp.shape == (n, 9) and ob.shape == (n, 6) and cp.shape == (n, 3)
    # spins.dat: %.5g of Re/Im <S_d>, then 1.5 + 2 Re(sum), (2 Im(sum))
    want = np.column_stack([spin.real[:, 0], spin.imag[:, 0], spin.real[:, 1], spin.imag[:, 1],
                            spin.real[:, 2], spin.imag[:, 2], 1.5 + 2 * stot.real, 2 * stot.imag])
    assert np.allclose(sp[:, 1:], want, rtol=1e-4, atol=1e-9)
    # orbital.dat and couple.dat: %.5f
    assert np.allclose(ob[:, 1:], np.column_stack([orb.real, otot.real, otot.imag]), atol=6e-6)
    assert np.allclose(cp[:, 1:], np.column_stack([lstot.real, lstot.imag]), atol=6e-6)


@pytest.mark.parametrize("name,cut,fermi,mh,me", [("cspbi3", 1e-4, -0.19, 10, 10), ("cspbi3", 1e-4, -0.19, -1, -1),
                                                  ("cspbi3", 1e-4, -0.19, 3, -1), ("cdse22", 1e-3, -0.18, 4, 3),
                                                  ("cdse22", 1e-3, -0.18, -1, 2), ("cdse22", 5e-4, -0.18, 100, 100)])
def test_qp_basis_matches_reference(rb, tmp_path, monkeypatch, name, cut, fermi, mh, me):
    """get_qp_basis_indices (bse_cplx/basis.c:7-254) on the examples' eval.dat
    against the library's host fbse_qp_basis: the kept holes (nearest the gap)
    and electrons, their eval.dat indices and counts, and the energies the
    reference carries for them"""
    import filterbse_gb300 as F
    monkeypatch.chdir(tmp_path)
    rb.ref_bse_qp_basis.argtypes = [D, D, ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_long,
                                    ctypes.c_long, ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_long)]
    ev = np.loadtxt(os.path.join(ROOT, "tests", "golden", name, "eval.dat"))
    n = len(ev)
    e, s = np.ascontiguousarray(ev[:, 1]), np.ascontiguousarray(ev[:, 2])
    sel = np.zeros(n, np.int64)
    info = np.zeros(4, np.int64)
    er, sr = e.copy(), s.copy()  # the reference reorders them in place
    rb.ref_bse_qp_basis(_p(er), _p(sr), n, cut, fermi, mh, me, sel.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                        info.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
    nh, ne = int(info[0]), int(info[1])
    assert nh >= 1 and ne >= 1 and info[3] == info[2] + 1 == nh
    L = F.load()
    Lp = ctypes.POINTER(ctypes.c_long)
    L.fbse_qp_basis.argtypes = [D, D, ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_long, ctypes.c_long,
                                Lp, Lp, Lp]
    L.fbse_qp_basis.restype = ctypes.c_long
    mine = np.zeros(n, np.int64)
    hn, hne = ctypes.c_long(), ctypes.c_long()
    nq = L.fbse_qp_basis(_p(e), _p(s), n, cut, fermi, mh, me, mine.ctypes.data_as(Lp), ctypes.byref(hn),
                         ctypes.byref(hne))
    assert (hn.value, hne.value, nq) == (nh, ne, nh + ne)
    assert np.array_equal(mine[:nq], sel[:nq])
    assert np.array_equal(er[:nh], e[mine[:nh]])
    conv = np.flatnonzero(s < cut)
    if me == -1 and mh != -1 and int(np.sum(e[conv] < fermi)) > mh:
        # holes cut to maxHoleStates with maxElecStates = -1: the reference
        # skips its electron reordering (basis.c:176-198), so the energies it
        # keeps for the electrons are the converged list's entries after the
        # kept holes -- dropped holes -- not the electrons'
        compact = e[conv]
        assert np.array_equal(er[nh:nq], compact[nh:nq]) and not np.array_equal(er[nh:nq], e[mine[nh:nq]])
    else:
        assert np.array_equal(er[nh:nq], e[mine[nh:nq]])


class BseParams(ctypes.Structure):
    _fields_ = [("max_hole_states", ctypes.c_long), ("max_elec_states", ctypes.c_long),
                ("sigma_e_cut", ctypes.c_double), ("eps_x", ctypes.c_double), ("eps_y", ctypes.c_double),
                ("eps_z", ctypes.c_double), ("fermi_e", ctypes.c_double), ("delta_e_hole", ctypes.c_double),
                ("delta_e_elec", ctypes.c_double), ("precision", ctypes.c_int), ("coulomb_done", ctypes.c_int),
                ("restart_coulomb", ctypes.c_int), ("calc_coulomb_only", ctypes.c_int),
                ("calc_spin_ang_stat", ctypes.c_int)]


@pytest.mark.parametrize("text", [
    "epsX = 5.0\nepsY = 5.0\nepsZ = 5.0\n",
    "maxHoleStates = 10\nmaxElecStates = 10\nsigmaECut = 0.0001\nepsX = 6.1\nepsY = 6.1\nepsZ = 6.1\n"
    "nThreads = 1\nspinOrbit = 1\nNonLocal = 1\ncalcDarkStates = 0\ncalcSpinAngStat = 0\n",
    "maxHoleStates = 4\nmaxElecStates = 3\nsigmaECut = 0.01\nepsX = 5.0\nepsY = 5.5\nepsZ = 6.0\n"
    "fermiEnergy = -0.2\ndeltaEhole = 0.1\ndeltaEelec = 0.05\ncoulombDone = 1\nrestartCoulomb = 0\n"
    "calcCoulombOnly = 1\n"])
def test_bse_input_parser_matches_reference(rb, tmp_path, monkeypatch, text):
    """read_input of the BSE stage (bse_cplx/read.c:7-220) against the
    library's host fbse_read_bse_params: basis limits, cut, dielectric
    constants, Fermi energy, energy spans, kernel-file switches and
    calcSpinAngStat, defaults included"""
    import filterbse_gb300 as F
    (tmp_path / "input.par").write_text(text)
    monkeypatch.chdir(tmp_path)
    rb.ref_bse_read_input.argtypes = [D, ctypes.POINTER(ctypes.c_long)]
    d = np.zeros(8)
    lv = np.zeros(9, np.int64)
    rb.ref_bse_read_input(_p(d), lv.ctypes.data_as(ctypes.POINTER(ctypes.c_long)))
    L = F.load()
    L.fbse_read_bse_params.argtypes = [ctypes.c_char_p, ctypes.POINTER(BseParams), ctypes.c_char_p, ctypes.c_size_t]
    p = BseParams()
    err = ctypes.create_string_buffer(512)
    assert L.fbse_read_bse_params(b"input.par", ctypes.byref(p), err, 512) == 0, err.value
    assert [p.sigma_e_cut, p.eps_x, p.eps_y, p.eps_z, p.fermi_e, p.delta_e_hole, p.delta_e_elec] == list(d[:7])
    assert [p.max_hole_states, p.max_elec_states, p.coulomb_done, p.restart_coulomb, p.calc_coulomb_only,
            p.calc_spin_ang_stat] == [int(v) for v in lv[:6]]


def test_qp_spins_dat_matches_reference(rb, tmp_path, monkeypatch):
    """qp_spin_frac (bse_cplx/spin.c:3-60) against the library's host
    fbse_write_qp_spins: qp_spins.dat byte for byte"""
    import filterbse_gb300 as F
    monkeypatch.chdir(tmp_path)
    rb.ref_bse_qp_spins.argtypes = [D, D] + [ctypes.c_long] * 4 + [ctypes.c_double]
    psi = np.ascontiguousarray(qp_states(GRID, 7, 79))
    ev = np.ascontiguousarray(np.linspace(-0.31, -0.02, 7))
    rb.ref_bse_qp_spins(_p(psi.view(np.float64)), _p(ev), 7, GRID.nx, GRID.ny, GRID.nz, GRID.dv)
    L = F.load()
    L.fbse_write_qp_spins.argtypes = [ctypes.c_char_p, D, D, ctypes.c_long, ctypes.c_long, ctypes.c_double]
    assert L.fbse_write_qp_spins(b"mine_qp_spins.dat", _p(psi.view(np.float64)), _p(ev), 7, GRID.ngrid, GRID.dv) == 0
    assert open("mine_qp_spins.dat", "rb").read() == open("qp_spins.dat", "rb").read()


def test_kernel_files_match_reference(rb, tmp_path, monkeypatch):
    """direct-0.dat / exchange-0.dat as calc_eh_kernel_cplx writes them
    (bse_cplx/coulomb.c:289-371, 534-602) against the library's host
    fbse_write_kernel_files on the reference's own kernels, byte for byte"""
    import filterbse_gb300 as F
    nh, ne, lumo = 3, 2, 4
    psi = np.ascontiguousarray(qp_states(GRID, lumo + ne, 83))
    _, _, dr, xr = _kernels(rb, GRID, psi, nh, ne, lumo, tmp_path, monkeypatch)
    mine = tmp_path / "mine"
    mine.mkdir()
    monkeypatch.chdir(mine)
    L = F.load()
    L.fbse_write_kernel_files.argtypes = [D, D] + [ctypes.c_long] * 3 + [ctypes.c_int]
    assert L.fbse_write_kernel_files(_p(dr.view(np.float64)), _p(xr.view(np.float64)), nh, ne, lumo, 0) == 0
    for name in ("direct-0.dat", "exchange-0.dat"):
        assert (mine / name).read_bytes() == (tmp_path / name).read_bytes(), name


def test_bse_matrix_files_match_reference(rb, tmp_path, monkeypatch):
    """h0.dat, bsRE/IM.dat, HBSmatRE/IM.dat and BSEcoeffRE/IM.dat as
    build_h0_mat / build_BSE_mat / bethe_salpeter write them
    (bse_cplx/mod_bse.c:54-148, bethe-salpeter.c:7-133) against the library's
    host fbse_write_bse_matrices on the same kernels (full Hermitian) and the
    reference's own eigenvectors, byte for byte"""
    import filterbse_gb300 as F
    nh, ne, lumo = 3, 2, 4
    psi = np.ascontiguousarray(qp_states(GRID, lumo + ne, 97))
    _, _, dr, xr = _kernels(rb, GRID, psi, nh, ne, lumo, tmp_path, monkeypatch)
    ev = np.ascontiguousarray(np.linspace(-0.3, 0.02, lumo + ne))
    n = nh * ne
    xe = np.zeros(n)
    cf = np.zeros((n, n), np.complex128)
    rb.ref_bse_solve(_p(dr.copy().view(np.float64)), _p(xr.copy().view(np.float64)), _p(ev), nh, ne, lumo, _p(xe),
                     _p(cf.view(np.float64)))
    full = [np.ascontiguousarray(np.tril(m) + np.conj(np.tril(m, -1)).T) for m in (dr, xr)]
    mine = tmp_path / "mine"
    mine.mkdir()
    monkeypatch.chdir(mine)
    L = F.load()
    L.fbse_write_bse_matrices.argtypes = [D, D, D, D] + [ctypes.c_long] * 3 + [ctypes.c_int]
    assert L.fbse_write_bse_matrices(_p(full[0].view(np.float64)), _p(full[1].view(np.float64)),
                                     _p(cf.view(np.float64)), _p(ev), nh, ne, lumo, 0) == 0
    for name in ("h0.dat", "bsRE.dat", "bsIM.dat", "HBSmatRE.dat", "HBSmatIM.dat", "BSEcoeffRE.dat",
                 "BSEcoeffIM.dat"):
        assert (mine / name).read_bytes() == (tmp_path / name).read_bytes(), name
