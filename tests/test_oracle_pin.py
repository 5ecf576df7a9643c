"""Pins the oracle: the C/numpy restatement against the reference's own
compiled functions (oracle/_ref, built from the reference tree when it is
present) and against the golden vectors of the reference's example runs
(tests/golden/, always present)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import GOLD, cdse_tables, read_conf

REF_SO = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref", "libfbse_ref.so")
D = ctypes.POINTER(ctypes.c_double)


def _p(a, t=D):
    return a.ctypes.data_as(t)


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF_SO):
        pytest.skip("oracle/_ref not built (the reference tree is not mounted here)")
    L = ctypes.CDLL(REF_SO)
    L.ref_ran.restype = ctypes.c_double
    L.ref_ran.argtypes = [ctypes.POINTER(ctypes.c_long)]
    L.ref_samp_points.restype = ctypes.c_double
    L.ref_samp_points.argtypes = [ctypes.c_long, D, D]
    L.ref_newton_coeff.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   D, D, D]
    L.ref_def_LS.argtypes = [D]
    L.ref_p_potential.argtypes = [D, D, D, D, ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.POINTER(ctypes.c_long),
                                  ctypes.POINTER(ctypes.c_int), D, D, D, ctypes.POINTER(ctypes.c_int), ctypes.c_double]
    L.ref_normalize_all.argtypes = [D, ctypes.c_long, ctypes.c_long, ctypes.c_int, ctypes.c_int, ctypes.c_double]
    return L


REF_FFT_SO = os.path.join(os.path.dirname(REF_SO), "libfbse_ref_fft.so")


@pytest.fixture(scope="module")
def ref_fft():
    """The reference's FFT-dependent files (kinetic(), calc_angular_exp)
    compiled with the project-written FFTW subset (oracle/ref_build)."""
    if not os.path.exists(REF_FFT_SO):
        pytest.skip("oracle/_ref not built (the reference tree is not mounted here)")
    L = ctypes.CDLL(REF_FFT_SO)
    L.ref_kinetic.argtypes = [D, D, ctypes.c_long, ctypes.c_long, ctypes.c_long, D]
    L.ref_angular.argtypes = ([D] + [ctypes.c_long] * 4 + [ctypes.c_double] * 3 + [D] * 3 + [ctypes.c_double] * 3 +
                              [ctypes.c_int] * 2)
    LP, IP = ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_int)
    table = [ctypes.c_long] * 3 + [LP, IP, D, D, D, IP, ctypes.c_double]
    L.ref_hamiltonian.argtypes = [D, D] + [ctypes.c_long] * 3 + [ctypes.c_int] * 4 + [D] * 3 + table
    L.ref_filter_cycle.argtypes = ([D] + [ctypes.c_long] * 3 + [ctypes.c_int] * 4 + [D] * 3 + table +
                                   [D, D, ctypes.c_long, ctypes.c_long, ctypes.c_double, ctypes.c_double])
    L.ref_ritz.argtypes = [D] + [ctypes.c_long] * 4 + [ctypes.c_int] * 3 + [D] * 3 + table + [D, D]
    L.ref_ritz.restype = ctypes.c_long
    L.ref_set_lapack.argtypes = [ctypes.c_char_p]
    L.ref_energy_range.argtypes = [ctypes.c_long] * 3 + [ctypes.c_int] * 3 + [D] * 3 + table + [D, D]
    return L


def _numpy_lapack():
    """numpy's bundled ILP64 LAPACK (OpenBLAS), which the reference's LAPACK
    calls are forwarded to in the pin library"""
    import glob
    here = os.path.dirname(os.path.dirname(np.__file__))
    found = glob.glob(os.path.join(here, "numpy.libs", "libscipy_openblas64_*.so"))
    return found[0] if found else None


def _table_args(sysm, so, nl):
    """the projector-table arguments of the reference harness for sysm"""
    pr = sysm.proj
    if pr is None:
        pr = O.Projectors(np.zeros(1, np.int64), 1, np.zeros(1, np.int32), np.zeros(6), np.zeros(5), np.zeros(5),
                          np.zeros(5, np.int32))
    return [pr.nat if (so or nl) else 0, pr.npts, pr.nproj, pr.nl.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
            pr.jxyz.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(pr.y1), _p(pr.proj), _p(pr.nlp),
            pr.sgn.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), sysm.grid.dv]


# ---------------------------------------------------------------- golden vectors

def test_rng_seed_sequence_golden():
    """seed.dat of a reference run: each random start draws 57*52*45 values."""
    rows = [l.split() for l in open(os.path.join(GOLD, "seed_2.2nm_CdSe.txt")).read().splitlines()[1:] if l.strip()]
    seeds = [int(r[1]) for r in rows]
    s = seeds[0]
    for want in seeds[1:]:
        _, s = O.ran_fill(s, 57 * 52 * 45, out=False)
        assert s == want


def test_leja_nodes_golden():
    ref = np.loadtxt(os.path.join(GOLD, "zn_2048.txt"))
    zn, _, _ = O.samp_points(2048)
    # the file holds "%lg" (6 significant digits)
    assert np.allclose(zn, ref[:, 1], rtol=6e-6, atol=1e-6)


def test_ksqr_golden():
    rows = np.loadtxt(os.path.join(GOLD, "ksqr_57x52x45.txt"), comments="#")
    # grid of that run: 57 x 52 x 45 at dx = 0.8, KEmax = 10; the version that
    # wrote it used box = n d on odd axes too (the current init.c uses (n-1) d)
    g = O.Grid(57, 52, 45, 0.8, 0.8, 0.8, -22.8, -20.8, -18.0, 10.0, box_n=True)
    k = g.ksqr()
    idx = rows[:, 0].astype(int)
    assert np.allclose(k[idx], rows[:, 1], rtol=6e-6, atol=1e-12)


def test_local_potential_golden():
    """build_local_pot on the 2.2 nm CdSe example vs the reference's localPot.cube."""
    lines = open(os.path.join(GOLD, "cdse22", "localPot_sample.txt")).read().splitlines()
    hdr = [l[1:].split() for l in lines if l.startswith("#")][2:6]
    xmin, ymin, zmin = float(hdr[0][1]), float(hdr[0][2]), float(hdr[0][3])
    nx, ny, nz = int(hdr[1][0]), int(hdr[2][0]), int(hdr[3][0])
    d = float(hdr[1][1])
    vals = np.array([l.split() for l in lines if not l.startswith("#")], float)
    atyp, xyz = read_conf(os.path.join(GOLD, "cdse22", "conf.par"))
    types = sorted(set(atyp), key=atyp.index)
    g = O.Grid(nx, ny, nz, d, d, d, xmin, ymin, zmin, 10.0)
    pot = O.local_pot(g, xyz, np.array([types.index(a) for a in atyp]), cdse_tables(types))
    ci = vals[:, 0].astype(int)  # cube order: x outer, y, z inner
    ix, rem = np.divmod(ci, ny * nz)
    iy, iz = np.divmod(rem, nz)
    got = pot[nx * (ny * iz + iy) + ix]
    # "%.5g" in the cube file
    assert np.allclose(got, vals[:, 1], rtol=1e-4, atol=6e-5)


def test_def_LS_eigenvalues():
    """L.S in the p shell has eigenvalues +1/2 (j = 3/2, x4) and -1 (j = 1/2, x2)."""
    ls = O.def_LS()
    ev = np.sort(np.linalg.eigvalsh(ls.T))
    assert np.allclose(ev, [-1, -1, 0.5, 0.5, 0.5, 0.5], atol=1e-14)


def test_eval_golden_files_parse():
    for sub in ("cdse22", "cspbi3"):
        ev = np.loadtxt(os.path.join(GOLD, sub, "eval.dat"))
        assert ev.shape[1] == 3 and np.all(np.diff(ev[:, 1]) >= -1e-12)


# ---------------------------------------------------------------- reference functions

def test_rng_matches_reference(ref):
    s_ref = ctypes.c_long(-987654)
    s = -987654
    for _ in range(3):
        vals, s = O.ran_fill(s, 1000)
        got = np.array([ref.ref_ran(ctypes.byref(s_ref)) for _ in range(1000)])
        assert np.array_equal(vals, got)
        assert s == s_ref.value
        s = -s - 17  # re-initialise both
        s_ref.value = s


def test_samp_points_match_reference(ref):
    for nc in (64, 257):
        re = np.empty(nc)
        im = np.empty(nc)
        fk = ref.ref_samp_points(nc, _p(re), _p(im))
        a, b, fk2 = O.samp_points(nc)
        assert np.array_equal(a, re) and np.array_equal(b, im) and fk == fk2


def test_newton_coeff_match_reference(ref, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)  # the reference writes zn.dat / coeff-*.dat / func.dat
    nc, m = 200, 4
    zn, _, _ = O.samp_points(nc)
    targets = np.array([-0.31, -0.25, -0.14, -0.07])
    vmin, de = -1.35, 14.2
    dt = O.filter_dt(nc, de)
    an_ref = np.empty(2 * m * nc)
    ref.ref_newton_coeff(nc, m, vmin, de, dt, _p(zn), _p(targets), _p(an_ref))
    an = O.newton_coeff(zn, targets, vmin, de, dt)
    assert np.array_equal(an.view(np.float64).reshape(-1), an_ref)


def test_def_LS_matches_reference(ref):
    ls = np.empty(72)
    ref.ref_def_LS(_p(ls))
    assert np.array_equal(O.def_LS().reshape(-1).view(np.float64), ls)


@pytest.mark.parametrize("so,nl,cplx", [(1, 1, 1), (1, 0, 1), (0, 1, 1), (0, 1, 0), (0, 0, 0)])
def test_potential_matches_reference(ref, so, nl, cplx):
    from tests.systems import tiny_cluster
    nspin = 2 if so else 1
    sysm = tiny_cluster(14, 15, 13, natoms=8, nspin=nspin, is_complex=bool(cplx), so=bool(so), nl=bool(nl))
    rng = np.random.default_rng(11)
    L = nspin * sysm.ngrid
    psi = rng.uniform(-1, 1, L) + 1j * (rng.uniform(-1, 1, L) if cplx else 0)
    base = rng.uniform(-1, 1, L) + 1j * rng.uniform(-1, 1, L)
    mine = base.copy()
    O.potential_add(mine, psi, sysm)
    theirs = base.copy()
    pr = sysm.proj
    pot2 = np.concatenate([sysm.pot, sysm.pot])  # the reference stores V twice
    ls = np.ascontiguousarray(sysm.LS).view(np.float64)
    if pr is None:
        pr = O.Projectors(np.zeros(1, np.int64), 1, np.zeros(1, np.int32), np.zeros(6), np.zeros(5), np.zeros(5),
                          np.zeros(5, np.int32))
    ref.ref_p_potential(_p(theirs.view(np.float64)), _p(psi.view(np.float64)), _p(pot2), _p(ls), sysm.ngrid, nspin,
                        cplx, so, nl, pr.nat if (so or nl) else 0, pr.npts, pr.nproj,
                        pr.nl.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                        pr.jxyz.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _p(pr.y1), _p(pr.proj), _p(pr.nlp),
                        pr.sgn.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), sysm.grid.dv)
    assert np.array_equal(mine, theirs)


def test_normalize_all_matches_reference(ref):
    rng = np.random.default_rng(3)
    ngrid, n = 1000, 4
    for cplx in (0, 1):
        a = rng.uniform(-1, 1, (n, ngrid * (1 + cplx)))
        b = a.copy()
        ref.ref_normalize_all(_p(b), n, ngrid, 1, cplx, 0.37)
        want = a / np.sqrt(np.sum(a ** 2, axis=1) * 0.37)[:, None]
        assert np.allclose(b, want, rtol=1e-14, atol=0)


# ------------------------------------------- the reference's FFT-dependent code

@pytest.mark.parametrize("shape", [(9, 8, 10), (6, 7, 5)])
def test_kinetic_matches_reference(ref_fft, shape):
    """kinetic() (filter_mpi/hamiltonian.c:62-99) run from the reference's own
    source against the oracle's numpy restatement, on the same ksqr."""
    nx, ny, nz = shape
    g = O.Grid(nx, ny, nz, 0.6, 0.6, 0.6, -nx * 0.3, -ny * 0.3, -nz * 0.3, 4.0)
    sysm = O.System(g, np.zeros(g.ngrid), nspin=1, is_complex=True)
    rng = np.random.default_rng(sum(shape))
    psi = rng.normal(size=g.ngrid) + 1j * rng.normal(size=g.ngrid)
    ksqr = np.ascontiguousarray(g.ksqr())
    theirs = np.empty(g.ngrid, np.complex128)
    ref_fft.ref_kinetic(_p(theirs.view(np.float64)), _p(psi.view(np.float64)), nx, ny, nz, _p(ksqr))
    mine = O.kinetic(psi, sysm)
    assert np.max(np.abs(mine - theirs)) < 1e-13 * np.max(np.abs(theirs))


def _angular_rows(ref_fft, states, g, start, stop, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    gx, gy, gz = (np.ascontiguousarray(a) for a in g.axes())
    dkx, dky, dkz = g.dk()
    buf = np.ascontiguousarray(states, np.float64)
    ref_fft.ref_angular(_p(buf), len(states), g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, _p(gx), _p(gy), _p(gz), dkx, dky, dkz,
                        start, stop)
    return np.loadtxt(tmp_path / "angular.dat", comments="#").reshape(-1, 9)


def test_angular_stats_match_reference(ref_fft, tmp_path, monkeypatch):
    """calc_angular_exp (filter_mpi/angular.c:4-165) run from the reference's
    own source against the oracle on the same spinors: state 0 to the printed
    digits ("%f"); for state 1 the reference reads its spin-up imaginary part
    from offset nspinngrid (angular.c:63, state 0's spin-down block) instead
    of its own, and the oracle reproduces that row when given the state so
    assembled -- the one quirk the library does not copy."""
    g = O.Grid(12, 11, 10, 0.7, 0.7, 0.7, -4.2, -3.5, -3.15, 4.0)
    n = g.ngrid
    gx, gy, gz = g.axes()
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    env = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 4.0).reshape(-1)
    rng = np.random.default_rng(21)
    states = []
    for _ in range(2):
        z = (rng.normal(size=2 * n) + 1j * rng.normal(size=2 * n)) * np.concatenate([env, env])
        states.append(z.view(np.float64))
    states = np.array(states)
    rows = _angular_rows(ref_fft, states, g, 0, 2, tmp_path, monkeypatch)
    assert np.array_equal(rows[:, 0], [0, 1])
    mine0 = O.filter_angular_stats(states[:1], g)[0]
    assert np.max(np.abs(rows[0, 1:] - mine0)) < 6e-7
    # state 1 as the reference reads it
    s0, s1 = states[0].view(np.complex128), states[1].view(np.complex128)
    quirk = s1.copy()
    quirk[:n] = s1[:n].real + 1j * s0[n:].imag
    mine1 = O.filter_angular_stats([quirk.view(np.float64)], g)[0]
    assert np.max(np.abs(rows[1, 1:] - mine1)) < 6e-7
    assert np.max(np.abs(rows[1, 1:] - O.filter_angular_stats(states[1:], g)[0])) > 1e-3


@pytest.mark.parametrize("so,nl,cplx", [(1, 1, 1), (0, 1, 0), (0, 0, 1)])
def test_hamiltonian_matches_reference(ref_fft, so, nl, cplx):
    """p_hamiltonian (filter_mpi/phamiltonian.c:10-60: kinetic FFT term, local
    potential, spin-orbit and nonlocal projectors) run from the reference's
    own source against the oracle's H psi."""
    from tests.systems import tiny_cluster
    nspin = 2 if so else 1
    sysm = tiny_cluster(12, 11, 13, natoms=6, nspin=nspin, is_complex=bool(cplx), so=bool(so), nl=bool(nl))
    rng = np.random.default_rng(17)
    L = nspin * sysm.ngrid
    psi = rng.uniform(-1, 1, L) + 1j * (rng.uniform(-1, 1, L) if cplx else 0)
    pot2 = np.concatenate([sysm.pot, sysm.pot])
    ls = np.ascontiguousarray(sysm.LS).view(np.float64)
    ksqr = np.ascontiguousarray(sysm.grid.ksqr())
    theirs = np.empty(L, np.complex128)
    g = sysm.grid
    ref_fft.ref_hamiltonian(_p(theirs.view(np.float64)), _p(psi.view(np.float64)), g.nx, g.ny, g.nz, nspin, cplx, so,
                            nl, _p(pot2), _p(ls), _p(ksqr), *_table_args(sysm, so, nl))
    mine = O.hamiltonian(psi, sysm)
    assert np.max(np.abs(mine - theirs)) < 1e-12 * np.max(np.abs(theirs))


def test_filter_cycle_matches_reference(ref_fft):
    """filter_cycle (filter_mpi/filter.c:187-371, with p_hnorm :375-410) of one
    spinor start with spin-orbit and nonlocal projectors, 24 Newton terms and
    3 energy targets, run from the reference's own source against the
    oracle's Newton recursion."""
    from tests.systems import tiny_cluster
    sysm = tiny_cluster(10, 11, 9, natoms=5, nspin=2, is_complex=True, so=True, nl=True)
    g = sysm.grid
    rng = np.random.default_rng(23)
    L = 2 * g.ngrid
    psi0 = rng.uniform(-1, 1, L) + 1j * rng.uniform(-1, 1, L)
    psi0 /= np.sqrt(np.sum(np.abs(psi0) ** 2) * g.dv)
    nc, m = 24, 3
    zn, _, _ = O.samp_points(nc)
    emin, emax = float(sysm.pot.min()) - 1.0, float(sysm.pot.max()) + g.ke_max + 2.0
    de = emax - emin
    an = O.newton_coeff(zn, np.array([emin + 0.2 * de, emin + 0.3 * de, emin + 0.4 * de]), emin, de,
                        O.filter_dt(nc, de))
    mine = O.filter_cycle(psi0, sysm, an, zn, emin, de)
    psi_rank = np.zeros(m * L, np.complex128)
    psi_rank[:L] = psi0
    pot2 = np.concatenate([sysm.pot, sysm.pot])
    ls = np.ascontiguousarray(sysm.LS).view(np.float64)
    ksqr = np.ascontiguousarray(g.ksqr())
    anc = np.ascontiguousarray(an, np.complex128)
    znc = np.ascontiguousarray(zn, np.float64)
    ref_fft.ref_filter_cycle(_p(psi_rank.view(np.float64)), g.nx, g.ny, g.nz, 2, 1, 1, 1, _p(pot2), _p(ls),
                             _p(ksqr), *_table_args(sysm, 1, 1), _p(anc.view(np.float64)), _p(znc), nc, m, emin, de)
    theirs = psi_rank.reshape(m, L)
    assert np.max(np.abs(mine - theirs)) < 1e-10 * np.max(np.abs(theirs))


def test_rayleigh_ritz_matches_reference(ref_fft, tmp_path, monkeypatch):
    """The reference's own mod_ortho + mod_diag + mod_sigma sequence
    (ortho_cplx with LAPACK's zgesvd, normalize_all, diag_H with zheev,
    normalize_all, calc_sigma_E; filter_mpi/ortho.c:93-185, Hmat.c:5-297,
    energy.c:383-539) against the oracle's ortho / diag / sigma_e on the same
    spinor states: the kept count, the Ritz values, sigma_E and every Ritz
    vector (up to its phase)."""
    from tests.systems import tiny_cluster
    lap = _numpy_lapack()
    if lap is None or not ref_fft.ref_set_lapack(lap.encode()):
        pytest.skip("numpy's ILP64 LAPACK is not available")
    monkeypatch.chdir(tmp_path)  # diag_H and calc_sigma_E write hmat-0.dat / eval_aux.dat
    sysm = tiny_cluster(10, 9, 11, natoms=5, nspin=2, is_complex=True, so=True, nl=True)
    g = sysm.grid
    L = 2 * g.ngrid
    rng = np.random.default_rng(31)
    n = 6
    base = rng.normal(size=(4, L)) + 1j * rng.normal(size=(4, L))
    # two of the six states lie in the span of the others: the rank cut keeps four
    psis = np.concatenate([base, (base[:2].T @ rng.normal(size=(2, 2))).T])
    assert psis.shape == (n, L)
    ov, s = O.ortho(psis, True, 1e-10, g.dv)
    e_mine, v_mine = O.diag(ov, sysm)
    _, sg_mine = O.sigma_e(v_mine, sysm)
    buf = np.ascontiguousarray(psis)
    ev, sg = np.zeros(n), np.zeros(n)
    pot2 = np.concatenate([sysm.pot, sysm.pot])
    ls = np.ascontiguousarray(sysm.LS).view(np.float64)
    ksqr = np.ascontiguousarray(g.ksqr())
    kept = ref_fft.ref_ritz(_p(buf.view(np.float64)), n, g.nx, g.ny, g.nz, 2, 1, 1, _p(pot2), _p(ls), _p(ksqr),
                            *_table_args(sysm, 1, 1), _p(ev), _p(sg))
    assert kept == len(e_mine) == 4
    print(f"\n[reference Rayleigh-Ritz] Ritz values {ev[:kept]}, max |dE| {np.max(np.abs(ev[:kept] - e_mine)):.1e}, "
          f"sigma {sg[:kept]}")
    assert np.allclose(ev[:kept], e_mine, rtol=0, atol=1e-11 * np.max(np.abs(e_mine)))
    assert np.allclose(sg[:kept], sg_mine, rtol=1e-7, atol=1e-9)
    theirs = buf[:kept]
    for a, b in zip(theirs, v_mine):
        assert abs(abs(np.vdot(a, b)) * g.dv - 1.0) < 1e-10


def test_energy_range_matches_reference(ref_fft, tmp_path, monkeypatch):
    """get_energy_range (filter_mpi/energy.c:169-379: imaginary-time descent to
    E_min, power iteration to E_max from init_psi's random states, then the
    inflation) run from the reference's own source against the oracle, spinor
    job with spin-orbit and nonlocal projectors."""
    from tests.systems import tiny_cluster
    monkeypatch.chdir(tmp_path)  # Emin-init.dat / Emax-init.dat
    sysm = tiny_cluster(9, 10, 8, natoms=4, nspin=2, is_complex=True, so=True, nl=True)
    g = sysm.grid
    pot2 = np.concatenate([sysm.pot, sysm.pot])
    ls = np.ascontiguousarray(sysm.LS).view(np.float64)
    ksqr = np.ascontiguousarray(g.ksqr())
    vmin, de = ctypes.c_double(), ctypes.c_double()
    ref_fft.ref_energy_range(g.nx, g.ny, g.nz, 2, 1, 1, _p(pot2), _p(ls), _p(ksqr), *_table_args(sysm, 1, 1),
                             ctypes.byref(vmin), ctypes.byref(de))
    mine_vmin, mine_de, _, _ = O.energy_range(sysm)
    print(f"\n[reference energy range] Vmin {vmin.value:.10f} dE {de.value:.10f}; oracle {mine_vmin:.10f} {mine_de:.10f}")
    assert abs(vmin.value - mine_vmin) < 1e-9 * abs(mine_vmin)
    assert abs(de.value - mine_de) < 1e-9 * mine_de


def _align(mine, ref):
    """mine with each row's sign chosen to match ref (eigenvector phase)"""
    s = np.sign(np.sum(mine * ref, axis=-1, keepdims=True))
    s[s == 0] = 1.0
    return mine * s


def test_projector_table_and_nl_bounds_match_reference(ref_fft, tmp_path, monkeypatch):
    """gen_SO_projectors (projectors.c:12-84) against the oracle's radial SO
    projectors (up to sign); then init_NL_projectors (init.c:848-1135) with the
    NL radial projectors made on the fly by gen_nlc_projectors
    (projectors.c:87-228; one atom with NL_par 0): point counts, grid indices,
    Y_1m, SO projectors, NL projectors (up to sign per atom and projector),
    signs, and the NL spectral bounds (init.c:1095-1130) against the oracle's
    table and bounds and the library's host fbse_nl_bounds"""
    import filterbse_gb300 as F
    lap = _numpy_lapack()
    if lap is None or not ref_fft.ref_set_lapack(lap.encode()):
        pytest.skip("numpy's ILP64 LAPACK is not available")
    monkeypatch.chdir(tmp_path)  # the reference's projector files
    LP, IP = ctypes.POINTER(ctypes.c_long), ctypes.POINTER(ctypes.c_int)
    ref_fft.ref_so_projectors.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_long, D]
    ref_fft.ref_nl_projectors.argtypes = ([ctypes.c_long] * 3 + [ctypes.c_double] * 3 + [D] * 3 + [ctypes.c_long] +
                                          [D] * 4 + [ctypes.c_double, ctypes.c_long, ctypes.c_long, LP, IP, D, D, D,
                                                     IP, D])
    g = O.Grid(18, 17, 16, 0.8, 0.8, 0.8, -6.8, -6.4, -6.0)
    rc2 = O.r_nlcut2(g.dx)
    so_ref = np.zeros((O.NPROJ, O.PROJ_LEN))
    ref_fft.ref_so_projectors(g.dx, rc2, O.NPROJ, _p(so_ref))
    so_me = O.so_radial(g.dx, np.sqrt(rc2))
    assert np.max(np.abs(_align(so_me, so_ref) - so_ref)) < 1e-9 * np.max(np.abs(so_ref))

    coords = np.array([[0.3, -0.2, 0.1], [-2.1, 1.7, 0.4], [2.4, 0.9, -1.8]])
    so_par = np.array([0.4, 0.0, 1.3])
    nl_par = np.array([[-0.35, 0.6], [0.0, 0.0], [0.5, -0.2]])
    tabs, sgns = zip(*(O.nl_radial(g.dx, np.sqrt(rc2), *p) for p in nl_par))
    me = O.nlc_table(g, coords, so_par, so_ref, np.array(tabs), np.concatenate(sgns))
    nat, npts, np_ = len(coords), me.npts, O.NPROJ
    nl = np.zeros(nat, np.int64)
    jx = np.zeros(nat * npts, np.int32)
    y1 = np.zeros(nat * npts * 6)
    pr = np.zeros(nat * npts * np_)
    nlp = np.zeros(nat * npts * np_)
    sgn = np.zeros(nat * np_, np.int32)
    lam = np.zeros(2)
    axes = [np.ascontiguousarray(a) for a in g.axes()]
    ref_fft.ref_nl_projectors(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, *[_p(a) for a in axes], nat,
                              _p(np.ascontiguousarray(coords)), _p(so_par), _p(np.ascontiguousarray(nl_par)),
                              _p(so_ref), rc2, np_, npts, _p(nl, LP), _p(jx, IP), _p(y1), _p(pr), _p(nlp),
                              _p(sgn, IP), _p(lam))
    assert np.array_equal(nl, me.nl) and nl.max() == npts
    assert np.array_equal(sgn, me.sgn)
    assert list(sgn[np_:2 * np_]) == [0] * np_  # NL_par 0: zero projectors, sign 0 (projectors.c:113-125)
    for a in range(nat):
        sl = slice(a * npts, a * npts + int(nl[a]))
        assert np.array_equal(jx[sl], me.jxyz[sl])
        assert np.max(np.abs(y1.reshape(-1, 6)[sl] - me.y1.reshape(-1, 6)[sl])) < 1e-15
        assert np.max(np.abs(pr.reshape(-1, np_)[sl] - me.proj.reshape(-1, np_)[sl])) < 1e-13
        r, m = nlp.reshape(-1, np_)[sl].T, me.nlp.reshape(-1, np_)[sl].T
        assert np.max(np.abs(_align(m, r) - r)) <= 1e-9 * max(1.0, np.max(np.abs(r)))
    lo, hi = O.nl_bounds(me, g.dv)
    assert lam[0] < 0.0 < lam[1]
    assert abs(lo - lam[0]) < 1e-9 * abs(lam[0]) and abs(hi - lam[1]) < 1e-9 * abs(lam[1])
    L = F.load()
    L.fbse_nl_bounds.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_int, LP, D, D, IP, ctypes.c_double, D, D]
    L.fbse_nl_bounds.restype = None
    hlo, hhi = ctypes.c_double(), ctypes.c_double()
    L.fbse_nl_bounds(nat, npts, np_, _p(nl, LP), _p(y1), _p(nlp), _p(sgn, IP), g.dv, ctypes.byref(hlo),
                     ctypes.byref(hhi))
    assert abs(hlo.value - lam[0]) <= 1e-14 * abs(lam[0]) and abs(hhi.value - lam[1]) <= 1e-14 * abs(lam[1])


@pytest.mark.parametrize("so,nl,lmin,lmax", [(0, 1, -0.7, 0.9), (1, 1, -0.7, 0.9), (0, 1, 0.0, 0.4),
                                             (0, 1, -0.3, 0.0), (1, 0, 0.0, 0.0), (0, 0, 0.0, 0.0)])
def test_approx_energy_range_matches_reference(ref_fft, so, nl, lmin, lmax):
    """get_energy_range's approxEnergyRange branch with the projector pads and
    the range inflation (energy.c:302-369) against the library's host
    fbse_energy_range_rule and the oracle; the rule's iterated branch (approx
    = 0) against the oracle's inflate_range"""
    import types
    import filterbse_gb300 as F
    ref_fft.ref_energy_range_approx.argtypes = [ctypes.c_int] * 2 + [ctypes.c_double] * 5 + [D, D]
    vmin, vmax, ke = -1.3, 0.9, 7.5
    e, de = ctypes.c_double(), ctypes.c_double()
    ref_fft.ref_energy_range_approx(so, nl, vmin, vmax, ke, lmin, lmax, ctypes.byref(e), ctypes.byref(de))
    L = F.load()
    L.fbse_energy_range_rule.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 5 + [D, D]
    L.fbse_energy_range_rule.restype = None
    lo, hi = ctypes.c_double(), ctypes.c_double()
    L.fbse_energy_range_rule(1, so, nl, vmin, vmax, ke, lmin, lmax, ctypes.byref(lo), ctypes.byref(hi))
    assert lo.value == e.value and abs((hi.value - lo.value) - de.value) <= 1e-15 * de.value
    sysm = types.SimpleNamespace(nlflag=bool(nl), so=bool(so), pot=np.array([vmin, vmax]))
    oe, oE = O.approx_energy_range(vmax, ke, bool(so), bool(nl), lmin, lmax)
    emin_i, de_i, _, _ = O.inflate_range(sysm, oe, oE, lmin)
    assert emin_i == e.value and abs(de_i - de.value) <= 1e-15 * de.value
    # the iterated branch: the extremes come in, only the inflation applies
    lo.value, hi.value = -0.91, 4.37
    L.fbse_energy_range_rule(0, so, nl, vmin, vmax, ke, lmin, lmax, ctypes.byref(lo), ctypes.byref(hi))
    emin_i, de_i, _, _ = O.inflate_range(sysm, -0.91, 4.37, lmin)
    assert lo.value == emin_i and abs((hi.value - lo.value) - de_i) <= 1e-15 * de_i


@pytest.mark.parametrize("nspin,cplx", [(1, False), (1, True), (2, True)])
def test_init_filter_states_match_reference(ref_fft, tmp_path, monkeypatch, nspin, cplx):
    """init_filter_states + init_psi (init.c:1138-1306) at one rank: every
    start bit for bit against the oracle (start j at state j * m of the
    reference's psi_rank), the seeds of seed-<rank>.dat and the advanced seed"""
    monkeypatch.chdir(tmp_path)
    ref_fft.ref_init_filter_states.argtypes = [D] + [ctypes.c_long] * 3 + [ctypes.c_int] * 2 + [ctypes.c_double] + \
        [ctypes.c_long] * 3
    ref_fft.ref_init_filter_states.restype = ctypes.c_long
    nx, ny, nz, dv = 9, 8, 7, 0.512
    n_filters, m = 3, 4
    stlen = (2 if cplx else 1) * nspin * nx * ny * nz
    rk = np.zeros(n_filters * m * stlen)
    end = ref_fft.ref_init_filter_states(_p(rk), nx, ny, nz, nspin, int(cplx), dv, n_filters, m, -4242)
    want, seeds, w_end = O.init_filter_states(-4242, n_filters, nx * ny * nz, nspin, cplx, dv)
    got = rk.reshape(n_filters, m, stlen)[:, 0, :]
    w = np.ascontiguousarray(want).view(np.float64) if cplx else np.ascontiguousarray(want.real)
    assert np.array_equal(got, w.reshape(n_filters, stlen))
    assert end == w_end
    rows = np.loadtxt(tmp_path / "seed-1.dat", skiprows=1, dtype=np.int64)
    assert np.array_equal(rows[:, 0], np.arange(n_filters * nspin))
    assert np.array_equal(rows[:, 1], np.asarray(seeds, np.int64).reshape(-1))


@pytest.mark.parametrize("m,n_vb,win", [(16, 10, (-0.31, -0.24, -0.15, -0.06)), (16, 8, (-0.50, -0.20, -0.167, -0.10)),
                                        (5, 1, (-0.4, -0.3, -0.1, 0.2)), (7, 6, (-1.0, -0.5, 0.0, 0.5))])
def test_ene_targets_match_reference(ref_fft, tmp_path, monkeypatch, m, n_vb, win):
    """set_ene_targets (init.c:401-478) with setTargets = 1 against the
    library's host fbse_ene_targets, bit for bit"""
    import filterbse_gb300 as F
    monkeypatch.chdir(tmp_path)
    ref_fft.ref_ene_targets.argtypes = [ctypes.c_long] * 2 + [ctypes.c_double] * 4 + [D]
    L = F.load()
    L.fbse_ene_targets.argtypes = [ctypes.c_long] * 2 + [ctypes.c_double] * 4 + [D]
    L.fbse_ene_targets.restype = None
    ref, mine = np.zeros(m), np.zeros(m)
    ref_fft.ref_ene_targets(m, n_vb, *win, _p(ref))
    L.fbse_ene_targets(m, n_vb, *win, _p(mine))
    assert np.array_equal(ref, mine)
    assert ref[n_vb - 1] == win[1] and ref[n_vb] == win[2]
