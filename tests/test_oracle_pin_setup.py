"""Pins the setup chain that the drop-in filter runs before the hot path
against the reference's own code (oracle/_ref/libfbse_ref_fft.so, CPU):
read_conf, init_grid_params, build_grid_ksqr and build_local_pot (with its
read_pot), on the example configurations and pseudopotential files, against
the library's host conf.par reader, grid rule and table reader and the
oracle's k^2 grid and local potential, at full precision."""
import ctypes
import os
import shutil

import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import GOLD
from tests.test_dropin import FilterParams
from tests.test_oracle_pin import REF_FFT_SO

D = ctypes.POINTER(ctypes.c_double)
LP = ctypes.POINTER(ctypes.c_long)
IP = ctypes.POINTER(ctypes.c_int)


def _p(a, t=D):
    return a.ctypes.data_as(t)


@pytest.fixture(scope="module")
def rs():
    if not os.path.exists(REF_FFT_SO):
        pytest.skip("oracle/_ref not built (the reference tree is not mounted here)")
    L = ctypes.CDLL(REF_FFT_SO)
    L.ref_setup.argtypes = ([ctypes.c_double, LP, ctypes.c_double, ctypes.c_int, ctypes.c_int] + [ctypes.c_long] * 3 +
                            [LP, LP, LP, D, D, LP, D, D, D, D, D, D, D, LP])
    L.ref_setup.restype = ctypes.c_int
    return L


@pytest.fixture(scope="module")
def host():
    import filterbse_gb300 as F
    L = F.load()
    L.fbse_read_filter_params.argtypes = [ctypes.c_char_p, ctypes.POINTER(FilterParams), ctypes.c_char_p,
                                          ctypes.c_size_t]
    L.fbse_read_conf.argtypes = [ctypes.c_char_p, LP, ctypes.POINTER(D), ctypes.POINTER(IP),
                                 ctypes.POINTER(ctypes.c_char * 8), IP, ctypes.c_char_p, ctypes.c_size_t]
    L.fbse_grid_rule.argtypes = [D, ctypes.c_long, ctypes.c_double, ctypes.c_long, ctypes.c_int, LP, D]
    L.fbse_grid_rule.restype = None
    L.fbse_grid_axis.argtypes = [ctypes.c_long, ctypes.c_double, ctypes.c_double, D]
    L.fbse_grid_axis.restype = None
    L.fbse_read_table.argtypes = [ctypes.c_char_p, ctypes.POINTER(D), ctypes.POINTER(D)]
    L.fbse_read_table.restype = ctypes.c_long
    L.fbse_is_ligand.argtypes = [ctypes.c_char_p]
    L.fbse_read_so_params.argtypes = [ctypes.c_char_p, D, D, ctypes.c_char_p, ctypes.c_size_t]
    return L


@pytest.mark.parametrize("name", ["cdse22", "cspbi3"])
def test_setup_chain_matches_reference(rs, host, tmp_path, monkeypatch, name):
    """read_conf (read.c:998-1172) with centerConf, init_grid_params
    (init.c:5-256), build_grid_ksqr (init.c:259-398) and build_local_pot
    (init.c:481-703) with read_pot (read.c:1175-1800) on an example's
    conf.par and pot<Atm>.par: atoms, type indices and centred coordinates,
    grid counts and origins, the axes, the SO / NL parameters of SO_<Atm>.par
    and the NL sphere size exactly; ksqr and the local potential to 1e-14 of
    their largest magnitude"""
    src = os.path.join(GOLD, name)
    for f in os.listdir(src):
        if f == "conf.par" or (f.startswith(("pot", "SO_")) and f.endswith(".par")):
            shutil.copy(os.path.join(src, f), tmp_path / f)
    monkeypatch.chdir(tmp_path)
    prm = FilterParams()
    err = ctypes.create_string_buffer(512)
    assert host.fbse_read_filter_params(os.path.join(src, "input.par").encode(), ctypes.byref(prm), err, 512) == 0
    so, nl = int(prm.so), int(prm.nl)

    cap_atoms, cap_axis, cap_grid = 4096, 512, 8_000_000
    natoms = ctypes.c_long()
    zval = np.zeros(cap_atoms, np.int64)
    tidx = np.zeros(cap_atoms, np.int64)
    xyz = np.zeros(3 * cap_atoms)
    sonl = np.zeros(3 * cap_atoms)
    n = np.zeros(3, np.int64)
    lo = np.zeros(3)
    axes = [np.zeros(cap_axis) for _ in range(3)]
    ksqr = np.zeros(cap_grid)
    pot = np.zeros(cap_grid)
    vr = np.zeros(2)
    nlinfo = np.zeros(2, np.int64)
    n_in = np.array([prm.nx, prm.ny, prm.nz], np.int64)
    rc = rs.ref_setup(prm.dx, _p(n_in, LP), prm.ke_max, so, nl, cap_atoms, cap_axis, cap_grid, ctypes.byref(natoms),
                      _p(zval, LP), _p(tidx, LP), _p(xyz), _p(sonl), _p(n, LP), _p(lo), *[_p(a) for a in axes], _p(ksqr),
                      _p(pot), _p(vr), _p(nlinfo, LP))
    assert rc == 0
    na = natoms.value

    # the library's host reader: same atoms, first-appearance type order, centred coordinates
    hn = ctypes.c_long()
    hx, ht = D(), IP()
    names = (ctypes.c_char * 8 * 32)()
    nt = ctypes.c_int()
    assert host.fbse_read_conf(b"conf.par", ctypes.byref(hn), ctypes.byref(hx), ctypes.byref(ht), names,
                               ctypes.byref(nt), err, 512) == 0, err.value
    assert hn.value == na
    hxyz = np.ctypeslib.as_array(hx, (3 * na,)).copy()
    htyp = np.ctypeslib.as_array(ht, (na,)).copy()
    assert np.array_equal(hxyz, xyz[:3 * na])
    assert np.array_equal(htyp, tidx[:na])

    # grid rule and axes
    g_n, g_lo = [], []
    for ax in range(3):
        nn, x0 = ctypes.c_long(), ctypes.c_double()
        host.fbse_grid_rule(_p(hxyz), na, prm.dx, int(n_in[ax]), ax, ctypes.byref(nn), ctypes.byref(x0))
        g_n.append(nn.value)
        g_lo.append(x0.value)
        hax = np.zeros(nn.value)
        host.fbse_grid_axis(nn.value, x0.value, prm.dx, _p(hax))
        assert np.array_equal(hax, axes[ax][:nn.value])
    assert g_n == list(n) and g_lo == list(lo)
    g = O.Grid(int(n[0]), int(n[1]), int(n[2]), prm.dx, prm.dx, prm.dx, lo[0], lo[1], lo[2], prm.ke_max)
    N = g.ngrid
    assert np.max(np.abs(g.ksqr() - ksqr[:N])) <= 1e-14 * np.max(ksqr[:N])

    # local potential from the host-read tables, per type in first-appearance order
    tables = []
    for k in range(nt.value):
        r, v = D(), D()
        m = host.fbse_read_table(f"pot{names[k].value.decode()}.par".encode(), ctypes.byref(r), ctypes.byref(v))
        assert m > 1
        tables.append((np.ctypeslib.as_array(r, (m,)).copy(), np.ctypeslib.as_array(v, (m,)).copy()))
    mine = O.local_pot(g, hxyz.reshape(-1, 3), htyp, tables)
    ref = pot[:N]
    print(f"\n[{name}] grid {tuple(n)}, {na} atoms, V in [{vr[0]:.6f}, {vr[1]:.6f}], "
          f"max |dV| {np.max(np.abs(mine - ref)):.2e}")
    assert np.max(np.abs(mine - ref)) <= 1e-14 * np.max(np.abs(ref))
    assert (vr[0], vr[1]) == (ref.min(), ref.max())

    # SO_par / NL_par per atom: the host reader per type, zero on ligands
    if so or nl:
        for a in range(na):
            t = names[htyp[a]].value
            if host.fbse_is_ligand(t):
                assert not np.any(sonl[3 * a:3 * a + 3])
                continue
            sp, lam = ctypes.c_double(), np.zeros(2)
            assert host.fbse_read_so_params(t, ctypes.byref(sp), _p(lam), err, 512) == 0, err.value
            assert (sp.value, lam[0], lam[1]) == tuple(sonl[3 * a:3 * a + 3])

    # the NL sphere size (build_grid_ksqr counts the points within R_NLcut of
    # the first n_NL_atoms atoms): the oracle table's row stride
    if so or nl:
        assert nlinfo[0] == na  # no ligands in this configuration
        rc2 = O.r_nlcut2(prm.dx)
        gx, gy, gz = g.axes()
        cnt = max(int(np.count_nonzero((gx[None, None, :] - c[0]) ** 2 + (gy[None, :, None] - c[1]) ** 2 +
                                       (gz[:, None, None] - c[2]) ** 2 < rc2)) for c in hxyz.reshape(-1, 3))
        assert nlinfo[1] == cnt


@pytest.mark.parametrize("name", ["cdse22", "cspbi3"])
def test_output_writers_match_reference(rs, host, tmp_path, monkeypatch, name):
    """write_cube_file, write_eval_dat and write_psi_dat (write.c:65-296)
    against the library's host fbse_write_cube / fbse_write_eval /
    fbse_write_psi, byte for byte: the cube of an example's atoms (read back
    from the conf.dat that read_conf writes) on its grid, an eval.dat and a
    psi.dat"""
    src = os.path.join(GOLD, name)
    shutil.copy(os.path.join(src, "conf.par"), tmp_path / "conf.par")
    monkeypatch.chdir(tmp_path)
    err = ctypes.create_string_buffer(512)
    hn = ctypes.c_long()
    hx, ht = D(), IP()
    names = (ctypes.c_char * 8 * 32)()
    nt = ctypes.c_int()
    assert host.fbse_read_conf(b"conf.par", ctypes.byref(hn), ctypes.byref(hx), ctypes.byref(ht), names,
                               ctypes.byref(nt), err, 512) == 0
    na = hn.value
    xyz = np.ctypeslib.as_array(hx, (3 * na,)).copy()
    typ = np.ctypeslib.as_array(ht, (na,)).copy()
    # conf.dat as read_conf writes it (read.c:1150-1156), which write_cube_file reads
    with open("conf.dat", "w") as f:
        f.write(f"{na}\n")
        for a in range(na):
            f.write("%3s % .16g % .16g % .16g\n" % (names[typ[a]].value.decode(), *xyz[3 * a:3 * a + 3]))
    rng = np.random.default_rng(3)
    nx, ny, nz, d = 13, 11, 9, 0.7
    lo = (-4.55, -3.85, -3.15)
    rho = np.ascontiguousarray(rng.standard_normal(nx * ny * nz) * np.logspace(-9, 2, nx * ny * nz))
    ev = np.ascontiguousarray(np.sort(rng.uniform(-0.5, 0.1, 40)))
    sg = np.ascontiguousarray(10.0 ** rng.uniform(-9, -2, 40))
    psi = np.ascontiguousarray(rng.standard_normal(3 * 2 * 2 * nx * ny * nz))
    rs.ref_write_outputs.argtypes = [D] + [ctypes.c_long] * 3 + [ctypes.c_double] * 6 + [D, D, ctypes.c_long, D,
                                                                                          ctypes.c_long]
    rs.ref_write_outputs(_p(rho), nx, ny, nz, d, d, d, *lo, _p(ev), _p(sg), len(ev), _p(psi), psi.size)
    sym8 = np.zeros((na, 8), np.uint8)
    for a in range(na):
        b = names[typ[a]].value
        sym8[a, :len(b)] = np.frombuffer(b, np.uint8)
    host.fbse_write_cube.argtypes = [ctypes.c_char_p, D] + [ctypes.c_long] * 3 + [ctypes.c_double] * 6 + \
        [ctypes.c_long, ctypes.c_char_p, D]
    host.fbse_write_eval.argtypes = [ctypes.c_char_p, D, D, ctypes.c_long]
    host.fbse_write_psi.argtypes = [ctypes.c_char_p, D, ctypes.c_long]
    assert host.fbse_write_cube(b"mine.cube", _p(rho), nx, ny, nz, d, d, d, *lo, na, sym8.tobytes(), _p(xyz)) == 0
    assert host.fbse_write_eval(b"mine_eval.dat", _p(ev), _p(sg), len(ev)) == 0
    assert host.fbse_write_psi(b"mine_psi.dat", _p(psi), psi.size) == 0
    for mine, ref in (("mine.cube", "ref.cube"), ("mine_eval.dat", "ref_eval.dat"), ("mine_psi.dat", "ref_psi.dat")):
        assert open(mine, "rb").read() == open(ref, "rb").read(), mine


_SYNTH = """nx = 48
ny = 44
nz = 40
dx = 0.7
dy = 0.75
dz = 0.8
mStatesPerFilter = 12
nFilterCycles = 3
nCheby = 512
VBmin = -0.42
VBmax = -0.21
CBmin = -0.16
CBmax = -0.02
KEmax = 12.5
fermiEnergy = -0.185
sigmaECut = 0.0005
setTargets = 1 7 5
setSeed = 1 -12345
spinOrbit = 1
NonLocal = 1
getAllStates = 1
approxEnergyRange = 1
printPsiFilt = 0
printPsiDiag = 1
calcFilterOnly = 0
restartFromOrtho = 1 36
printCubes = 1 6
readCoeffs = 1
inputPsiFilt = 1 4 40
calcSpinAngStat = 1
"""


@pytest.mark.parametrize("name", ["cdse22", "cspbi3", "synthetic"])
def test_input_parser_matches_reference(rs, host, tmp_path, monkeypatch, name):
    """read_input (read.c:5-995) against the library's host
    fbse_read_filter_params on the examples' input.par and on one that sets
    every key the drop-in reads, multi-value keys included: grid, windows,
    targets, seed, projector switches (spinors and complex storage follow
    spinOrbit), output and restart switches with their counts"""
    if name == "synthetic":
        (tmp_path / "input.par").write_text(_SYNTH)
        shutil.copy(os.path.join(GOLD, "cspbi3", "conf.par"), tmp_path / "conf.par")
    else:
        for f in ("input.par", "conf.par"):
            shutil.copy(os.path.join(GOLD, name, f), tmp_path / f)
    monkeypatch.chdir(tmp_path)
    rs.ref_read_input.argtypes = [D, LP]
    d = np.zeros(10)
    lv = np.zeros(31, np.int64)
    rs.ref_read_input(_p(d), _p(lv, LP))
    p = FilterParams()
    err = ctypes.create_string_buffer(512)
    assert host.fbse_read_filter_params(b"input.par", ctypes.byref(p), err, 512) == 0, err.value
    mine_d = [p.dx, p.dy, p.dz, p.vbmin, p.vbmax, p.cbmin, p.cbmax, p.ke_max, p.fermi_e, p.sigma_e_cut]
    assert mine_d == list(d)
    keys = ["nx", "ny", "nz", "m_states_per_filter", "n_filter_cycles", "ncheby", "set_targets", "n_targets_vb",
            "n_targets_cb", "set_seed", "seed", "use_spinors", "so", "nl", "get_all_states", "approx_energy_range",
            "print_psi_filt", "print_psi_diag", "calc_filter_only", "restart_from_ortho", "restart_from_sigma",
            "n_states_for_ortho", "n_states_for_sigma", "print_cubes", "ncubes", "read_coeffs", "input_psi_filt",
            "init_psi_start", "init_psi_end", "calc_spin_ang_stat"]
    ref = dict(zip(keys + ["is_complex"], (int(v) for v in lv)))
    if not ref["set_targets"]:
        # read_input leaves the counts unset; the host holds set_ene_targets' half / half split
        for k in ("n_targets_vb", "n_targets_cb"):
            ref.pop(k)
    mine = {k: int(getattr(p, k)) for k in keys if k in ref}
    assert mine == {k: v for k, v in ref.items() if k != "is_complex"}
    assert ref["is_complex"] == ref["use_spinors"]  # complex storage follows the spinors (read.c:916-920)


@pytest.mark.parametrize("name", ["cdse22", "cspbi3"])
def test_output_dat_matches_reference(rs, host, tmp_path, monkeypatch, name):
    """save_output (save.c:446-503) after read_conf / init_grid_params /
    build_grid_ksqr against the library's host fbse_write_output on the same
    job: every byte after the random tag of the first line (sizes, the types'
    atom ids, switches, centred atoms, the grid metadata, axes, eigenvalues,
    variances and states)"""
    src = os.path.join(GOLD, name)
    shutil.copy(os.path.join(src, "conf.par"), tmp_path / "conf.par")
    monkeypatch.chdir(tmp_path)
    prm = FilterParams()
    err = ctypes.create_string_buffer(512)
    assert host.fbse_read_filter_params(os.path.join(src, "input.par").encode(), ctypes.byref(prm), err, 512) == 0
    so, nl = int(prm.so), int(prm.nl)
    nspin, cplx = (2, 1) if so else (1, 0)
    hn = ctypes.c_long()
    hx, ht = D(), IP()
    names = (ctypes.c_char * 8 * 32)()
    nt = ctypes.c_int()
    assert host.fbse_read_conf(b"conf.par", ctypes.byref(hn), ctypes.byref(hx), ctypes.byref(ht), names,
                               ctypes.byref(nt), err, 512) == 0
    na = hn.value
    xyz = np.ctypeslib.as_array(hx, (3 * na,)).copy()
    n3, lo, axes = [], [], []
    for ax, nin in enumerate((prm.nx, prm.ny, prm.nz)):
        nn, x0 = ctypes.c_long(), ctypes.c_double()
        host.fbse_grid_rule(_p(xyz), na, prm.dx, nin, ax, ctypes.byref(nn), ctypes.byref(x0))
        a = np.zeros(nn.value)
        host.fbse_grid_axis(nn.value, x0.value, prm.dx, _p(a))
        n3.append(nn.value)
        lo.append(x0.value)
        axes.append(a)
    ngrid = n3[0] * n3[1] * n3[2]
    rng = np.random.default_rng(11)
    n = 3
    ev = np.ascontiguousarray(np.sort(rng.uniform(-0.4, 0.0, n)))
    sg = np.ascontiguousarray(10.0 ** rng.uniform(-8, -3, n))
    psi = np.ascontiguousarray(rng.standard_normal(n * (cplx + 1) * nspin * ngrid))
    rs.ref_save_output.argtypes = [ctypes.c_double, LP, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_long, D, D, D]
    n_in = np.array([prm.nx, prm.ny, prm.nz], np.int64)
    assert rs.ref_save_output(prm.dx, _p(n_in, LP), prm.ke_max, prm.fermi_e, so, nl, n, _p(ev.copy()), _p(sg.copy()),
                              _p(psi)) == 0
    host.fbse_write_output.argtypes = ([ctypes.c_char_p, ctypes.c_long, ctypes.c_long, D, ctypes.c_int,
                                        ctypes.c_char_p] + [ctypes.c_long] * 3 + [ctypes.c_double] * 3 + [D] * 3 +
                                       [ctypes.c_double] * 5 + [ctypes.c_int] * 5 + [ctypes.c_long, D, D, D])
    labels = b"".join(names[k].value.ljust(8, b"\0") for k in range(nt.value))
    assert host.fbse_write_output(b"mine_output.dat", 0, na, _p(xyz), nt.value, labels, *n3, prm.dx, prm.dx, prm.dx,
                                  *[_p(a) for a in axes], *lo, prm.ke_max, prm.fermi_e, so, nl, so, nspin, cplx, n,
                                  _p(ev), _p(sg), _p(psi)) == 0
    ref = open("ref_output.dat", "rb").read()
    mine = open("mine_output.dat", "rb").read()
    assert mine.split(b"\n", 1)[1] == ref.split(b"\n", 1)[1]
