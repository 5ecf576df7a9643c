"""Host logic of the drop-in executables, on the CPU: input.par / conf.par
parsing, the grid rule, the radial projectors against the oracle, and the
executables' refusal to run without a GPU (the projector table is built on
the GPU: tests/test_setup_gpu.py)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import GOLD, read_conf

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "filterbse_gb300", "bin")
D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)
Lp = ctypes.POINTER(ctypes.c_long)


class FilterParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_long), ("ny", ctypes.c_long), ("nz", ctypes.c_long), ("dx", ctypes.c_double),
                ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("m_states_per_filter", ctypes.c_long),
                ("n_filter_cycles", ctypes.c_long), ("ncheby", ctypes.c_long), ("vbmin", ctypes.c_double),
                ("vbmax", ctypes.c_double), ("cbmin", ctypes.c_double), ("cbmax", ctypes.c_double),
                ("ke_max", ctypes.c_double), ("fermi_e", ctypes.c_double), ("sigma_e_cut", ctypes.c_double),
                ("set_targets", ctypes.c_int), ("n_targets_vb", ctypes.c_long), ("n_targets_cb", ctypes.c_long),
                ("set_seed", ctypes.c_int), ("seed", ctypes.c_long), ("use_spinors", ctypes.c_int),
                ("so", ctypes.c_int), ("nl", ctypes.c_int), ("get_all_states", ctypes.c_int),
                ("approx_energy_range", ctypes.c_int), ("precision", ctypes.c_int),
                ("print_psi_filt", ctypes.c_int), ("print_psi_diag", ctypes.c_int),
                ("calc_filter_only", ctypes.c_int), ("restart_from_ortho", ctypes.c_int),
                ("restart_from_sigma", ctypes.c_int), ("n_states_for_ortho", ctypes.c_long),
                ("n_states_for_sigma", ctypes.c_long), ("print_cubes", ctypes.c_int), ("ncubes", ctypes.c_long),
                ("read_coeffs", ctypes.c_int), ("input_psi_filt", ctypes.c_int), ("init_psi_start", ctypes.c_long),
                ("init_psi_end", ctypes.c_long), ("calc_spin_ang_stat", ctypes.c_int)]


@pytest.fixture(scope="module")
def lib():
    import filterbse_gb300 as F
    L = F.load()
    L.fbse_read_filter_params.argtypes = [ctypes.c_char_p, ctypes.POINTER(FilterParams), ctypes.c_char_p,
                                          ctypes.c_size_t]
    L.fbse_grid_rule.argtypes = [D, ctypes.c_long, ctypes.c_double, ctypes.c_long, ctypes.c_int, Lp, D]
    L.fbse_grid_rule.restype = None
    L.fbse_radial_projectors.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_int, D, I]
    return L


def test_read_filter_params_example(lib):
    p = FilterParams()
    err = ctypes.create_string_buffer(512)
    rc = lib.fbse_read_filter_params(os.path.join(GOLD, "cspbi3", "input.par").encode(), ctypes.byref(p), err, 512)
    assert rc == 0, err.value
    assert (p.nx, p.ny, p.nz, p.dx, p.dz) == (44, 44, 44, 0.5, 0.5)
    assert (p.m_states_per_filter, p.n_filter_cycles, p.ncheby) == (16, 16, 2048)
    assert (p.n_targets_vb, p.n_targets_cb, p.set_targets) == (10, 6, 1)
    assert p.so == 1 and p.nl == 1 and p.use_spinors == 1 and p.get_all_states == 1
    assert p.fermi_e == -0.19 and p.vbmin == -0.5 and p.cbmax == -0.1 and p.ke_max == 20.0
    # printPsiFilt is on unless input.par says otherwise (read.c:34)
    assert p.print_psi_filt == 1 and p.restart_from_ortho == 0 and p.restart_from_sigma == 0


def test_read_filter_params_restarts(lib, tmp_path):
    base = "dGrid = 0.5\nmStatesPerFilter = 4\nnFilterCycles = 2\nnCheby = 16\n"
    err = ctypes.create_string_buffer(512)
    p = FilterParams()
    (tmp_path / "a.par").write_text(base + "restartFromOrtho = 1 8\nprintPsiFilt = 0\nprintPsiDiag = 1\n"
                                    "calcFilterOnly = 0\nsaveCheckpoints = 1\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "a.par").encode(), ctypes.byref(p), err, 512) == 0, err.value
    assert (p.restart_from_ortho, p.n_states_for_ortho, p.print_psi_filt, p.print_psi_diag) == (1, 8, 0, 1)
    (tmp_path / "e.par").write_text(base + "readCoeffs = 1\nprintCubes = 1 2\ncalcSpinAngStat = 1\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "e.par").encode(), ctypes.byref(p), err, 512) == 0, err.value
    assert (p.read_coeffs, p.print_cubes, p.ncubes, p.calc_spin_ang_stat) == (1, 1, 2, 1)
    (tmp_path / "f.par").write_text(base + "inputPsiFilt = 1 4 20\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "f.par").encode(), ctypes.byref(p), err, 512) == 0, err.value
    assert (p.input_psi_filt, p.init_psi_start, p.init_psi_end) == (1, 4, 20)
    (tmp_path / "b.par").write_text(base + "restartFromSigma = 1 12\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "b.par").encode(), ctypes.byref(p), err, 512) == 0, err.value
    assert (p.restart_from_sigma, p.n_states_for_sigma) == (1, 12)
    # the state count must follow (read.c:770-773)
    (tmp_path / "c.par").write_text(base + "restartFromOrtho = 1\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "c.par").encode(), ctypes.byref(p), err, 512) != 0
    # checkpoint_<id>.dat restarts are refused with the key named
    (tmp_path / "d.par").write_text(base + "restartFromCheckpoint = 2\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "d.par").encode(), ctypes.byref(p), err, 512) != 0
    assert b"restartFromCheckpoint" in err.value


def test_read_filter_params_cdse_example(lib):
    # the 2.2 nm CdSe example's keys (crystalStructure, outmostMaterial,
    # useStrain = 0, printCubes with its second value) are accepted
    p = FilterParams()
    err = ctypes.create_string_buffer(512)
    rc = lib.fbse_read_filter_params(os.path.join(GOLD, "cdse22", "input.par").encode(), ctypes.byref(p), err, 512)
    assert rc == 0, err.value
    assert (p.dx, p.so, p.use_spinors, p.m_states_per_filter) == (0.8, 0, 0, 16)


def test_read_filter_params_rejects(lib, tmp_path):
    err = ctypes.create_string_buffer(512)
    p = FilterParams()
    (tmp_path / "a.par").write_text("dGrid = 0.5\nmStatesPerFilter = 4\nnFilterCycles = 2\nnCheby = 16\nperiodic = 1\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "a.par").encode(), ctypes.byref(p), err, 512) != 0
    assert b"periodic" in err.value
    (tmp_path / "b.par").write_text("dGrid = 0.5\nmStatesPerFilter = 4\nnFilterCycles = 2\nnCheby = 16\nbogusKey = 3\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "b.par").encode(), ctypes.byref(p), err, 512) != 0
    assert b"bogusKey" in err.value
    (tmp_path / "c.par").write_text("dGrid = 0.5\nmStatesPerFilter = 4\nnFilterCycles = 2\nnCheby = 16\n"
                                    "setTargets = 1 3 3\n")
    assert lib.fbse_read_filter_params(str(tmp_path / "c.par").encode(), ctypes.byref(p), err, 512) != 0


@pytest.mark.parametrize("name,n_in", [("cspbi3", 44), ("cdse22", 0)])
def test_grid_rule_matches_oracle(lib, name, n_in):
    _, xyz = read_conf(os.path.join(GOLD, name, "conf.par"))
    xyz = np.ascontiguousarray(xyz)
    ref = O.reference_grid(xyz, 0.8 if name == "cdse22" else 0.5, (n_in,) * 3)
    for ax, (rn, rlo) in enumerate(((ref.nx, ref.xmin), (ref.ny, ref.ymin), (ref.nz, ref.zmin))):
        n = ctypes.c_long()
        lo = ctypes.c_double()
        lib.fbse_grid_rule(xyz.reshape(-1).ctypes.data_as(D), len(xyz), 0.8 if name == "cdse22" else 0.5, n_in, ax,
                           ctypes.byref(n), ctypes.byref(lo))
        assert n.value == rn and lo.value == rlo


@pytest.mark.parametrize("kind,lam", [(0, (0.0, 0.0)), (1, (0.5, -0.3)), (1, (-0.8, 0.2))])
def test_radial_projectors_match_oracle(lib, kind, lam):
    dx = 0.5
    rc = np.sqrt(O.r_nlcut2(dx))
    out = np.empty(5 * 1024)
    sg = np.zeros(5, np.int32)
    assert lib.fbse_radial_projectors(dx, rc, kind, lam[0], lam[1], 5, out.ctypes.data_as(D), sg.ctypes.data_as(I)) == 0
    if kind == 0:
        ref, rs = O.so_radial(dx, rc), np.ones(5, np.int32)
    else:
        ref, rs = O.nl_radial(dx, rc, *lam)
    o = out.reshape(5, 1024)
    for p in range(5):
        s = np.sign(np.dot(o[p], ref[p]))  # eigenvector signs are free; the projectors enter squared
        assert np.max(np.abs(s * o[p] - ref[p])) < 1e-10 * np.max(np.abs(ref[p]))
    if kind == 1:
        assert np.array_equal(sg, rs)


def _cube_text(rho, n, d, lo, atoms):
    """write_cube_file's layout (filter_mpi/write.c:65-139), restated."""
    nx, ny, nz = n
    out = ["CUBE FILE", "OUTER LOOP: X, MIDDLE LOOP: Y, INNER LOOP: Z",
           "%5li%12.6f%12.6f%12.6f" % (len(atoms), *lo), "%5li%12.6f%12.6f%12.6f" % (nx, d[0], 0.0, 0.0),
           "%5li%12.6f%12.6f%12.6f" % (ny, 0.0, d[1], 0.0), "%5li%12.6f%12.6f%12.6f" % (nz, 0.0, 0.0, d[2])]
    out += ["%5li%12.6f%12.6f%12.6f%12.6f" % (z, 0.0, *xyz) for z, xyz in atoms]
    body = []
    r = rho.reshape(nz, ny, nx)
    for ix in range(nx):
        for iy in range(ny):
            line = ""
            for iz in range(nz):
                line += "%.5g " % r[iz, iy, ix]
                if iz % 6 == 5:
                    line += "\n"
            body.append(line + "\n")
    return "\n".join(out) + "\n" + "".join(body)


def test_cube_file_matches_reference_layout(lib, tmp_path):
    lib.fbse_write_cube.argtypes = ([ctypes.c_char_p, D] + [ctypes.c_long] * 3 + [ctypes.c_double] * 6 +
                                    [ctypes.c_long, ctypes.c_char_p, D])
    rng = np.random.default_rng(3)
    n, d, lo = (5, 4, 13), (0.5, 0.6, 0.7), (-1.25, -1.2, -4.55)
    rho = rng.normal(size=n[0] * n[1] * n[2]) * 1e-3
    syms = ["Cd", "Se", "P1", "I", "Cs"]
    xyz = rng.uniform(-2, 2, (5, 3))
    sym8 = b"".join(s.encode().ljust(8, b"\0") for s in syms)
    path = tmp_path / "x.cube"
    assert lib.fbse_write_cube(str(path).encode(), rho.ctypes.data_as(D), *n, *d, *lo, 5, sym8,
                               np.ascontiguousarray(xyz).ctypes.data_as(D)) == 0
    want = _cube_text(rho, n, d, lo, list(zip([48, 34, 84, 53, 55], xyz)))
    assert path.read_text() == want
    # an atom the reference's table does not know is an error
    assert lib.fbse_write_cube(str(path).encode(), rho.ctypes.data_as(D), *n, *d, *lo, 1, b"Xx\0\0\0\0\0\0",
                               np.ascontiguousarray(xyz).ctypes.data_as(D)) != 0


def test_executables_fail_loudly_without_gpu(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    exe = os.path.join(BIN, "fbse_filter")
    assert os.path.exists(exe), "build() makes the drop-in executables"
    for f in ("input.par", "conf.par", "potCs.par", "potPb.par", "potI.par", "SO_Cs.par", "SO_Pb.par", "SO_I.par"):
        shutil.copy(os.path.join(GOLD, "cspbi3", f), tmp_path / f)
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "ERROR" in r.stderr
    assert not (tmp_path / "eval.dat").exists()


def test_xton_ang_stats_match_oracle(lib):
    """calc_xton_spin_mtrx / calc_xton_ang_mom_mtrx on random Hermitian pair
    matrices and a random unitary coefficient matrix (host code)."""
    rng = np.random.default_rng(12)
    nh, ne = 3, 4
    nx, n = nh * ne, nh * nh + ne * ne

    def herm_blocks(k):
        out = np.zeros((n, k), np.complex128) if k else np.zeros(n, np.complex128)
        for off, m in ((0, nh), (nh * nh, ne)):
            for d in range(max(k, 1)):
                A = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
                A = A + A.conj().T
                if k:
                    out[off:off + m * m, d] = A.reshape(-1)
                else:
                    out[off:off + m * m] = A.reshape(-1)
        return out

    S, Lm, L2, LS = herm_blocks(3), herm_blocks(3), herm_blocks(0), herm_blocks(0)
    C, _ = np.linalg.qr(rng.normal(size=(nx, nx)) + 1j * rng.normal(size=(nx, nx)))
    C = np.ascontiguousarray(C)
    out = [np.empty(nx * 3, np.complex128), np.empty(nx, np.complex128), np.empty(nx * 3, np.complex128),
           np.empty(nx, np.complex128), np.empty(nx, np.complex128)]
    lib.fbse_xton_ang_stats.argtypes = [ctypes.c_long, ctypes.c_long] + [D] * 10
    v = lambda a: np.ascontiguousarray(a).view(np.float64).ctypes.data_as(D)
    assert lib.fbse_xton_ang_stats(nh, ne, v(C), v(S), v(Lm), v(L2), v(LS), *[v(o) for o in out]) == 0
    want = O.xton_ang_stats(C, S, Lm, L2, LS, nh, ne)
    got = [out[0].reshape(nx, 3), out[1], out[2].reshape(nx, 3), out[3], out[4]]
    for g_, w in zip(got, want):
        assert np.max(np.abs(g_ - w)) < 1e-12 * max(1.0, np.max(np.abs(w)))
