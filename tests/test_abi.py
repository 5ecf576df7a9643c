"""CPU checks of the product library: it loads, exports every symbol that
include/fbse.h declares, and its host-side helpers (random starts, Newton
nodes and coefficients) reproduce the oracle bit for bit."""
import os
import re

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "fbse.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fbse_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(fbse):
    L = fbse.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(fbse.EXPORTED) | set(names)


def test_null_context_is_an_argument_error(fbse):
    """Every entry point that takes a context returns FBSE_ERR_ARG for a NULL
    context (and NULL buffers, zero sizes) without touching a device; argument
    types come from the header's declarations."""
    import ctypes
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "fbse.h")).read(), flags=re.S)
    decls = re.findall(r"\b(?:int|long|double|void|const char)\s*\*?\s*(fbse_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src)
    assert len(decls) == len(_declared())
    L = ctypes.CDLL(fbse.load()._name)
    checked = 0
    for name, params in decls:
        ps = [p.strip() for p in params.split(",") if p.strip() and p.strip() != "void"]
        if not ps or not ps[0].startswith("fbse_ctx") or name in ("fbse_destroy", "fbse_last_error", "fbse_stream"):
            continue
        types, args = [], []
        for p in ps:
            if "*" in p:
                types.append(ctypes.c_void_p); args.append(None)
            elif "double" in p:
                types.append(ctypes.c_double); args.append(0.0)
            elif "size_t" in p:
                types.append(ctypes.c_size_t); args.append(0)
            elif "long" in p:
                types.append(ctypes.c_long); args.append(0)
            else:
                assert "int" in p, (name, p)
                types.append(ctypes.c_int); args.append(0)
        fn = getattr(L, name)
        fn.argtypes, fn.restype = types, ctypes.c_int
        assert fn(*args) == -1, name  # FBSE_ERR_ARG
        checked += 1
    assert checked >= 20


def test_version(fbse):
    src = open(os.path.join(ROOT, "include", "fbse.h")).read()
    want = int(re.search(r"#define FBSE_ABI_VERSION (\d+)", src).group(1))
    assert fbse.load().fbse_version() == want


def test_context_without_gpu_fails_cleanly(fbse):
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    g = O.Grid(8, 8, 8, 0.8, 0.8, 0.8, -3.2, -3.2, -3.2, 10.0)
    with pytest.raises(fbse.FbseError):
        fbse.Context(g, np.zeros(g.ngrid))


def test_samp_points_bit_exact(fbse):
    for nc in (2, 3, 64, 1024):
        zn, fk = fbse.samp_points(nc)
        re, im, fk2 = O.samp_points(nc)
        assert np.array_equal(zn, re) and np.all(im == 0)


def test_newton_coeff_bit_exact(fbse):
    zn, _ = fbse.samp_points(300)
    t = np.array([-0.3, -0.29, -0.12])
    de, vmin = 13.46, -1.1327
    dt = O.filter_dt(300, de)
    assert np.array_equal(fbse.newton_coeff(zn, t, vmin, de, dt), O.newton_coeff(zn, t, vmin, de, dt))


@pytest.mark.parametrize("nspin,cplx", [(1, False), (1, True), (2, True)])
def test_init_filter_states_bit_exact(fbse, nspin, cplx):
    ngrid, n, dv = 2000, 3, 0.512
    got, seeds, s_end = fbse.init_filter_states(n, ngrid, nspin, cplx, dv, -4242)
    want, wseeds, w_end = O.init_filter_states(-4242, n, ngrid, nspin, cplx, dv)
    if cplx:
        want = want.view(np.float64).reshape(n, -1)
    else:
        want = want.real
    assert np.array_equal(got, want)
    assert list(seeds) == list(wseeds) and s_end == w_end


def test_newton_interpolant_approximates_filter():
    """check_function (coeff.c:297-325): the Newton form reproduces the Gaussian."""
    nc = 512
    zn, _, _ = O.samp_points(nc)
    de, vmin = 10.0, -1.0
    dt = O.filter_dt(nc, de)
    t = np.array([0.5])
    an = O.newton_coeff(zn, t, vmin, de, dt)[0].real
    xs = np.linspace(-2, 2, 81)
    f = np.full_like(xs, an[0])
    w = np.ones_like(xs)
    for j in range(1, nc):
        w = w * (xs - zn[j - 1])
        f = f + an[j] * w
    e = (xs + 2.0) * de / 4.0 + vmin
    g = np.sqrt(dt / np.pi) * np.exp(-dt * (e - t[0]) ** 2)
    assert np.max(np.abs(f - g)) < 1e-5 * np.max(g)
