"""fbse_normalize_all_noalloc against fbse_normalize_all.

The no-allocation variant keeps its scratch in a file-scope device array; it
must give the same norms and normalised states as the allocating entry point,
call after call, and refuse a state count above its scratch size.  This file
is collected last so that it also runs after every other GPU test."""
import ctypes

import numpy as np
import pytest

from tests.systems import tiny_cluster

pytestmark = pytest.mark.gpu

MAX_STATES = 1024


def _bind(L):
    f = L.fbse_normalize_all_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long, ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    return f


def _run_noalloc(fbse, ctx, psitot):
    f = _bind(fbse.load())
    n = psitot.shape[0]
    norms = np.empty(n)
    ctx._torch_sync()
    rc = f(ctx._h, ctypes.c_void_p(psitot.data_ptr()), n, norms.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if rc:
        raise fbse.FbseError(rc, fbse.load().fbse_last_error(ctx._h).decode())
    return norms


@pytest.mark.parametrize("cplx", [False, True])
def test_noalloc_matches_normalize_all_twice(fbse, cuda, cplx):
    import torch
    sysm = tiny_cluster(10, 9, 8, natoms=4, nspin=2 if cplx else 1, is_complex=cplx, so=False, nl=False)
    ctx = fbse.Context(sysm.grid, sysm.pot, nspin=sysm.nspin, is_complex=cplx)
    stlen = (2 if cplx else 1) * sysm.nspin * sysm.ngrid
    rng = np.random.default_rng(11)
    for call, n in enumerate((37, 200)):
        x = rng.normal(size=(n, stlen)) * rng.uniform(0.1, 10.0, size=(n, 1))
        a = torch.tensor(x, device=cuda)
        b = a.clone()
        na = ctx.normalize_all(a)
        nb = _run_noalloc(fbse, ctx, b)
        assert np.allclose(nb, na, rtol=1e-14, atol=0), f"call {call}"
        assert torch.allclose(b, a, rtol=1e-14, atol=0), f"call {call}"
        nrm = (b.double() ** 2).sum(dim=1).cpu().numpy() * sysm.grid.dv
        assert np.allclose(nrm, 1.0, atol=1e-12)


def test_noalloc_rejects_oversize_and_zero_norm(fbse, cuda):
    import torch
    sysm = tiny_cluster(8, 8, 8, natoms=2, nspin=1, is_complex=False, so=False, nl=False)
    ctx = fbse.Context(sysm.grid, sysm.pot, nspin=1, is_complex=False)
    big = torch.ones((MAX_STATES + 1, sysm.ngrid), dtype=torch.float64, device=cuda)
    with pytest.raises(fbse.FbseError, match="exceed"):
        _run_noalloc(fbse, ctx, big)
    x = torch.ones((3, sysm.ngrid), dtype=torch.float64, device=cuda)
    x[1] = 0
    before = x.clone()
    f = _bind(fbse.load())
    norms = np.full(3, -7.0)
    ctx._torch_sync()
    rc = f(ctx._h, ctypes.c_void_p(x.data_ptr()), 3, norms.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc != 0 and "Norm is 0" in fbse.load().fbse_last_error(ctx._h).decode()
    assert torch.equal(x, before)
    # norms as fbse_normalize_all leaves them: written up to the failing state
    assert np.allclose(norms[:2], [sysm.ngrid * sysm.grid.dv, 0.0]) and norms[2] == -7.0
    with pytest.raises(fbse.FbseError, match="Norm is 0"):
        ctx.normalize_all(before.clone())
    # the key is reset per call: a good call right after the failing one succeeds
    y = torch.ones((3, sysm.ngrid), dtype=torch.float64, device=cuda)
    n = _run_noalloc(fbse, ctx, y)
    assert np.allclose(n, sysm.ngrid * sysm.grid.dv)
