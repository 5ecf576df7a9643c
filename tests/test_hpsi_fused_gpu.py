"""H psi with the projector gather and scatter fused into the xy plane passes
of the 3D FFT (FP32, 128 x 128 x nz grids; fbse_tuning.hpsi_fused = 1).
Checked against the FP64 oracle (mixed-path tolerance), against the separate
projector kernels (rounding only), and for run-to-run and batch-size
determinism."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import random_states, tiny_cluster

pytestmark = pytest.mark.gpu

TOL = 3e-6  # relative max-norm error of the mixed path against the FP64 oracle


def _ctx(F, sysm, fused=1):
    c = F.Context(sysm.grid, sysm.pot, nspin=sysm.nspin, is_complex=sysm.is_complex, so=sysm.so, nl=sysm.nlflag,
                  proj=sysm.proj, precision=F.MIXED)
    c.set_tuning(hpsi_fused=fused)
    return c


def _hpsi(ctx, psis, dev):
    import torch
    x = torch.tensor(np.asarray(psis), dtype=ctx.working_dtype(), device=dev).contiguous()
    y = torch.empty_like(x)
    ctx.hpsi(x, y)
    return y.cpu().numpy().astype(np.complex128)


def _relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _launches(fbse, ctx, psis, dev):
    """kernels launched by one H psi of psis (after a first call has set up)"""
    _hpsi(ctx, psis, dev)
    c0 = fbse.launch_count()
    _hpsi(ctx, psis, dev)
    return fbse.launch_count() - c0


@pytest.mark.parametrize("nz,so,nl", [(64, True, False), (64, False, True), (64, True, True), (128, True, False),
                                      (45, True, False)])
def test_fused_matches_oracle(fbse, cuda, nz, so, nl):
    sysm = tiny_cluster(128, 128, nz, natoms=10, nspin=2, is_complex=True, so=so, nl=nl)
    psis = random_states(2, sysm, np.random.default_rng(11))
    ctx = _ctx(fbse, sysm)
    got = _hpsi(ctx, psis, cuda)
    # the fused path: two plane launches, the coefficient sums and the z pass
    assert _launches(fbse, ctx, psis, cuda) == 4
    want = np.array([O.hamiltonian(p, sysm) for p in psis])
    err = _relerr(got, want)
    print(f"\n[fused H psi 128x128x{nz} so={so} nl={nl}] relative error {err:.2e}")
    assert err < TOL


def test_fused_real_packing(fbse, cuda):
    """Real job with NL projectors: two real states packed as re / im."""
    sysm = tiny_cluster(128, 128, 64, natoms=10, nspin=1, is_complex=False, nl=True)
    rng = np.random.default_rng(12)
    a = rng.uniform(-1, 1, (2, sysm.ngrid))
    ctx = _ctx(fbse, sysm)
    got = _hpsi(ctx, (a[0] + 1j * a[1]).reshape(1, -1), cuda)[0]
    assert _launches(fbse, ctx, (a[0] + 1j * a[1]).reshape(1, -1), cuda) == 4
    w0 = O.hamiltonian(a[0].astype(np.complex128), sysm).real
    w1 = O.hamiltonian(a[1].astype(np.complex128), sysm).real
    scale = max(np.abs(w0).max(), np.abs(w1).max())
    assert np.max(np.abs(got.real - w0)) / scale < TOL
    assert np.max(np.abs(got.imag - w1)) / scale < TOL


def test_fused_against_separate_kernels_on_the_3nm_dot(fbse, cuda):
    """The 3 nm CdSe dot of the throughput benchmark (693 atoms, spinor + SO,
    128^3): the fused and the separate projector kernels differ in rounding
    only; the fused path is bit-identical over repeated runs and batch sizes."""
    from filterbse_gb300 import workload as W
    dot = W.cdse_dot(15.0, d=0.5, ke_max=10.0, spinor=True)
    g = dot.grid

    def mk(fused):
        c = fbse.Context(g, dot.pot, nspin=2, is_complex=True, so=True, nl=False, proj=dot.proj, precision=fbse.MIXED)
        c.set_tuning(hpsi_fused=fused)
        return c
    rng = np.random.default_rng(13)
    n = 5
    psis = (rng.uniform(-1, 1, (n, 2 * g.ngrid)) + 1j * rng.uniform(-1, 1, (n, 2 * g.ngrid))).astype(np.complex64)
    fused = mk(1)
    sep = mk(0)
    a = _hpsi(fused, psis, cuda)
    b = _hpsi(sep, psis, cuda)
    # fused: 4 kernels; separate: gather, three FFT passes and scatter for each
    # half of the batch (the halves run on the context's two streams)
    assert _launches(fbse, fused, psis, cuda) == 4 and _launches(fbse, sep, psis, cuda) == 2 * 5
    err = _relerr(a, b)
    print(f"\n[fused vs separate, 3 nm dot] relative difference {err:.2e}")
    assert err < 2e-6
    assert np.array_equal(a, _hpsi(fused, psis, cuda))
    for lo, hi in ((0, 1), (1, 4), (3, 5)):
        assert np.array_equal(a[lo:hi], _hpsi(fused, psis[lo:hi], cuda)), (lo, hi)
