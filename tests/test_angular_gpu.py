"""fbse_angular_stats (the filter's calcSpinAngStat, filter_mpi/angular.c:4-165)
against the oracle's restatement, on random spinors over grids with odd and
even axes (both reciprocal-spacing rules and every FFT path), on states of
known angular momentum, in both context precisions (the statistics are FP64
either way), and its error cases."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import tiny_cluster
from tests.test_angular import analytic_states

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,prec", [((20, 18, 21), 0), ((16, 15, 12), 1), ((64, 64, 64), 0)])
def test_angular_stats_match_oracle(fbse, cuda, shape, prec):
    import torch
    sysm = tiny_cluster(*shape, natoms=4, nspin=2, is_complex=True)
    ctx = fbse.Context(sysm.grid, sysm.pot, nspin=2, is_complex=True, precision=prec)
    g = sysm.grid
    rng = np.random.default_rng(5)
    gx, gy, gz = g.axes()
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    env = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 8.0).reshape(-1)
    rows = []
    for k in range(4):
        z = rng.normal(size=2 * g.ngrid) + 1j * rng.normal(size=2 * g.ngrid)
        if k % 2:  # smooth, localised states as well as white noise
            z = z * np.concatenate([env, env])
        rows.append(z.view(np.float64))
    rows = np.array(rows)
    got = ctx.angular_stats(torch.tensor(rows, device=cuda), gx, gy, gz)
    want = O.filter_angular_stats(rows, g)
    scale = np.max(np.abs(want), axis=1, keepdims=True)
    err = np.max(np.abs(got - want) / scale)
    print(f"\n[angular {shape} prec {prec}] max rel dev {err:.2e}")
    assert err < 1e-11
    ctx.close()


def test_angular_stats_known_states(fbse, cuda):
    import torch
    g = O.Grid(32, 32, 32, 0.5, 0.5, 0.5, -8.0, -8.0, -8.0, 10.0)
    ctx = fbse.Context(g, np.zeros(g.ngrid), nspin=2, is_complex=True)
    rows, want = analytic_states(g)
    got = ctx.angular_stats(torch.tensor(rows, device=cuda), *g.axes())
    assert np.allclose(got, want, atol=1e-8, rtol=0), got
    ctx.close()


def test_angular_stats_errors(fbse, cuda):
    import torch
    sysm = tiny_cluster(12, 12, 12, natoms=2, nspin=1, is_complex=False)
    g = sysm.grid
    real = fbse.Context(g, sysm.pot, nspin=1, is_complex=False)
    with pytest.raises(fbse.FbseError, match="spinor"):
        real.angular_stats(torch.zeros((1, g.ngrid), dtype=torch.float64, device=cuda), *g.axes())
    real.close()
    ctx = fbse.Context(g, sysm.pot, nspin=2, is_complex=True)
    with pytest.raises(fbse.FbseError, match="Norm is 0"):
        ctx.angular_stats(torch.zeros((1, 4 * g.ngrid), dtype=torch.float64, device=cuda), *g.axes())
    ctx.close()
