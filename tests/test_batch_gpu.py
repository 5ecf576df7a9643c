"""Multi-dot filter in one CUDA graph (fbse_batch_*): uneven dots (different
grids, atoms and start counts) filtered by one graph launch give bit-identical
states to the dot-by-dot path, on every replay, and match the FP64 oracle's
filter_cycle on a dot small enough for it."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import tiny_cluster

pytestmark = pytest.mark.gpu


def _dots(fbse, cuda, precision):
    import torch
    out = []
    for k, (shape, nat, nstart, nc) in enumerate((((16, 18, 15), 6, 2, 40), ((20, 20, 21), 10, 3, 33),
                                                   ((12, 14, 13), 4, 1, 50))):
        sysm = tiny_cluster(*shape, natoms=nat, nspin=2, is_complex=True, so=True, nl=True, seed=7 + k)
        ctx = fbse.Context(sysm.grid, sysm.pot, nspin=2, is_complex=True, so=True, nl=True, proj=sysm.proj,
                           precision=precision)
        emin, emax = float(sysm.pot.min()) - 1.5, float(sysm.pot.max()) + sysm.grid.ke_max + 2.0
        de = emax - emin
        zn, _, _ = O.samp_points(nc)
        an = O.newton_coeff(zn, np.linspace(emin + 0.1 * de, emin + 0.3 * de, 3), emin, de, O.filter_dt(nc, de))
        starts, _, _ = O.init_filter_states(-100 - k, nstart, sysm.ngrid, 2, True, sysm.grid.dv)
        p0 = torch.tensor(np.ascontiguousarray(starts.view(np.float64).reshape(nstart, -1)), device=cuda)
        out.append((sysm, ctx, zn, an, emin, de, p0, starts))
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_graph_batch_matches_sequential(fbse, cuda, precision):
    dots = _dots(fbse, cuda, precision)
    b = fbse.Batch([(ctx, zn, an, emin, de, p0) for _, ctx, zn, an, emin, de, p0, _ in dots])
    assert b.nodes > 100
    seq_first = [o.cpu().numpy().copy() for o in b.out]  # the ordinary run made by create
    b.run()
    g1 = [o.cpu().numpy().copy() for o in b.out]
    b.run()
    g2 = [o.cpu().numpy().copy() for o in b.out]
    b.run(sequential=True)
    s1 = [o.cpu().numpy().copy() for o in b.out]
    for a, c, d, e in zip(seq_first, g1, g2, s1):
        assert np.array_equal(a, c) and np.array_equal(c, d) and np.array_equal(c, e)
    # the smallest dot against the FP64 oracle
    sysm, ctx, zn, an, emin, de, p0, starts = dots[2]
    want = O.filter_cycle(starts[0], sysm, an, zn, emin, de).view(np.float64).reshape(3, -1)
    err = np.max(np.abs(g1[2][0] - want)) / np.max(np.abs(want))
    assert err < (1e-10 if precision == 0 else 2e-4), err
    b.close()
