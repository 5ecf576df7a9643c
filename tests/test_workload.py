"""The synthetic workload generator's grid choices (CPU): the uneven-dot
grids grow from the reference's rule to the next size whose prime factors are
at most 7, never shrink, and keep the rule's centring."""
import numpy as np

from filterbse_gb300 import workload as W


def test_smooth_size():
    assert [W.smooth_size(n) for n in (116, 148, 104, 100, 120, 127, 128, 149, 1)] == \
        [120, 150, 105, 100, 120, 128, 128, 150, 1]
    for n in range(1, 400):
        m = W.smooth_size(n)
        assert m >= n
        r = m
        for p in (2, 3, 5, 7):
            while r % p == 0:
                r //= p
        assert r == 1


def test_smooth_grid_contains_the_rule_grid():
    cat, an, a_ang, _ = W.MATERIALS["InP"]
    types, coords = W.zincblende_dot(5.0 * 2.5, a_ang, cat, an)
    g = W.reference_grid(coords, 0.5, 10.0)
    n = tuple(W.smooth_size(v) for v in (g.nx, g.ny, g.nz))
    g2 = W.reference_grid(coords, 0.5, 10.0, n_in=n)
    assert (g2.nx, g2.ny, g2.nz) == n
    for lo, lo2 in ((g.xmin, g2.xmin), (g.ymin, g2.ymin), (g.zmin, g2.zmin)):
        assert lo2 <= lo  # the larger box still holds the rule's box
    assert np.all(coords.min(axis=0) > np.array([g2.xmin, g2.ymin, g2.zmin]))
