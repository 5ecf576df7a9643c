"""The oracle's restatement of the filter's spin / angular-momentum statistics
(calc_angular_exp, filter_mpi/angular.c:4-165) on states whose angular
quantum numbers are known: a spherical Gaussian times spin up (l = 0,
j = 1/2) and the p orbitals (x +- iy) g(r) times one spin (l = 1, |m| = 1,
j = 3/2, |mj| = 3/2), where <J^2> = 15/4, <Jz^2> = 9/4 and <Jx^2> = <Jy^2> =
(j(j+1) - mj^2)/2 = 3/4.  CPU only."""
import numpy as np

from oracle import oracle as O


def _grid(n=32, d=0.5):
    return O.Grid(n, n, n, d, d, d, -n * d / 2, -n * d / 2, -n * d / 2, 10.0)


def analytic_states(g):
    """(rows in psitot layout, expected angular.dat columns)"""
    gx, gy, gz = g.axes()
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    gs = np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (2 * 1.5 ** 2))

    def row(up, dn):
        return np.concatenate([up.reshape(-1), dn.reshape(-1)]).astype(np.complex128).view(np.float64)

    zero = np.zeros_like(gs)
    rows = [row(gs, zero), row((X + 1j * Y) * gs, zero), row(zero, (X - 1j * Y) * gs), row(zero, 3.0 * gs)]
    want = [[0, 0.25, 0, 0.25, 0.5, 0.25, 0.75, 1], [0, 0.75, 0, 0.75, 1.5, 2.25, 3.75, 1],
            [0, 0.75, 0, 0.75, -1.5, 2.25, 3.75, 1], [0, 0.25, 0, 0.25, -0.5, 0.25, 0.75, 1]]
    return np.array(rows), np.array(want, float)


def test_oracle_angular_stats_known_states():
    g = _grid()
    rows, want = analytic_states(g)
    got = O.filter_angular_stats(rows, g)
    assert np.allclose(got, want, atol=1e-8, rtol=0), got


def test_oracle_angular_stats_invariances():
    """A global phase and the scale of the state do not change the statistics;
    rotating a spin-up s state into spin down flips <Jz> only."""
    g = _grid(24, 0.6)
    rng = np.random.default_rng(3)
    n = g.ngrid
    z = (rng.normal(size=2 * n) + 1j * rng.normal(size=2 * n))
    a = O.filter_angular_stats([z.view(np.float64)], g)[0]
    b = O.filter_angular_stats([(3.7 * np.exp(0.4j) * z).view(np.float64)], g)[0]
    assert np.allclose(a, b, atol=1e-12 * np.max(np.abs(a)))
    assert abs(a[7] - 1.0) < 1e-12
    # <J^2> is the sum of the three squares (angular.c:142)
    assert abs(a[6] - (a[1] + a[3] + a[5])) < 1e-12 * a[6]
