"""Newton filter, spectrum range, normalisation and energies on the GPU
against the FP64 oracle (filter_cycle, get_energy_range, normalize_all,
energy_all)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import tiny_cluster

pytestmark = pytest.mark.gpu


def _ctx(F, sysm, precision):
    return F.Context(sysm.grid, sysm.pot, nspin=sysm.nspin, is_complex=sysm.is_complex, so=sysm.so, nl=sysm.nlflag,
                     proj=sysm.proj, precision=precision)


def _range(sysm):
    return float(np.min(sysm.pot)) - 1.5, float(np.max(sysm.pot)) + sysm.grid.ke_max + 2.0


def _filter_case(fbse, cuda, sysm, nstart, ncheby, m, precision, seed=-12345):
    import torch
    emin, emax = _range(sysm)
    de = emax - emin
    zn, _, _ = O.samp_points(ncheby)
    targets = np.linspace(emin + 0.15 * de, emin + 0.2 * de, m)
    an = O.newton_coeff(zn, targets, emin, de, O.filter_dt(ncheby, de))
    starts, _, _ = O.init_filter_states(seed, nstart, sysm.ngrid, sysm.nspin, sysm.is_complex, sysm.grid.dv)
    # psitot layout for the GPU
    if sysm.is_complex:
        p0 = starts.view(np.float64).reshape(nstart, -1)
    else:
        p0 = starts.real.copy()
    ctx = _ctx(fbse, sysm, precision)
    out = ctx.newton_filter(zn, an, emin, de, torch.tensor(p0, device=cuda)).cpu().numpy()
    want = np.array([O.filter_cycle(s, sysm, an, zn, emin, de) for s in starts])  # [nstart, m, L] complex
    if sysm.is_complex:
        want = want.view(np.float64).reshape(nstart, m, -1)
    else:
        want = want.real
    return out, want


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 2e-4)])
def test_newton_filter_real(fbse, cuda, precision, tol):
    sysm = tiny_cluster(18, 17, 16, natoms=8, is_complex=False, nl=True)
    out, want = _filter_case(fbse, cuda, sysm, nstart=3, ncheby=40, m=3, precision=precision)
    for s in range(3):
        for t in range(3):
            err = np.max(np.abs(out[s, t] - want[s, t])) / np.max(np.abs(want[s, t]))
            assert err < tol, (s, t, err)


@pytest.mark.parametrize("precision,tol", [(0, 1e-10), (1, 2e-4)])
def test_newton_filter_spinor(fbse, cuda, precision, tol):
    sysm = tiny_cluster(16, 18, 15, natoms=8, nspin=2, is_complex=True, so=True, nl=True)
    out, want = _filter_case(fbse, cuda, sysm, nstart=2, ncheby=37, m=2, precision=precision)
    for s in range(2):
        for t in range(2):
            err = np.max(np.abs(out[s, t] - want[s, t])) / np.max(np.abs(want[s, t]))
            assert err < tol, (s, t, err)


def test_newton_filter_single_term(fbse, cuda):
    """ncheby = 1: the filter is a0 * psi0 (edge of the K-blocked ring)."""
    sysm = tiny_cluster(12, 12, 12, natoms=4, is_complex=True)
    out, want = _filter_case(fbse, cuda, sysm, nstart=1, ncheby=2, m=1, precision=0)
    assert np.max(np.abs(out - want)) <= 1e-12 * np.max(np.abs(want))


@pytest.mark.parametrize("precision,tol", [(0, 1e-9), (1, 1e-5)])
def test_energy_range(fbse, cuda, precision, tol):
    sysm = tiny_cluster(16, 14, 15, natoms=6, is_complex=False)
    ctx = _ctx(fbse, sysm, precision)
    e0, e1, it = ctx.energy_range(max_iter=60)
    # the oracle runs the same iteration with the same random starts
    r = O.energy_range(sysm, max_iter=60)
    assert abs(e0 - r[2]) < tol * abs(r[2]) + 1e-12
    assert abs(e1 - r[3]) < tol * abs(r[3]) + 1e-12


@pytest.mark.parametrize("cplx", [False, True])
def test_normalize_and_energy(fbse, cuda, cplx):
    import torch
    sysm = tiny_cluster(14, 15, 16, natoms=6, nspin=2 if cplx else 1, is_complex=cplx, so=cplx, nl=True)
    rng = np.random.default_rng(9)
    n = 5
    L = sysm.nspin * sysm.ngrid * (2 if cplx else 1)
    psitot = rng.uniform(-1, 1, (n, L))
    ctx = _ctx(fbse, sysm, 0)
    t = torch.tensor(psitot, device=cuda)
    norms = ctx.normalize_all(t)
    got = t.cpu().numpy()
    want_n = np.sum(psitot ** 2, axis=1) * sysm.grid.dv
    assert np.allclose(norms, want_n, rtol=1e-13)
    want = psitot / np.sqrt(want_n)[:, None]
    assert np.max(np.abs(got - want)) < 1e-13 * np.max(np.abs(want))
    ene = ctx.energy_all(t)
    st = got.view(np.complex128) if cplx else got.astype(np.complex128)
    wantE = [O.energy(s if cplx else s.real.astype(np.complex128), sysm) for s in st]
    assert np.allclose(ene, wantE, rtol=1e-11, atol=1e-12)
    # calc_sigma_E on the same normalised states (n = 5: an odd tail of packed real pairs)
    ev, sg = ctx.sigma_e(t)
    wev, wsg = O.sigma_e(st, sysm)
    assert np.allclose(ev, wev, rtol=1e-11, atol=1e-12)
    assert np.allclose(sg, wsg, rtol=1e-9)


def test_normalize_zero_norm_errors(fbse, cuda):
    import torch
    sysm = tiny_cluster(10, 10, 10, natoms=2)
    ctx = _ctx(fbse, sysm, 0)
    t = torch.zeros((2, sysm.ngrid), dtype=torch.float64, device=cuda)
    with pytest.raises(fbse.FbseError) as ei:
        ctx.normalize_all(t)
    assert ei.value.code == -4
