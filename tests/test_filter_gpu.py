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


@pytest.mark.parametrize("pinned", [True, False])
def test_filter_job_matches_device_path(fbse, cuda, pinned):
    """fbse_filter_job on host buffers = newton_filter + ortho_diag_sigma on
    device buffers, with mod_output's sigma cut; pinned output buffers are
    filled by the device directly, pageable ones by copies."""
    import torch
    sysm = tiny_cluster(16, 18, 15, natoms=8, nspin=2, is_complex=True, so=True, nl=True)
    emin, emax = _range(sysm)
    de = emax - emin
    ncheby, m, nstart = 60, 3, 3
    zn, _, _ = O.samp_points(ncheby)
    targets = np.linspace(emin + 0.1 * de, emin + 0.3 * de, m)
    an = O.newton_coeff(zn, targets, emin, de, O.filter_dt(ncheby, de))
    starts, _, _ = O.init_filter_states(-777, nstart, sysm.ngrid, sysm.nspin, sysm.is_complex, sysm.grid.dv)
    p0 = np.ascontiguousarray(starts.view(np.float64).reshape(nstart, -1))
    ctx = _ctx(fbse, sysm, 0)
    filt = ctx.newton_filter(zn, an, emin, de, torch.tensor(p0, device=cuda))
    nk, ev, sg = ctx.ortho_diag_sigma(filt.reshape(nstart * m, -1))
    ref_states = filt.reshape(nstart * m, -1)[:nk].cpu().numpy()
    stlen = p0.shape[1]
    dv = sysm.grid.dv

    def run(cut):
        out = torch.zeros((nstart * m, stlen), dtype=torch.float64)
        if pinned:
            out = out.pin_memory()
        k, e, s_ = ctx.filter_job(zn, an, emin, de, p0, sigma_cut=cut, psi_out=out)
        return k, e, s_, out.numpy()

    # every state (getAllStates): the same Ritz values and the same span (the
    # spin-orbit levels are Kramers pairs, so compare subspaces, not vectors)
    k, ev_j, sg_j, got = run(0.0)
    assert k == nk and np.max(np.abs(ev_j - ev)) < 1e-10
    a = got[:k].view(np.complex128)
    b = ref_states.view(np.complex128)
    sv = np.linalg.svd(a @ b.conj().T * dv, compute_uv=False)
    assert np.max(np.abs(sv - 1.0)) < 1e-8
    assert not np.any(got[k:])
    # the sigma cut of mod_output
    srt = np.sort(sg_j)
    gaps = [(srt[i + 1] - srt[i], i) for i in range(len(srt) - 1) if srt[i + 1] - srt[i] > 1e-9 * srt[i + 1]]
    assert gaps
    i_cut = min(gaps, key=lambda t: abs(t[1] - len(srt) // 2))[1]
    cut = float(0.5 * (srt[i_cut] + srt[i_cut + 1]))  # between two separated values
    k2, ev2, sg2, got2 = run(cut)
    assert k2 == int(np.sum(sg_j <= cut)) and np.all(sg2 <= cut)
    assert np.max(np.abs(ev2 - ev_j[sg_j <= cut])) < 1e-10
    nrm = np.sum(got2[:k2] ** 2, axis=1) * dv
    assert np.max(np.abs(nrm - 1.0)) < 1e-10 and not np.any(got2[k2:])


@pytest.mark.parametrize("precision", [0, 1])
def test_filter_and_ritz_determinism(fbse, cuda, precision):
    """The same starts give bit-identical filtered states whether they are
    filtered together or in two batches and on a second run, and the
    Rayleigh-Ritz step (Gram products, Jacobi eigensolver, rotation) gives
    bit-identical Ritz values, residuals and vectors on a second run."""
    import torch
    sysm = tiny_cluster(16, 18, 15, natoms=10, nspin=2, is_complex=True, so=True, nl=True)
    emin, emax = _range(sysm)
    de = emax - emin
    ncheby, m, nstart = 40, 3, 4
    zn, _, _ = O.samp_points(ncheby)
    targets = np.linspace(emin + 0.1 * de, emin + 0.3 * de, m)
    an = O.newton_coeff(zn, targets, emin, de, O.filter_dt(ncheby, de))
    starts, _, _ = O.init_filter_states(-4242, nstart, sysm.ngrid, sysm.nspin, sysm.is_complex, sysm.grid.dv)
    p0 = torch.tensor(np.ascontiguousarray(starts.view(np.float64).reshape(nstart, -1)), device=cuda)
    ctx = _ctx(fbse, sysm, precision)
    a = ctx.newton_filter(zn, an, emin, de, p0).cpu().numpy()
    b = ctx.newton_filter(zn, an, emin, de, p0).cpu().numpy()
    c = np.concatenate([ctx.newton_filter(zn, an, emin, de, p0[:1]).cpu().numpy(),
                        ctx.newton_filter(zn, an, emin, de, p0[1:]).cpu().numpy()])
    assert np.array_equal(a, b) and np.array_equal(a, c)
    res = []
    for _ in range(2):
        t = torch.tensor(a.reshape(nstart * m, -1), device=cuda)
        nk, ev, sg = ctx.ortho_diag_sigma(t)
        res.append((nk, ev, sg, t[:nk].cpu().numpy()))
    assert res[0][0] == res[1][0]
    for x, y in zip(res[0][1:], res[1][1:]):
        assert np.array_equal(x, y)
