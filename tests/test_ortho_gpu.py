"""Orthogonalisation + subspace diagonalisation + sigma_E on the GPU.

The oracle builds the dense H of a tiny system (H applied to every unit
vector), so exact eigenpairs are known; the GPU's Rayleigh-Ritz over a
subspace spanned by mixtures of exact eigenvectors (plus a rank-deficient
duplicate) must return those eigenvalues with tiny residuals, and on a
generic subspace must agree with the oracle's SVD + dense diagonalisation
(ortho.c / Hmat.c restated with numpy.linalg)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import tiny_cluster

pytestmark = pytest.mark.gpu


def _dense_h(sysm):
    n = sysm.nspin * sysm.ngrid
    H = np.empty((n, n), np.complex128)
    e = np.zeros(n, np.complex128)
    for j in range(n):
        e[:] = 0
        e[j] = 1.0
        H[:, j] = O.hamiltonian(e, sysm)
    if not sysm.is_complex:
        H = H.real
    return 0.5 * (H + H.conj().T)


def _ctx(F, sysm, precision):
    return F.Context(sysm.grid, sysm.pot, nspin=sysm.nspin, is_complex=sysm.is_complex, so=sysm.so, nl=sysm.nlflag,
                     proj=sysm.proj, precision=precision)


@pytest.mark.parametrize("cplx", [False, True])
def test_ritz_recovers_exact_eigenpairs(fbse, cuda, cplx):
    import torch
    sysm = tiny_cluster(8, 9, 10, natoms=5, nspin=2 if cplx else 1, is_complex=cplx, so=cplx, nl=True)
    H = _dense_h(sysm)
    w, v = np.linalg.eigh(H)
    dv = sysm.grid.dv
    rng = np.random.default_rng(5)
    k = 10
    pick = np.arange(3, 3 + k)
    mix = rng.normal(size=(k, k)) + (1j * rng.normal(size=(k, k)) if cplx else 0)
    psis = (v[:, pick] @ mix).T  # k states spanning the eigenvectors
    psis = np.vstack([psis, psis[0] + psis[1]])  # a dependent state: rank stays k
    psis /= np.sqrt(dv)
    if cplx:
        tot = np.ascontiguousarray(psis).view(np.float64).reshape(len(psis), -1)
    else:
        tot = np.ascontiguousarray(psis.real)
    ctx = _ctx(fbse, sysm, 0)
    t = torch.tensor(tot, device=cuda)
    nk, ev, sg = ctx.ortho_diag_sigma(t)
    assert nk == k
    assert np.allclose(ev, w[pick], atol=1e-11)
    assert np.max(sg) < 1e-8
    # returned states are normalised eigenvectors: each lies in the exact
    # eigenspace of its eigenvalue (spin-orbit spectra are Kramers-degenerate,
    # so compare against the whole degenerate cluster)
    out = t.cpu().numpy()[:nk]
    st = out.view(np.complex128) if cplx else out
    for i in range(nk):
        cl = np.nonzero(np.abs(w - ev[i]) < 1e-8)[0]
        proj = v[:, cl].conj().T @ st[i] * np.sqrt(dv)
        assert abs(np.linalg.norm(proj) - 1.0) < 1e-9
        assert abs(np.linalg.norm(st[i]) * np.sqrt(dv) - 1.0) < 1e-12


@pytest.mark.parametrize("precision,etol", [(0, 1e-10), (1, 2e-5)])
def test_ritz_matches_oracle_on_generic_subspace(fbse, cuda, precision, etol):
    import torch
    sysm = tiny_cluster(9, 8, 10, natoms=5, is_complex=False, nl=True)
    H = _dense_h(sysm)
    w, v = np.linalg.eigh(H)
    rng = np.random.default_rng(8)
    # smooth-ish subspace: low eigenvectors plus a little of everything
    n = 12
    psis = (v[:, :20] @ rng.normal(size=(20, n))).T + 1e-3 * rng.normal(size=(n, H.shape[0]))
    psis /= np.sqrt(sysm.grid.dv)
    u, keep = O.ortho(psis.astype(np.complex128), False, dv=sysm.grid.dv)
    e_or, vec = O.diag(u.astype(np.complex128), sysm)
    e_or2, s_or = O.sigma_e(vec, sysm)
    ctx = _ctx(fbse, sysm, precision)
    t = torch.tensor(np.ascontiguousarray(psis), device=cuda)
    nk, ev, sg = ctx.ortho_diag_sigma(t)
    assert nk == len(e_or)
    assert np.allclose(ev, e_or, atol=etol * max(1.0, np.max(np.abs(e_or))))
    assert np.allclose(sg, s_or, rtol=1e-3 if precision == 0 else 3e-2, atol=etol * 10)


@pytest.mark.parametrize("cplx", [True, False])
def test_slab_gram_and_rotation(fbse, cuda, cplx):
    """fbse_gram / fbse_rotate against numpy, and the sharded step's identity:
    the sum of the Grams of the slabs of the points is the Gram of the whole
    states, and rotating each slab gives the slabs of the rotated states."""
    import torch
    sysm = tiny_cluster(12, 11, 10, natoms=4, nspin=2 if cplx else 1, is_complex=cplx)
    rng = np.random.default_rng(21)
    na, nb, k = 7, 5, 3
    L = sysm.nspin * sysm.ngrid
    stlen = (2 if cplx else 1) * L
    A = rng.normal(size=(na, stlen))
    B = rng.normal(size=(nb, stlen))
    ctx = fbse.Context(sysm.grid, sysm.pot, nspin=sysm.nspin, is_complex=cplx)
    Ad, Bd = torch.tensor(A, device=cuda), torch.tensor(B, device=cuda)
    ac = A.view(np.complex128) if cplx else A
    bc = B.view(np.complex128) if cplx else B
    want = ac.conj() @ bc.T * sysm.grid.dv
    got = ctx.gram(Ad, Bd)
    assert np.max(np.abs(got - want)) < 1e-12 * np.max(np.abs(want))
    bounds = [(0, L // 3), (L // 3, L // 2), (L // 2, L)]
    parts = sum(ctx.gram(Ad, Bd, lo, hi - lo) for lo, hi in bounds)
    assert np.max(np.abs(parts - want)) < 1e-12 * np.max(np.abs(want))
    C = rng.normal(size=(na, k)) + (1j * rng.normal(size=(na, k)) if cplx else 0)
    out = torch.zeros((k, stlen), dtype=torch.float64, device=cuda)
    for lo, hi in bounds:
        ctx.rotate(Ad, C, out, lo, hi - lo)
    rot = (C.T @ ac) if cplx else (C.real.T @ ac)
    got_r = out.cpu().numpy().view(np.complex128) if cplx else out.cpu().numpy()
    assert np.max(np.abs(got_r - rot)) < 1e-12 * np.max(np.abs(rot))


def test_sharded_ritz_through_the_library(fbse, cuda, tmp_path):
    """shard.ritz_library on one rank (a gloo group of one, the whole grid as
    its slab) gives the Ritz values of fbse_ortho_diag_sigma."""
    import torch
    import torch.distributed as dist
    from filterbse_gb300 import shard
    sysm = tiny_cluster(14, 13, 12, natoms=6, nspin=2, is_complex=True, so=True)
    ctx = fbse.Context(sysm.grid, sysm.pot, nspin=2, is_complex=True, so=True, proj=sysm.proj)
    rng = np.random.default_rng(8)
    n = 6
    psi = torch.tensor(rng.normal(size=(n, ctx.stlen)), device=cuda)
    hpsi = ctx.residual(psi, np.zeros(n))  # H psi
    ref = psi.clone()
    _, ev, sg = ctx.ortho_diag_sigma(ref)
    dist.init_process_group("gloo", init_method=f"file://{tmp_path}/pg", rank=0, world_size=1)
    try:
        exch = shard.ShardedRitz(deadline=10.0)
        e, s, rot = shard.ritz_library(exch, ctx, psi, hpsi, 0, sysm.nspin * sysm.ngrid)
    finally:
        dist.destroy_process_group()
    assert len(e) == len(ev) and np.max(np.abs(np.sort(e) - np.sort(ev))) < 1e-10
    assert np.max(np.abs(np.sort(s) - np.sort(sg))) < 1e-6
