"""Bethe-Salpeter stage on the GPU against the oracle (bse_cplx/ restated).

Quasiparticle states are smooth seeded spinors (sums of complex Gaussians) on
small grids, cubic and not, with odd extents; holes at 0..n_h-1 and the
electrons after a gap state, as get_qp_basis (bse_cplx/basis.c:258) lays them
out.  FP64 results must match the oracle to round-off; the mixed-precision
kernel (FP32 pair densities, FFTs and products, FP64 sums) to 3e-5 of the
largest element."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

GRIDS = {
    "cubic24": O.Grid(24, 24, 24, 0.7, 0.7, 0.7, -8.4, -8.4, -8.4),
    "odd21x20x18": O.Grid(21, 20, 18, 0.75, 0.8, 0.85, -7.5, -8.0, -7.65),
    "ymin_smallest": O.Grid(20, 18, 22, 0.8, 0.8, 0.8, -8.0, -7.2, -8.8),
    "cubic64": O.Grid(64, 64, 64, 0.4, 0.4, 0.4, -12.8, -12.8, -12.8),
}


def qp_states(g: O.Grid, n_qp: int, seed: int, nspin: int = 2):
    rng = np.random.default_rng(seed)
    gx, gy, gz = O.bse_axes(g)
    Z, Y, X = np.meshgrid(gz, gy, gx, indexing="ij")
    N = g.ngrid
    out = np.zeros((n_qp, nspin * N), np.complex128)
    for s in range(n_qp):
        for sp in range(nspin):
            f = np.zeros(X.shape, np.complex128)
            for _ in range(3):
                c = rng.uniform(-3, 3, 3)
                w = rng.uniform(1.2, 2.2)
                amp = rng.normal() + 1j * rng.normal()
                f += amp * (1 + 0.3 * (X - c[0])) * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / w**2)
            out[s, sp * N:(sp + 1) * N] = f.reshape(-1)
        out[s] /= np.sqrt(np.sum(np.abs(out[s]) ** 2) * g.dv)
    return out


def _ctx(F, g, precision=0, nspin=2, cplx=True):
    return F.Context(g, np.zeros(g.ngrid), nspin=nspin, is_complex=cplx, precision=precision)


def _relmax(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("name", list(GRIDS))
def test_bse_potentials_match_oracle(fbse, cuda, name):
    g = GRIDS[name]
    ctx = _ctx(fbse, g)
    eps = (6.1, 5.3, 7.2)
    bare, scr = ctx.bse_potentials(*O.bse_axes(g), g.xmin, g.ymin, g.zmin, eps)
    rb, rs = O.bse_potentials(g, eps)
    assert _relmax(bare.cpu().numpy(), rb) < 1e-12
    assert _relmax(scr.cpu().numpy(), rs) < 1e-12


def _setup(fbse, cuda, name, nh, ne, gap, precision=0, seed=7):
    import torch
    g = GRIDS[name]
    ctx = _ctx(fbse, g, precision)
    lumo = nh + gap
    psi = qp_states(g, lumo + ne, seed)
    bare, scr = ctx.bse_potentials(*O.bse_axes(g), g.xmin, g.ymin, g.zmin, (6.1, 6.1, 6.1))
    psi_d = torch.tensor(psi, device=cuda)
    return g, ctx, lumo, psi, psi_d, bare, scr


@pytest.mark.parametrize("name,nh,ne,gap", [("cubic24", 3, 4, 1), ("odd21x20x18", 4, 2, 0), ("ymin_smallest", 2, 3, 2),
                                            ("cubic64", 2, 2, 0)])
def test_bse_kernel_fp64_matches_oracle(fbse, cuda, name, nh, ne, gap):
    g, ctx, lumo, psi, psi_d, bare, scr = _setup(fbse, cuda, name, nh, ne, gap)
    D, X = ctx.bse_kernel(psi_d, nh, ne, lumo, bare, scr)
    rD, rX = O.bse_kernels(psi, nh, ne, lumo, bare.cpu().numpy(), scr.cpu().numpy(), g)
    D, X = D.cpu().numpy(), X.cpu().numpy()
    assert _relmax(D, rD) < 1e-10
    assert _relmax(X, rX) < 1e-10
    iu = np.triu_indices(nh * ne, 1)
    assert np.all(D[iu] == 0) and np.all(X[iu] == 0)


# the mixed path contracts on the tensor cores (split-TF32, tcgemm.cu); 12 x 12
# pairs span two 128-row tiles of the tensor-core GEMM
@pytest.mark.parametrize("name,nh,ne", [("cubic24", 3, 4), ("cubic64", 3, 4), ("cubic24", 12, 12)])
def test_bse_kernel_mixed_within_tolerance(fbse, cuda, name, nh, ne):
    g, ctx, lumo, psi, psi_d, bare, scr = _setup(fbse, cuda, name, nh, ne, 1, precision=1)
    D, X = ctx.bse_kernel(psi_d, nh, ne, lumo, bare, scr)
    rD, rX = O.bse_kernels(psi, nh, ne, lumo, bare.cpu().numpy(), scr.cpu().numpy(), g)
    assert _relmax(D.cpu().numpy(), rD) < 3e-5
    assert _relmax(X.cpu().numpy(), rX) < 3e-5


def test_bse_solve_matches_oracle(fbse, cuda):
    nh, ne, gap = 3, 4, 1
    g, ctx, lumo, psi, psi_d, bare, scr = _setup(fbse, cuda, "cubic24", nh, ne, gap)
    rng = np.random.default_rng(3)
    evq = np.sort(np.concatenate([rng.uniform(-0.4, -0.25, lumo), rng.uniform(-0.12, 0.0, ne)]))
    D, X = ctx.bse_kernel(psi_d, nh, ne, lumo, bare, scr)
    rD, rX = D.cpu().numpy().copy(), X.cpu().numpy().copy()
    e, C, h, d, x, h0 = ctx.bse_solve(evq, nh, ne, lumo, D, X)
    re, rC, rh, rd, rx, rh0 = O.bse_solve(evq, nh, ne, lumo, rD, rX)
    assert np.max(np.abs(e - re)) < 1e-11
    for a, b in ((h, rh), (d, rd), (x, rx), (h0, rh0)):
        assert np.max(np.abs(a - b)) < 1e-10
    # completed Hermitian kernels (build_BSE_mat's fill)
    Df = D.cpu().numpy()
    assert np.max(np.abs(Df - Df.conj().T)) == 0
    # eigenvectors, up to phase, for non-degenerate excitons
    C = C.cpu().numpy()
    gaps = np.minimum(np.diff(re, prepend=-np.inf), np.diff(re, append=np.inf))
    ov = np.abs(np.sum(np.conj(rC) * C, axis=0))
    assert np.all(np.abs(ov[gaps > 1e-6] - 1) < 1e-9)
    # orthonormal columns
    assert np.max(np.abs(C.conj().T @ C - np.eye(nh * ne))) < 1e-12


def test_bse_dipoles_match_oracle(fbse, cuda):
    nh, ne, gap = 3, 4, 1
    g, ctx, lumo, psi, psi_d, bare, scr = _setup(fbse, cuda, "odd21x20x18", nh, ne, gap)
    mu = ctx.bse_dipoles(psi_d, *O.bse_axes(g), nh, ne, lumo)
    ref = O.bse_dipoles(psi, nh, ne, lumo, g)
    assert _relmax(mu, ref) < 1e-12


@pytest.mark.parametrize("name,precision,tol", [("odd21x20x18", 0, 1e-12), ("cubic24", 0, 1e-12), ("cubic24", 1, 3e-5)])
def test_bse_kernel_real_matches_oracle(fbse, cuda, name, precision, tol):
    """bse_real: real one-component states, real kernels, exchange x 2."""
    import torch
    nh, ne, gap = 3, 3, 1
    g = GRIDS[name]
    ctx = _ctx(fbse, g, precision, nspin=1, cplx=False)
    lumo = nh + gap
    psi = qp_states(g, lumo + ne, 11, nspin=1).real.copy()
    psi /= np.sqrt(np.sum(psi ** 2, axis=1) * g.dv)[:, None]
    bare, scr = ctx.bse_potentials(*O.bse_axes(g), g.xmin, g.ymin, g.zmin, (5.0, 5.0, 5.0))
    D, X = ctx.bse_kernel_real(torch.tensor(psi, device=cuda), nh, ne, lumo, bare, scr)
    rD, rX = O.bse_kernels_real(psi, nh, ne, lumo, bare.cpu().numpy(), scr.cpu().numpy(), g)
    assert _relmax(D.cpu().numpy(), rD) < tol
    assert _relmax(X.cpu().numpy(), rX) < tol
    # the complex kernel on the same states as complex spinless states: same
    # direct, half the exchange (no singlet factor)
    if precision == 0:
        cctx = _ctx(fbse, g, 0, nspin=1, cplx=True)
        Dc, Xc = cctx.bse_kernel(torch.tensor(psi.astype(np.complex128), device=cuda), nh, ne, lumo, bare, scr)
        assert _relmax(Dc.cpu().numpy().real, rD) < 1e-12 and _relmax(2 * Xc.cpu().numpy().real, rX) < 1e-12


@pytest.mark.parametrize("name", ["odd21x20x18", "cubic24"])
def test_bse_mag_dipoles_match_oracle(fbse, cuda, name):
    """calc_mag_dipole: p by FFT (init_kvec's k, Nyquist negative), L = -(r x p)."""
    nh, ne, gap = 3, 4, 1
    g, ctx, lumo, psi, psi_d, bare, scr = _setup(fbse, cuda, name, nh, ne, gap)
    m = ctx.bse_mag_dipoles(psi_d, *O.bse_axes(g), nh, ne, lumo)
    ref = O.bse_mag_dipoles(psi, nh, ne, lumo, g)
    assert _relmax(m, ref) < 1e-12


def test_bse_qp_ang_mom_matches_oracle(fbse, cuda):
    """calc_qp_spin_mtrx / calc_qp_ang_mom_mtrx: spin, L, L^2 and L.S matrices
    of both blocks with the reference's per-block conventions."""
    nh, ne, gap = 3, 2, 1
    g, ctx, lumo, psi, psi_d, bare, scr = _setup(fbse, cuda, "odd21x20x18", nh, ne, gap)
    got = ctx.bse_qp_ang_mom(psi_d, *O.bse_axes(g), nh, ne, lumo)
    want = O.bse_qp_ang_mom(psi, nh, ne, lumo, g)
    for a, b in zip(got, want):
        assert _relmax(a, b) < 1e-11
    # Hermitian blocks (spins, L, L^2, L.S)
    for m in (got[0][:, 0], got[1][:, 2], got[2], got[3]):
        for off, n in ((0, nh), (nh * nh, ne)):
            M = m[off:off + n * n].reshape(n, n)
            assert np.max(np.abs(M - M.conj().T)) < 1e-10 * max(1.0, np.max(np.abs(M)))


def test_bse_optical_matches_oracle(fbse, cuda):
    nh, ne, gap = 3, 4, 1
    g, ctx, lumo, psi, psi_d, bare, scr = _setup(fbse, cuda, "cubic24", nh, ne, gap)
    evq = np.linspace(-0.4, 0.0, lumo + ne)
    D, X = ctx.bse_kernel(psi_d, nh, ne, lumo, bare, scr)
    e, C, *_ = ctx.bse_solve(evq, nh, ne, lumo, D, X)
    mu = ctx.bse_dipoles(psi_d, *O.bse_axes(g), nh, ne, lumo)
    mx = ctx.bse_optical(C, mu, nh, ne)
    ref = O.bse_optical(C.cpu().numpy(), mu, nh, ne)
    assert _relmax(mx, ref) < 1e-13


def test_bse_argument_errors(fbse, cuda):
    import torch
    g = GRIDS["cubic24"]
    ctx = _ctx(fbse, g)
    psi = torch.zeros((4, 2 * g.ngrid), dtype=torch.complex128, device=cuda)
    bare = torch.zeros(g.ngrid, dtype=torch.complex128, device=cuda)
    with pytest.raises(fbse.FbseError, match="bad arguments"):
        ctx.bse_kernel(psi, 3, 1, 2, bare, bare)  # lumo_idx < n_h
    rctx = _ctx(fbse, g, nspin=1, cplx=False)
    with pytest.raises(fbse.FbseError, match="complex"):
        rctx.bse_kernel(psi, 2, 1, 2, bare, bare)


def test_bse_kernel_mixed_k_chunked(fbse, cuda):
    """The tensor-core contraction in several K chunks (a 30 MB image budget
    forces 5 chunks here) gives the same kernels as in one."""
    g, ctx, lumo, psi, psi_d, bare, scr = _setup(fbse, cuda, "cubic24", 3, 4, 1, precision=1)
    D1, X1 = ctx.bse_kernel(psi_d, 3, 4, lumo, bare, scr)
    ctx.set_tuning(tc_image_bytes=3.0e7)
    D2, X2 = ctx.bse_kernel(psi_d, 3, 4, lumo, bare, scr)
    rD, rX = O.bse_kernels(psi, 3, 4, lumo, bare.cpu().numpy(), scr.cpu().numpy(), g)
    assert _relmax(D2.cpu().numpy(), rD) < 3e-5 and _relmax(X2.cpu().numpy(), rX) < 3e-5
    assert _relmax(D2.cpu().numpy(), D1.cpu().numpy()) < 1e-5
