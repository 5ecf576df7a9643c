"""H psi on the GPU against the FP64 oracle (kinetic FFT, local potential,
spin-orbit and nonlocal projectors, p_hnorm), in FP64 and in the mixed (FP32)
working precision, on grids whose axis lengths exercise every FFT radix path
(2, 3, 4, odd primes 5, 7, 11, 13, 19 and a prime axis)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.systems import random_states, tiny_cluster

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 3e-6}  # relative max-norm error: FP64 path, mixed (FP32) path


def _ctx(F, sysm, precision):
    return F.Context(sysm.grid, sysm.pot, nspin=sysm.nspin, is_complex=sysm.is_complex, so=sysm.so, nl=sysm.nlflag,
                     proj=sysm.proj, precision=precision)


def _run_hpsi(F, ctx, psis, dev):
    import torch
    dt = ctx.working_dtype()
    x = torch.tensor(psis, dtype=dt, device=dev).contiguous()
    y = torch.empty_like(x)
    ctx.hpsi(x, y)
    return y.cpu().numpy().astype(np.complex128)


def _relerr(a, b, real_only=False):
    if real_only:
        a, b = a.real, b.real
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


# the last five shapes take the register-resident kernels (axes of 64, 128, 256):
# square planes of 64 / 128, non-square planes (line path), a 256-point z axis
# and a fast plane with a mixed-radix z axis
@pytest.mark.parametrize("shape", [(16, 16, 16), (24, 21, 22), (20, 26, 15), (19, 14, 33), (57, 52, 45), (13, 28, 17),
                                   (64, 64, 64), (128, 128, 64), (128, 64, 64), (64, 64, 256), (64, 64, 48)])
@pytest.mark.parametrize("precision", [0, 1])
def test_kinetic_and_local(fbse, cuda, shape, precision):
    nx, ny, nz = shape
    sysm = tiny_cluster(nx, ny, nz, natoms=6, is_complex=True)
    rng = np.random.default_rng(1)
    psis = random_states(3, sysm, rng)
    ctx = _ctx(fbse, sysm, precision)
    got = _run_hpsi(fbse, ctx, psis, cuda)
    want = np.array([O.hamiltonian(p, sysm) for p in psis])
    assert _relerr(got, want) < TOL[precision]


@pytest.mark.parametrize("precision", [0, 1])
def test_kinetic_plane_wave(fbse, cuda, precision):
    """A plane wave is an eigenvector of the kinetic operator with 0.5 k^2 (capped)."""
    sysm = tiny_cluster(18, 20, 15, natoms=1, is_complex=True)
    sysm.pot[:] = 0.0
    g = sysm.grid
    dkx, dky, dkz = g.dk()
    x = np.arange(g.nx)[None, None, :]
    y = np.arange(g.ny)[None, :, None]
    z = np.arange(g.nz)[:, None, None]
    kx, ky, kz = 3, -2, 5
    pw = np.exp(2j * np.pi * (kx * x / g.nx + ky * y / g.ny + kz * z / g.nz)).reshape(1, -1)
    ctx = _ctx(fbse, sysm, precision)
    got = _run_hpsi(fbse, ctx, pw, cuda)
    e = 0.5 * ((kx * dkx) ** 2 + (ky * dky) ** 2 + (kz * dkz) ** 2)
    e = min(e, g.ke_max)
    assert _relerr(got, e * pw) < TOL[precision] * 10


@pytest.mark.parametrize("precision", [0, 1])
def test_real_packing(fbse, cuda, precision):
    """Real jobs: two real states packed as re/im give each real H psi."""
    sysm = tiny_cluster(22, 18, 20, natoms=8, is_complex=False, nl=True)
    rng = np.random.default_rng(2)
    a = rng.uniform(-1, 1, (2, sysm.ngrid))
    packed = (a[0] + 1j * a[1]).reshape(1, -1)
    ctx = _ctx(fbse, sysm, precision)
    got = _run_hpsi(fbse, ctx, packed, cuda)[0]
    w0 = O.hamiltonian(a[0].astype(np.complex128), sysm).real
    w1 = O.hamiltonian(a[1].astype(np.complex128), sysm).real
    scale = max(np.abs(w0).max(), np.abs(w1).max())
    assert np.max(np.abs(got.real - w0)) / scale < TOL[precision]
    assert np.max(np.abs(got.imag - w1)) / scale < TOL[precision]


@pytest.mark.parametrize("so,nl", [(True, False), (False, True), (True, True)])
@pytest.mark.parametrize("precision", [0, 1])
def test_projectors_spinor(fbse, cuda, so, nl, precision):
    sysm = tiny_cluster(24, 22, 20, natoms=10, nspin=2, is_complex=True, so=so, nl=nl)
    rng = np.random.default_rng(3)
    psis = random_states(2, sysm, rng)
    ctx = _ctx(fbse, sysm, precision)
    got = _run_hpsi(fbse, ctx, psis, cuda)
    want = np.array([O.hamiltonian(p, sysm) for p in psis])
    assert _relerr(got, want) < TOL[precision]


@pytest.mark.parametrize("precision", [0, 1])
def test_hnorm(fbse, cuda, precision):
    import torch
    sysm = tiny_cluster(20, 20, 21, natoms=8, nspin=2, is_complex=True, so=True, nl=True)
    rng = np.random.default_rng(4)
    psis = random_states(2, sysm, rng)
    vmin, de, zn = -1.3, 27.0, 0.37
    ctx = _ctx(fbse, sysm, precision)
    x = torch.tensor(psis, dtype=ctx.working_dtype(), device=cuda)
    y = torch.empty_like(x)
    ctx.hnorm(x, y, vmin, de, zn)
    got = y.cpu().numpy()
    want = np.array([O.hnorm(p, sysm, 4.0 / de, vmin, zn) for p in psis])
    assert _relerr(got, want) < TOL[precision]


@pytest.mark.parametrize("precision", [0, 1])
def test_determinism(fbse, cuda, precision):
    """H psi is bit-identical from run to run and for every batch size: the
    projector scatter sums each point's entries in a fixed order (no atomics),
    and every other kernel works per state.  Overlapping spheres (the 10 atoms
    of this cluster are nearest neighbours) make the scatter a reduction."""
    sysm = tiny_cluster(16, 18, 20, natoms=10, nspin=2, is_complex=True, so=True, nl=True)
    rng = np.random.default_rng(5)
    psis = random_states(9, sysm, rng)
    ctx = _ctx(fbse, sysm, precision)
    full = _run_hpsi(fbse, ctx, psis, cuda)
    again = _run_hpsi(fbse, ctx, psis, cuda)
    assert np.array_equal(full, again)
    for lo, hi in ((2, 3), (0, 4), (4, 9)):
        part = _run_hpsi(fbse, ctx, psis[lo:hi], cuda)
        assert np.array_equal(full[lo:hi], part), (lo, hi)


@pytest.mark.parametrize("precision", [0, 1])
def test_autotuner_choices_are_bit_identical(fbse, cuda, precision):
    """Every autotuned launch shape (FFT blocks per launch, projector gather
    points per lane, scatter states per thread) gives the same bits; the
    autotuner records its decisions with the candidates' times."""
    sysm = tiny_cluster(16, 18, 20, natoms=10, nspin=2, is_complex=True, so=True, nl=True)
    psis = random_states(9, sysm, np.random.default_rng(6))
    ctx = _ctx(fbse, sysm, precision)
    auto = _run_hpsi(fbse, ctx, psis, cuda)
    rep = ctx.tuning_report()
    kernels = {r["kernel"].split(" (")[0] for r in rep}
    assert {"fft blocks per launch", "projector gather points per lane",
            "projector scatter states per thread"} <= kernels
    for r in rep:
        assert str(r["choice"]) in r["candidates"] and all(t > 0 for t in r["candidates"].values())
    for fixed in ({"fft_chunk_blocks": 2, "scatter_states": 1, "gather_points": 1},
                  {"fft_chunk_blocks": 18, "scatter_states": 8, "gather_points": 4},
                  {"fft_chunk_blocks": 5, "scatter_states": 2, "gather_points": 2},
                  {"fft_chunk_blocks": 3, "scatter_states": 18, "gather_points": 2},
                  {"fft_chunk_blocks": 1, "scatter_states": 20, "gather_points": 1}):
        ctx.set_tuning(**fixed)
        assert np.array_equal(_run_hpsi(fbse, ctx, psis, cuda), auto), fixed
    with pytest.raises(fbse.FbseError):
        ctx.set_tuning(scatter_states=3)


@pytest.mark.parametrize("shape,precision", [((128, 128, 64), 1), ((64, 64, 64), 0), ((64, 64, 256), 1)])
def test_plane_variants_are_bit_identical(fbse, cuda, shape, precision):
    """The one-CTA and the two-CTA-cluster plane kernels run the same
    arithmetic (the FP32 128-point rows as two 64-point transforms in both):
    H psi is bit-identical between them and matches the oracle."""
    sysm = tiny_cluster(*shape, natoms=8, nspin=2, is_complex=True, so=True, nl=True)
    psis = random_states(3, sysm, np.random.default_rng(8))
    ctx = _ctx(fbse, sysm, precision)
    outs = []
    for var in (0, 1):
        ctx.set_tuning(fft_plane_cluster=var)
        outs.append(_run_hpsi(fbse, ctx, psis, cuda))
    assert np.array_equal(outs[0], outs[1])
    want = np.array([O.hamiltonian(p, sysm) for p in psis])
    assert _relerr(outs[0], want) < TOL[precision]


@pytest.mark.parametrize("shape,precision", [((128, 128, 64), 1), ((20, 18, 21), 0)])
def test_stream_parts_are_bit_identical(fbse, cuda, shape, precision):
    """H psi as 2, 3 or 4 parts of the batch on the context's streams gives the
    same bits as the whole batch on one stream, call after call."""
    sysm = tiny_cluster(*shape, natoms=10, nspin=2, is_complex=True, so=True, nl=True)
    psis = random_states(5, sysm, np.random.default_rng(9))
    ctx = _ctx(fbse, sysm, precision)
    two = [_run_hpsi(fbse, ctx, psis, cuda) for _ in range(2)]
    ctx.set_tuning(hpsi_streams=1)
    one = _run_hpsi(fbse, ctx, psis, cuda)
    assert np.array_equal(two[0], one) and np.array_equal(two[1], one)
    for parts in (3, 4):
        ctx.set_tuning(hpsi_streams=parts)
        assert np.array_equal(_run_hpsi(fbse, ctx, psis, cuda), one), parts
    want = np.array([O.hamiltonian(p, sysm) for p in psis])
    assert _relerr(one, want) < TOL[precision]
