"""The learned preconditioner's CPU restatement (oracle/cnn.py): its gradient
against central finite differences, the data gradient as the adjoint of the
convolution, the BF16 rounding, the field layout round trip, and the C-ABI
symbols of the GPU implementation (no GPU needed)."""
import numpy as np

from oracle import cnn


def _system(rng, shape=(4, 5, 6), nspin=2, cplx=True, n=1):
    N = int(np.prod(shape))
    stlen = (2 if cplx else 1) * nspin * N
    resid = rng.normal(size=(n, stlen))
    corr = rng.normal(size=(n, stlen)) * 0.3
    pot = rng.uniform(-1.0, 0.5, N)
    ene = rng.uniform(-0.4, -0.1, n)
    return resid, corr, pot, ene


def test_bf16_rounding():
    # BF16 keeps 7 fraction bits: the spacing at 1 is 2^-7
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -2.5, 0.0, 3.14159265])
    r = cnn.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # a tie rounds to the even neighbour ...
    assert r[2] == 1.0 + 2 ** -6  # ... in both directions
    assert r[3] == 1.0 and r[4] == 1.0 + 2 ** -7
    assert r[5] == -2.5 and r[6] == 0.0
    assert r[7] == 3.140625


def test_conv_dgrad_is_the_adjoint():
    rng = np.random.default_rng(1)
    x = rng.normal(size=(3, 4, 5, 6))
    w = rng.normal(size=(2, 3, 27))
    y = rng.normal(size=(2, 4, 5, 6))
    lhs = np.sum(cnn.conv(x, w) * y)
    rhs = np.sum(x * cnn.conv_dgrad(y, w))
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
    # and the weight gradient is d<conv(x, w), y>/dw
    g = cnn.conv_wgrad(x, y)
    k = (1, 2, 13)
    e = np.zeros_like(w)
    e[k] = 1e-6
    fd = (np.sum(cnn.conv(x, w + e) * y) - np.sum(cnn.conv(x, w - e) * y)) / 2e-6
    assert abs(fd - g[k]) < 1e-6 * max(1.0, abs(g[k]))


def test_fields_round_trip():
    rng = np.random.default_rng(2)
    for nspin, cplx in ((2, True), (1, False), (1, True)):
        resid, _, _, _ = _system(rng, nspin=nspin, cplx=cplx, n=3)
        f = cnn.fields(resid, nspin, cplx, (4, 5, 6))
        assert f.shape == (3 * nspin * (2 if cplx else 1), 4, 5, 6)
        assert np.array_equal(cnn.unfields(f, nspin, cplx), resid)


def test_gradient_matches_finite_differences():
    """FP64 without the BF16 rounding: the restated backward pass is the exact
    gradient of the restated loss."""
    rng = np.random.default_rng(3)
    resid, corr, pot, ene = _system(rng, shape=(4, 4, 5), n=1)
    w = rng.uniform(-0.4, 0.4, cnn.NWEIGHTS)
    loss, g = cnn.loss_grad(w, resid, corr, ene, pot, 2, True, (4, 4, 5), round_bf16=False)
    assert loss > 0
    for i in (0, 500, cnn.OFFS[1] + 7, cnn.OFFS[2] + 4000, cnn.OFFS[3] + 100, cnn.NWEIGHTS - 1):
        e = np.zeros_like(w)
        h = 1e-5
        e[i] = h
        lp, _ = cnn.loss_grad(w + e, resid, corr, ene, pot, 2, True, (4, 4, 5), round_bf16=False)
        lm, _ = cnn.loss_grad(w - e, resid, corr, ene, pot, 2, True, (4, 4, 5), round_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) < 1e-6 * max(1e-3, abs(g[i])) + 1e-9, (i, fd, g[i])


def test_network_is_odd_in_the_residual():
    rng = np.random.default_rng(4)
    resid, _, pot, ene = _system(rng, n=2)
    w = rng.uniform(-0.3, 0.3, cnn.NWEIGHTS)
    a = cnn.apply(w, resid, ene, pot, 2, True, (4, 5, 6))
    b = cnn.apply(w, -resid, ene, pot, 2, True, (4, 5, 6))
    assert np.array_equal(a, -b)
    # and positively homogeneous: scaling a residual scales its correction
    c = cnn.apply(w, 3.0 * resid, ene, pot, 2, True, (4, 5, 6))
    assert np.allclose(c, 3.0 * a, rtol=1e-12, atol=1e-14)


def test_abi_exports_the_preconditioner():
    import ctypes
    import filterbse_gb300 as F
    L = F.load()
    for name in ("fbse_precond_create", "fbse_precond_destroy", "fbse_precond_get_weights",
                 "fbse_precond_set_weights", "fbse_precond_apply", "fbse_precond_grad", "fbse_precond_train_step",
                 "fbse_refine"):
        assert hasattr(L, name)
    # arguments are checked before any device work
    assert L.fbse_precond_create(None, ctypes.byref(ctypes.c_void_p()), None, 1) == -1
    assert L.fbse_refine(None, None, None, 1, 1, 1, 0.0, None, None, None) == -1
    assert F.PRECOND_NWEIGHTS == cnn.NWEIGHTS
