"""CPU restatement of the library's learned residual preconditioner (test
infrastructure only: imported by tests/, never by the library).

The network has no counterpart in the reference (its only remedy for
unconverged states is retryFilter, filter_mpi/mod_output.c:131-147); this file
restates the library's own definition in numpy so that the GPU forward and
backward kernels can be checked against it:

  per real field f of a residual (state-major, then spin block, then real /
  imaginary part), x0 = [f / rms(f), f / rms(f) * (V - E) / 1 Ha] rounded to
  BF16; a_l = BF16(tanh(W_l * a_{l-1})) for l = 1..3; y = W_4 * a_3 (FP32);
  correction = f + y * rms(f) (a residual connection).  "*" is a 3x3x3
  convolution with zero padding and no bias; W_l has the layout
  [c_out][c_in][27], k = (dz * 3 + dy) * 3 + dx.

The loss is the mean over all fields and points of (correction - corr)^2 / rms^2,
i.e. of (y - (corr - f) / rms)^2.
Arithmetic here is FP64 with the BF16 rounding of the stored activations
applied where the GPU stores them, so the two agree to FP32 summation-order
differences except where an FP32 and an FP64 value round to neighbouring BF16
numbers.
"""
import numpy as np

C = 16
CIN = (2, C, C, C)
COUT = (C, C, C, 1)
OFFS = np.cumsum([0] + [CIN[l] * COUT[l] * 27 for l in range(4)])
NWEIGHTS = int(OFFS[-1])
VSCALE = 1.0


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def layers(w):
    return [np.asarray(w[OFFS[l]:OFFS[l + 1]], np.float64).reshape(COUT[l], CIN[l], 27) for l in range(4)]


def conv(x, w):
    """y[o] = sum_c sum_k w[o, c, k] x[c](p + off_k); x [cin, nz, ny, nx]."""
    cin, nz, ny, nx = x.shape
    xp = np.zeros((cin, nz + 2, ny + 2, nx + 2))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    y = np.zeros((w.shape[0], nz, ny, nx))
    for k in range(27):
        dz, dy, dx = k // 9, (k // 3) % 3, k % 3
        y += np.einsum("oc,czyx->ozyx", w[:, :, k], xp[:, dz:dz + nz, dy:dy + ny, dx:dx + nx])
    return y


def conv_wgrad(x, dy):
    """dW[o, c, k] = sum_p dy[o](p) x[c](p + off_k)."""
    cin, nz, ny, nx = x.shape
    xp = np.zeros((cin, nz + 2, ny + 2, nx + 2))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    g = np.zeros((dy.shape[0], cin, 27))
    for k in range(27):
        dz, dyy, dx = k // 9, (k // 3) % 3, k % 3
        g[:, :, k] = np.einsum("ozyx,czyx->oc", dy, xp[:, dz:dz + nz, dyy:dyy + ny, dx:dx + nx])
    return g


def conv_dgrad(dy, w):
    """dx[c](q) = sum_o sum_k w[o, c, k] dy[o](q - off_k)."""
    o, nz, ny, nx = dy.shape
    dp = np.zeros((o, nz + 2, ny + 2, nx + 2))
    dp[:, 1:-1, 1:-1, 1:-1] = dy
    dx_ = np.zeros((w.shape[1], nz, ny, nx))
    for k in range(27):
        dz, dyy, dxx = k // 9, (k // 3) % 3, k % 3
        # q = p + off_k - 1  =>  p = q - (off_k - 1)
        sz, sy, sx = 2 - dz, 2 - dyy, 2 - dxx
        dx_ += np.einsum("oc,ozyx->czyx", w[:, :, k], dp[:, sz:sz + nz, sy:sy + ny, sx:sx + nx])
    return dx_


def fields(psitot, nspin, cplx, shape):
    """The real fields of n psitot states (FP64 rows), [nf, nz, ny, nx]."""
    nz, ny, nx = shape
    N = nx * ny * nz
    out = []
    for row in psitot:
        for s in range(nspin):
            if cplx:
                blk = row[2 * s * N:2 * (s + 1) * N]
                out.append(blk[0::2].reshape(nz, ny, nx))
                out.append(blk[1::2].reshape(nz, ny, nx))
            else:
                out.append(row[s * N:(s + 1) * N].reshape(nz, ny, nx))
    return np.array(out)


def unfields(f, nspin, cplx):
    """Inverse of fields: [nf, nz, ny, nx] -> psitot rows."""
    fps = nspin * (2 if cplx else 1)
    n = f.shape[0] // fps
    N = f[0].size
    rows = []
    for i in range(n):
        parts = []
        for s in range(nspin):
            if cplx:
                b = np.empty(2 * N)
                b[0::2] = f[i * fps + 2 * s].reshape(-1)
                b[1::2] = f[i * fps + 2 * s + 1].reshape(-1)
                parts.append(b)
            else:
                parts.append(f[i * fps + s].reshape(-1))
        rows.append(np.concatenate(parts))
    return np.array(rows)


def forward(w, resid, ene, pot, nspin, cplx, shape, round_bf16=True):
    """Returns (y [nf, grid], rms [nf], activations) for n residual rows."""
    W = layers(w)
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, np.float64))
    f = fields(resid, nspin, cplx, shape)
    fps = nspin * (2 if cplx else 1)
    rms = np.sqrt(np.mean(f.reshape(len(f), -1) ** 2, axis=1))
    v = pot.reshape(shape)
    ys, acts = [], []
    for i in range(len(f)):
        fh = f[i] / rms[i] if rms[i] > 0 else np.zeros_like(f[i])
        x0 = r(np.stack([fh, fh * (v - ene[i // fps]) / VSCALE]))
        a1 = r(np.tanh(conv(x0, W[0])))
        a2 = r(np.tanh(conv(a1, W[1])))
        a3 = r(np.tanh(conv(a2, W[2])))
        y = conv(a3, W[3])[0]
        ys.append(y)
        acts.append((x0, a1, a2, a3))
    return np.array(ys), rms, acts


def apply(w, resid, ene, pot, nspin, cplx, shape):
    y, rms, _ = forward(w, resid, ene, pot, nspin, cplx, shape)
    return np.asarray(resid, np.float64) + unfields(y * rms[:, None, None, None], nspin, cplx)


def loss_grad(w, resid, corr, ene, pot, nspin, cplx, shape, round_bf16=True):
    """(loss, gradient [NWEIGHTS]) of mean (y - (corr - resid) / rms)^2."""
    W = layers(w)
    y, rms, acts = forward(w, resid, ene, pot, nspin, cplx, shape, round_bf16)
    d = np.asarray(corr, np.float64) - np.asarray(resid, np.float64)
    t = fields(d, nspin, cplx, shape) / np.where(rms > 0, rms, np.inf)[:, None, None, None]
    M = y.size
    loss = float(np.sum((y - t) ** 2) / M)
    g = [np.zeros_like(Wl) for Wl in W]
    for i in range(len(y)):
        x0, a1, a2, a3 = acts[i]
        d4 = (2.0 / M) * (y[i] - t[i])[None]
        g[3] += conv_wgrad(a3, d4)
        d3 = conv_dgrad(d4, W[3]) * (1 - a3 ** 2)
        g[2] += conv_wgrad(a2, d3)
        d2 = conv_dgrad(d3, W[2]) * (1 - a2 ** 2)
        g[1] += conv_wgrad(a1, d2)
        d1 = conv_dgrad(d2, W[1]) * (1 - a1 ** 2)
        g[0] += conv_wgrad(x0, d1)
    return loss, np.concatenate([gl.reshape(-1) for gl in g])
