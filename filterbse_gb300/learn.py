"""Training data, training loop and refinement driver of the learned residual
preconditioner (fbse_precond_* / fbse_refine in include/fbse.h).

The reference has no counterpart: when states stay above its sigma cut it
filters again with more starts and Newton terms (retryFilter,
filter_mpi/mod_output.c:131-147).  Here the filter itself generates the
training pairs: a short filter run gives Ritz pairs (psi, E) with residuals
r = (H - E) psi; a longer run on the same starts -- the plain method with more
Newton terms, which is also the judge of the refined energies -- gives
converged eigenvectors.  The target correction of psi is the step to its
projection on the longer run's Ritz vectors near its energy:
    c = Q Q^H psi / |Q^H psi| - psi,
Q those Ritz vectors (energies within a window of E, small residuals).
Every product runs in the library on the GPU (fbse_gram, fbse_rotate,
fbse_hpsi); this module only moves pointers and picks clusters.
"""
from __future__ import annotations

import numpy as np

from . import Context, Precond

SIGMA_CONVERGED = 1e-5  # judge pairs that define the eigenspaces


def clusters(e, tol=1e-6):
    """Index groups of sorted energies closer than tol to their neighbour."""
    order = np.argsort(e)
    out, cur = [], [order[0]]
    for a, b in zip(order[:-1], order[1:]):
        if e[b] - e[a] < tol:
            cur.append(b)
        else:
            out.append(cur)
            cur = [b]
    out.append(cur)
    return out


def ritz(ctx: Context, zn, an, vmin, de, starts):
    """Newton filter + Rayleigh-Ritz of all starts: (psitot [n, stlen] device
    with the n Ritz vectors in the first rows, eval, sigma)."""
    filt = ctx.newton_filter(zn, an, vmin, de, starts)
    psitot = filt.reshape(-1, ctx.stlen)
    nk, ev, sg = ctx.ortho_diag_sigma(psitot)
    return psitot, nk, ev, sg


def residuals(ctx: Context, psitot, ev):
    """r_i = H psi_i - E_i psi_i of psitot rows (fbse_residual)."""
    return ctx.residual(psitot.contiguous(), np.asarray(ev, np.float64)[:psitot.shape[0]])


def training_pairs(short, judge, tol_lo=1e-5, tol_hi=0.1, window=0.02, judge_sigma=1e-3, min_weight=0.5):
    """(resid, corr, ene) of the short run's Ritz pairs with tol_lo < sigma <=
    tol_hi.  The target of pair (psi, E) is the step to its projection on the
    judge's Ritz vectors with energies within `window` of E and sigma <=
    judge_sigma, normalised: c = Q Q^H psi / |Q^H psi| - psi; pairs with less
    than min_weight of their norm in that span are left out.  short, judge:
    (ctx, psitot, n, ev, sg); the judge's ctx is FP64."""
    import torch
    ctx, ps, n, ev, sg = short
    jctx, pj, nj, evj, sgj = judge
    good = np.where(sgj[:nj] <= judge_sigma)[0]
    sel = [i for i in range(n) if tol_lo < sg[i] <= tol_hi]
    if len(good) == 0 or not sel:
        return None
    Q = pj[good].contiguous()
    ov = jctx.gram(Q, ps[sel].contiguous())  # [ngood, nsel], one FP64 product on the GPU
    keep, coef = [], []
    for col, i in enumerate(sel):
        near = np.abs(evj[good] - ev[i]) <= window
        w = float(np.sum(np.abs(ov[near, col]) ** 2))
        if w < min_weight:
            continue
        cf = np.where(near, ov[:, col], 0.0) / np.sqrt(w)
        keep.append(i)
        coef.append(cf)
    if not keep:
        return None
    tgt = torch.empty((len(keep), ctx.stlen), dtype=torch.float64, device=ps.device)
    jctx.rotate(Q, np.array(coef).T, tgt)
    psi = ps[keep].contiguous()
    corr = (tgt - psi).contiguous()
    res = residuals(jctx, psi, ev[keep])
    # only the direction of a correction matters to the Rayleigh-Ritz step that
    # uses it, and |c| / |r| spans orders of magnitude (about 1 / |E_k - E|):
    # every target is scaled to its residual's norm, so the network learns
    # directions and the loss weighs every pair alike
    scale = (res.norm(dim=1) / corr.norm(dim=1).clamp_min(1e-300))[:, None]
    corr = (corr * scale).contiguous()
    return res, corr, np.asarray(ev)[keep]


def train(pc: Precond, pairs, steps=200, lr=2e-3, batch=8, seed=0, log=None):
    """Adam on the pairs (mini-batches of `batch` states, reshuffled per
    epoch with a seeded generator); returns the loss history."""
    import torch
    res, corr, ene = pairs
    n = res.shape[0]
    rng = np.random.default_rng(seed)
    hist = []
    order = rng.permutation(n)
    pos = 0
    for s in range(steps):
        if pos + batch > n:
            order = rng.permutation(n)
            pos = 0
        idx = torch.tensor(order[pos:pos + batch], device=res.device)
        pos += batch
        loss = pc.train_step(res[idx].contiguous(), corr[idx].contiguous(), ene[order[pos - batch:pos]], lr)
        hist.append(loss)
        if log and s % 50 == 0:
            log(f"[train] step {s} loss {loss:.4e}")
    return hist


def match(ev, sg, ref, tol=1e-5, cut=1e-2):
    """Pairs with sigma <= cut matched one-to-one to reference levels within tol."""
    ref = np.sort(ref)
    mine = np.sort(ev[sg <= cut])
    i = j = good = 0
    while i < len(mine) and j < len(ref):
        if ref[j] < mine[i] - tol:
            j += 1
        elif ref[j] <= mine[i] + tol:
            good += 1
            i += 1
            j += 1
        else:
            i += 1
    return good
