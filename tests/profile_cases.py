"""Small GPU programs whose kernels the per-kernel ncu summaries under
profiles/ profile (pytest does not collect this file).  Each case builds its
workload, runs it once to warm up (autotuner decisions, buffers) and then once
more, so that a capture with `-s <launches of the warm-up>` sees the second
run.  The cases are sized to hold a few GB on the device.  It needs a GPU and
the built library.

  python tests/profile_cases.py rr        Rayleigh-Ritz of 64 filtered spinor states of
                                          a 2 nm CdSe dot, 96^3 (k_gram, k_jacobi_sweep,
                                          k_rotate, k_quad_diag)
  python tests/profile_cases.py filter    Newton filter of 8 spinor starts x 16 targets,
                                          nCheby 256, 2 nm dot, 32-slot ring (k_newton_acc)
  python tests/profile_cases.py bse       BSE kernel of 16 hole x 16 electron spinor states
                                          of the 2 nm dot, mixed path (k_pair_density,
                                          convolution FFTs, k_tc_images, k_tc_gemm_nt)
  python tests/profile_cases.py precond   learned preconditioner on 8 spinor residuals of a
                                          1.6 nm dot, 80^3: inference (k_conv, k_conv16_tc)
                                          and one gradient (k_conv, k_conv_wgrad)
  python tests/profile_cases.py step      one mixed step of the benchmark workload (3 nm dot,
                                          128^3, 16 starts x 16 targets, nCheby 2048: Newton
                                          filter + Rayleigh-Ritz), the second one inside the
                                          NVTX range "fbse_timed_steps" (a launch list selects
                                          it with --nvtx --nvtx-include "fbse_timed_steps/")
  python tests/profile_cases.py angular   spin / angular statistics of 8 random spinors of the
                                          3 nm dot, 128^3 (k_ang_sums and the FP64 FFT passes)
  python tests/profile_cases.py setup     local potential and projector table of the 3 nm dot,
                                          128^3 (k_local_pot, k_nlc_count, k_nlc_fill)
"""
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def _dot(radius):
    from filterbse_gb300 import workload as W
    return W.cdse_dot(radius, d=0.5, ke_max=10.0, spinor=True)


def _ctx(F, dot, prec, ring=0):
    g = dot.grid
    c = F.Context(g, dot.pot, nspin=2, is_complex=True, so=True, nl=False, proj=dot.proj, precision=prec)
    if ring:
        c.set_tuning(newton_ring=ring)
    return c


def _filter_setup(F, dot, ctx, nc, nstart):
    import torch
    import bench as B
    g = dot.grid
    e0, e1, _ = ctx.energy_range(max_iter=400)
    vmin, emax = e0 - 0.2 * abs(e0), e1 * 1.2
    de = emax - vmin
    zn, _ = F.samp_points(nc)
    an = F.newton_coeff(zn, B.ene_targets(**B.TARGETS), vmin, de, (nc / (2.5 * de)) ** 2)
    starts, _, _ = F.init_filter_states(nstart, g.ngrid, 2, True, g.dv, -(B.SEED))
    return zn, an, vmin, de, torch.tensor(starts, device="cuda:0")


def case_filter(F):
    dot = _dot(10.0)
    ctx = _ctx(F, dot, F.MIXED, ring=32)
    zn, an, vmin, de, d0 = _filter_setup(F, dot, ctx, 256, 8)
    for _ in range(2):
        t = time.time()
        ctx.newton_filter(zn, an, vmin, de, d0)
        print(f"filter: {time.time() - t:.3f}s")


def case_rr(F):
    import torch
    dot = _dot(10.0)
    ctx = _ctx(F, dot, F.MIXED, ring=32)
    zn, an, vmin, de, d0 = _filter_setup(F, dot, ctx, 256, 4)
    filt = ctx.newton_filter(zn, an, vmin, de, d0).reshape(64, -1)
    for _ in range(2):
        t = torch.clone(filt)
        t0 = time.time()
        nk, ev, sg = ctx.ortho_diag_sigma(t)
        print(f"rayleigh-ritz: {nk} pairs, {time.time() - t0:.3f}s")


def case_bse(F):
    import torch
    dot = _dot(10.0)
    ctx = _ctx(F, dot, F.MIXED)
    g = dot.grid
    nh = ne = 16
    gen = torch.Generator(device="cuda:0").manual_seed(1)
    pd = torch.randn((nh + ne, 2 * g.ngrid), dtype=torch.complex128, device="cuda:0", generator=gen)
    pd /= torch.sqrt((pd.abs() ** 2).sum(dim=1, keepdim=True) * g.dv)
    gx, gy, gz = g.axes()
    bare, scr = ctx.bse_potentials(gx, gy, gz, g.xmin, g.ymin, g.zmin)
    for _ in range(2):
        t = time.time()
        ctx.bse_kernel(pd, nh, ne, nh, bare, scr)
        torch.cuda.synchronize()
        print(f"bse kernel {nh}h x {ne}e: {time.time() - t:.3f}s")


def case_precond(F):
    import torch
    dot = _dot(8.0)
    ctx = _ctx(F, dot, F.MIXED)
    rng = np.random.default_rng(2)
    n = 8
    r = torch.tensor(rng.normal(size=(n, ctx.stlen)), device="cuda:0")
    c = torch.tensor(rng.normal(size=(n, ctx.stlen)) * 0.1, device="cuda:0")
    e = rng.uniform(-0.3, -0.1, n)
    pc = F.Precond(ctx, seed=3)
    for _ in range(2):
        torch.cuda.synchronize()
        t = time.time()
        pc.apply(r, e)
        torch.cuda.synchronize()
        t1 = time.time()
        pc.grad(r, c, e)
        print(f"precond inference {t1 - t:.3f}s, forward + gradient {time.time() - t1:.3f}s ({n} states)")


def case_step(F):
    import torch
    dot = _dot(15.0)
    ctx = _ctx(F, dot, F.MIXED)
    zn, an, vmin, de, d0 = _filter_setup(F, dot, ctx, 2048, 16)
    ext = torch.cuda.ExternalStream(ctx.stream_handle)
    for it in range(2):
        if it:
            torch.cuda.nvtx.range_push("fbse_timed_steps")
        l0 = F.launch_count()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(ext)
        filt = ctx.newton_filter(zn, an, vmin, de, d0)
        nk, ev, sg = ctx.ortho_diag_sigma(filt.reshape(256, -1))
        b.record(ext)
        b.synchronize()
        if it:
            torch.cuda.nvtx.range_pop()
        print(f"step: {a.elapsed_time(b):.1f} ms, {F.launch_count() - l0} launches, {nk} Ritz pairs")


def case_angular(F):
    import torch
    dot = _dot(15.0)
    ctx = _ctx(F, dot, F.FP64)
    g = dot.grid
    gen = torch.Generator(device="cuda:0").manual_seed(4)
    st = torch.randn((8, 4 * g.ngrid), dtype=torch.float64, device="cuda:0", generator=gen)
    for _ in range(2):
        torch.cuda.synchronize()
        t = time.time()
        ctx.angular_stats(st, *g.axes())
        print(f"angular statistics of 8 states: {time.time() - t:.3f}s")


def case_setup(F):
    for _ in range(2):
        t = time.time()
        dot = _dot(15.0)  # builds the local potential and the projector table on the GPU
        print(f"setup of the 3 nm dot: {time.time() - t:.3f}s, {int(np.sum(dot.proj.nl))} table entries")


def main():
    import filterbse_gb300 as F
    F.load()
    {"rr": case_rr, "filter": case_filter, "bse": case_bse, "precond": case_precond, "step": case_step,
     "angular": case_angular, "setup": case_setup}[sys.argv[1]](F)


if __name__ == "__main__":
    main()
