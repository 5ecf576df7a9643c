"""Benchmark: converged eigenpairs/s of the filter-diagonalization stage on a
3 nm (radius 15 A) passivated zincblende CdSe dot with spin-orbit coupling
(complex two-component spinors, grid 128^3 at 0.5 bohr by the reference's
grid rule), 16 random starts x 16 energy targets, Newton length 2048.

One step = one pass of the hot path over one batch: Newton filter of all 16
starts + orthogonalisation + subspace diagonalisation + sigma_E, in the mixed
precision path (FP32 recursion and FFTs, FP64 accumulators, FP64 eigensolves
and reductions).  KE_max = 10 Ha (the value of the reference's CdSe example).
A pair counts as converged when sigma_E <= 1e-2 Ha (the reference's default
sigmaECut, filter_mpi/read.c:86) and its eigenvalue is within 1e-5 Ha of an
eigenvalue of the plain FP64 GPU run on the same starts (run once, untimed; the FP64 path is itself checked against
the CPU oracle and the reference's example outputs by the tests).

Timing: W warm-up steps, then K steps bracketed by barrier + synchronize,
device time from CUDA events on the library's stream; the working set
(ring of 32 Newton vectors, accumulators, 16 states per pass) is far larger
than L2.  value = converged pairs of all ranks / max step time over ranks.
e2e: the same metric through fbse_filter_job with host buffers: the starts
are copied from pinned host memory and the converged eigenvalues, sigma_E and
eigenvectors copied back each step.

--impl reference: the CPU restatement of the reference (oracle; the full
reference needs FFTW/MKL/MPI and does not build here), timed on the host's
cores on a bounded sample of the same workload and extrapolated.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "converged eigenpairs/s at |dE|<=1e-5 Ha (mixed vs plain FP64 on one GB300)"
SIGMA_CUT = 1e-2
KE_MAX = 10.0
DE_TOL = 1e-5
TARGETS = dict(vbmin=-0.33, vbmax=-0.23, cbmin=-0.145, cbmax=-0.045, nvb=8, ncb=8)
SEED = 20261204


def ene_targets(vbmin, vbmax, cbmin, cbmax, nvb, ncb):
    """set_ene_targets (filter_mpi/init.c:401-478)."""
    t = np.empty(nvb + ncb)
    d = (vbmax - vbmin) / nvb
    for j in range(nvb):
        t[nvb - j - 1] = vbmax - j * d
    d = (cbmax - cbmin) / ncb
    for j in range(nvb, nvb + ncb):
        t[j] = cbmin + (j - nvb) * d
    return t


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index=0):
        self.samples = []
        self.stop = threading.Event()
        self.index = index
        self.t = threading.Thread(target=self.run, daemon=True)

    def run(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 3 + i and s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def count_converged(ev, sg, ev64, sg64):
    """Mixed-path Ritz pairs with sigma_E <= cut matched one-to-one to FP64
    pairs with sigma_E <= cut within DE_TOL: both lists sorted, each FP64 value
    claimed at most once (a maximum matching for tolerance windows on a line),
    so a degenerate FP64 level of multiplicity k credits at most k pairs."""
    return match_detail(ev, sg, ev64, sg64)["matched"]


def match_detail(ev, sg, ev64, sg64):
    ref = np.sort(ev64[sg64 <= SIGMA_CUT])
    mine = np.sort(ev[sg <= SIGMA_CUT])
    i = j = good = 0
    while i < len(mine) and j < len(ref):
        if ref[j] < mine[i] - DE_TOL:
            j += 1
        elif ref[j] <= mine[i] + DE_TOL:
            good += 1
            i += 1
            j += 1
        else:
            i += 1
    return {"matched": good, "ritz_pairs": int(len(ev)), "fail_sigma": int(np.sum(sg > SIGMA_CUT)),
            "fail_energy": int(len(mine) - good)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_gpu(args):
    import torch
    import filterbse_gb300 as F
    from filterbse_gb300 import workload as W

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    log = (lambda *a: print(*a, file=sys.stderr, flush=True)) if rank == 0 else (lambda *a: None)

    t0 = time.time()
    dot = W.cdse_dot(args.radius, d=0.5, ke_max=KE_MAX, spinor=True)
    g = dot.grid
    log(f"[setup] {len(dot.types)} atoms ({dot.n_core} core), grid {g.nx}x{g.ny}x{g.nz}, "
        f"{dot.proj.npts} projector points/atom, {time.time() - t0:.1f}s")
    mk = lambda prec: F.Context(g, dot.pot, nspin=2, is_complex=True, so=True, nl=False, proj=dot.proj, precision=prec)
    c64 = mk(F.FP64)
    cmx = mk(F.MIXED)
    t1 = time.time()
    e0, e1, its = c64.energy_range(max_iter=1500)
    vmin = e0 - 0.2 * abs(e0)
    emax = e1 * 1.2
    de = emax - vmin
    t_range = time.time() - t1
    log(f"[range] Emin={vmin:.6f} Emax={emax:.6f} ({its} iterations, {t_range:.1f}s)")
    nc, m, ns = args.ncheby, 16, args.nstart
    zn, _ = F.samp_points(nc)
    targets = ene_targets(**TARGETS)
    dt = (nc / (2.5 * de)) ** 2
    an = F.newton_coeff(zn, targets, vmin, de, dt)
    starts, _, _ = F.init_filter_states(ns, g.ngrid, 2, True, g.dv, -(SEED + rank))
    d_starts = torch.tensor(starts, device=dev)
    stlen = starts.shape[1]

    def step(ctx):
        filt = ctx.newton_filter(zn, an, vmin, de, d_starts)
        return ctx.ortho_diag_sigma(filt.reshape(ns * m, stlen))

    t2 = time.time()
    nk64, ev64, sg64 = step(c64)
    t_fp64 = time.time() - t2
    log(f"[fp64] {nk64} Ritz pairs, {np.sum(sg64 <= SIGMA_CUT)} with sigma<={SIGMA_CUT}, {t_fp64:.1f}s wall")
    c64.close()
    torch.cuda.empty_cache()

    ext = torch.cuda.ExternalStream(cmx.stream_handle)
    for _ in range(args.warmup):
        step(cmx)
    log(f"[launches] {F.launch_count()} library kernels launched before the timed steps")
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    times, counts = [], []
    l0 = F.launch_count()
    # the timed steps sit in an NVTX range so that a profiler can select them
    # (ncu --nvtx --nvtx-include "fbse_timed_steps/")
    torch.cuda.nvtx.range_push("fbse_timed_steps")
    with Clocks(local) as clk:
        for _ in range(args.steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(ext)
            nk, ev, sg = step(cmx)
            b.record(ext)
            b.synchronize()
            times.append(a.elapsed_time(b) / 1e3)
            counts.append(count_converged(ev, sg, ev64, sg64))
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    launches = F.launch_count() - l0  # all kernels of the K timed steps
    t_step = float(np.mean(times))
    n_conv = int(np.median(counts))
    detail = match_detail(ev, sg, ev64, sg64)
    log(f"[mixed] step {t_step * 1e3:.1f} ms, converged {counts}, Ritz pairs {nk}, fp64-run {t_fp64:.1f}s")

    # ---- e2e through the host-buffer entry point
    pinned = torch.from_numpy(starts).pin_memory()
    psi_out = torch.empty((ns * m, stlen), dtype=torch.float64).pin_memory()
    e2e_times = []
    for it in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        k, ev_e, sg_e = cmx.filter_job(zn, an, vmin, de, pinned.numpy(), sigma_cut=SIGMA_CUT, psi_out=psi_out)
        el = time.perf_counter() - t
        if it >= args.warmup:
            e2e_times.append(el)
    n_e2e = count_converged(ev_e, sg_e, ev64, sg64)
    t_e2e = float(np.mean(e2e_times))
    h2d = starts.nbytes
    d2h = int(k * stlen * 8 + 2 * k * 8)

    # ---- learned refinement, judged by the plain FP64 filter at 3x the terms
    learned = learned_leg(args, F, W, dot, g, cmx=cmx, zn_an=(vmin, de), d_starts=d_starts, stlen=stlen,
                          fp64=(ev64, sg64), log=log) if args.learned and world == 1 else None

    # ---- H psi roofline: one batched H psi of the 16 spinor starts (FP32)
    import torch as T
    x = T.tensor(starts.view(np.complex128), dtype=T.complex64, device=dev)
    y = T.empty_like(x)
    for _ in range(3):
        cmx.hpsi(x, y, sync=False)
    T.cuda.synchronize()
    nrep = 20
    a = T.cuda.Event(enable_timing=True)
    b = T.cuda.Event(enable_timing=True)
    a.record(ext)
    for _ in range(nrep):
        cmx.hpsi(x, y, sync=False)
    b.record(ext)
    b.synchronize()
    t_h = a.elapsed_time(b) / 1e3 / nrep
    N = g.ngrid
    pj = dot.proj
    t_proj = int(np.sum(pj.nl)) * (4 + 6 * 4 + 5 * 4)  # jxyz + Y_1m + SO radial, FP32
    bytes_h = ns * 2 * N * (8 + 8) + N * 4 + t_proj
    peak, peak_kind = measured_peaks()
    achieved = bytes_h / t_h / 1e9

    # ---- reduce over ranks
    tot_conv, t_max, tot_e2e, t_e2e_max = n_conv, t_step, n_e2e, t_e2e
    if dist:
        v = torch.tensor([float(n_conv), t_step, float(n_e2e), t_e2e], device=dev, dtype=torch.float64)
        s = v.clone()
        dist.all_reduce(s, op=dist.ReduceOp.SUM)
        mxv = v.clone()
        dist.all_reduce(mxv, op=dist.ReduceOp.MAX)
        tot_conv, t_max, tot_e2e, t_e2e_max = s[0].item(), mxv[1].item(), s[2].item(), mxv[3].item()
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # the CPU port is FP64: it converges what the FP64 pipeline converges
    n64 = int(np.sum(sg64 <= SIGMA_CUT))
    cpu = cpu_baseline(dot, args, n64, nk64, sample_states=1)
    out = {
        "metric": METRIC,
        "value": tot_conv / t_max,
        "unit": "eigenpairs/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": t_max * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 recursion/FFT, f64 accumulators/eigensolves",
        "data": "synthetic (seeded 3 nm CdSe dot, reference II-VI potential tables)",
        "config": {"workload": f"CdSe zincblende sphere r={args.radius}A, {len(dot.types)} atoms, spinor+SO, "
                               f"grid {g.nx}x{g.ny}x{g.nz} @0.5 bohr, {ns} starts x {m} targets, nCheby {nc}",
                   "grid": [g.nx, g.ny, g.nz], "n_states": ns * m, "ncheby": nc,
                   "converged_per_step": n_conv, "ritz_pairs": int(nk),
                   "unconverged_sigma": detail["fail_sigma"], "unconverged_energy": detail["fail_energy"],
                   "fp64_run_s": t_fp64,
                   "fp64_converged": n64, "fp64_eigenpairs_per_s": n64 / t_fp64,
                   "mixed_over_fp64": (n_conv / t_step) / (n64 / t_fp64) if n64 else None,
                   "energy_range_s": t_range, "l2": "working set >> L2 (no flush needed)",
                   "parallelism": f"replicas x{world} (independent starts per GPU)"},
        "e2e": {"value": tot_e2e / t_e2e_max, "unit": "eigenpairs/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "gpu_launches_per_step": int(round(launches / max(1, args.steps))),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": HPSI_DRAM_BYTES if (args.radius, args.nstart) == (15.0, 16) else None,
                     "traffic_source": "DRAM bytes read + written by the H psi kernels of one batched H psi of "
                                       "this workload, one ncu capture with cold caches",
                     "kernel": "H psi (5 FFT passes + projector gather/scatter), 16 spinor states",
                     "ms_per_launch": t_h * 1e3, "algorithmic_bytes": bytes_h, "peak_kind": peak_kind},
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        **({"learned": learned} if learned else {}),
    }
    print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


def learned_leg(args, F, W, dot, g, cmx, zn_an, d_starts, stlen, fp64, log):
    """The learned residual refinement on the headline workload.  Training
    pairs come from the filter on a 1.6 nm dot (mixed filter at nCheby/4
    against the plain FP64 filter at nCheby); the network trains on the GPU
    (untimed).  Judge: the plain FP64 filter at 3 x nCheby on the same 16
    starts; its levels with sigma <= 1e-6 are the reference.  Reported: pairs
    matching those levels to 1e-5 Ha (one-to-one, sigma <= 1e-2) for the
    plain FP64 filter, the mixed filter, and the mixed filter + 2 refinement
    rounds (timed, CUDA events) with the trained network and with plain
    residuals."""
    import torch
    from filterbse_gb300 import learn
    vmin, de = zn_an
    t0 = time.time()
    small = W.cdse_dot(8.0, d=0.5, ke_max=KE_MAX, spinor=True)
    gs = small.grid
    mk = lambda p: F.Context(gs, small.pot, nspin=2, is_complex=True, so=True, nl=False, proj=small.proj, precision=p)
    s64, smx = mk(F.FP64), mk(F.MIXED)
    e0, e1, _ = s64.energy_range(max_iter=1500)
    sv, sde = e0 - 0.2 * abs(e0), e1 * 1.2 - (e0 - 0.2 * abs(e0))
    st, _, _ = F.init_filter_states(16, gs.ngrid, 2, True, gs.dv, -(SEED + 7))
    sd0 = torch.tensor(st, device=d_starts.device)

    def run_small(ctx, nc):
        zn, _ = F.samp_points(nc)
        an = F.newton_coeff(zn, ene_targets(**TARGETS), sv, sde, (nc / (2.5 * sde)) ** 2)
        return learn.ritz(ctx, zn, an, sv, sde, sd0)
    short = run_small(smx, args.ncheby // 4)
    judge_small = run_small(s64, args.ncheby)
    pairs = learn.training_pairs((smx,) + short, (s64,) + judge_small)
    if pairs is None:
        return {"error": "no training pairs"}
    pc = F.Precond(smx, seed=5)
    hist = learn.train(pc, pairs, steps=300, lr=2e-3, batch=8)
    w = pc.weights
    t_train = time.time() - t0
    log(f"[learned] {pairs[0].shape[0]} pairs, loss {np.mean(hist[:5]):.3e} -> {np.mean(hist[-20:]):.3e}, "
        f"{t_train:.1f}s")
    del s64, smx, pc, pairs

    # the judge on the headline workload
    c64 = F.Context(g, dot.pot, nspin=2, is_complex=True, so=True, nl=False, proj=dot.proj, precision=F.FP64)
    m = 16

    def run(ctx, nc):
        zn, _ = F.samp_points(nc)
        an = F.newton_coeff(zn, ene_targets(**TARGETS), vmin, de, (nc / (2.5 * de)) ** 2)
        return learn.ritz(ctx, zn, an, vmin, de, d_starts)
    t1 = time.time()
    _, nj, evj, sgj = run(c64, 3 * args.ncheby)
    ref = evj[sgj <= 1e-6]
    t_judge = time.time() - t1
    ev64, sg64 = fp64  # the plain FP64 pipeline of the main leg, same starts
    c64.close()
    torch.cuda.empty_cache()
    log(f"[learned] judge: {len(ref)} levels with sigma <= 1e-6 ({t_judge:.0f}s)")
    ps, n, ev, sg = run(cmx, args.ncheby)
    out = {"judge_ncheby": 3 * args.ncheby, "judge_levels": int(len(ref)), "train_pairs_s": t_train,
           "fp64_matched": learn.match(ev64, sg64, ref), "mixed_matched": learn.match(ev, sg, ref)}
    ext = torch.cuda.ExternalStream(cmx.stream_handle)
    net = F.Precond(cmx, weights=w)
    for name, p in (("refined", net), ("refined_plain", None)):
        buf = torch.zeros((3 * n, stlen), dtype=torch.float64, device=d_starts.device)
        buf[:n] = ps[:n]
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(ext)
        k, e2, s2 = cmx.refine(buf, n, ev, sg, steps=2, tol=1e-3, precond=p)
        b.record(ext)
        b.synchronize()
        out[name + "_matched"] = learn.match(e2, s2, ref)
        out[name + "_ms"] = a.elapsed_time(b)
        del buf
    log(f"[learned] matched judge levels: fp64 {out['fp64_matched']}, mixed {out['mixed_matched']}, "
        f"mixed+refined {out['refined_matched']} ({out['refined_ms']:.0f} ms), plain residuals "
        f"{out['refined_plain_matched']}")
    net.close()
    return out


def _oracle_table(W, O, og, core_coords):
    """The projector table of the CPU legs, built by the oracle on the host
    (the same table as the library's GPU builder): spin-orbit channels of the
    workload (SO_par 0.01, no NL)."""
    n = len(core_coords)
    tab = W.so_radial(0.5, np.sqrt(W.r_nlcut2(0.5)))
    return O.nlc_table(og, np.ascontiguousarray(core_coords), np.full(n, 0.01), tab, np.zeros((n, 5, 1024)),
                       np.zeros((n, 5), np.int32))


def _cpu_sample(radius, ncheby, nstart, sample_terms, seed):
    """Times the oracle on one spinor start: one H psi and the m axpys of one
    Newton term (filter.c:318-359) at the full grid."""
    from filterbse_gb300 import workload as W
    from oracle import oracle as O
    types, coords = W.zincblende_dot(radius)
    g = W.reference_grid(coords, 0.5, KE_MAX)
    core = [i for i, t in enumerate(types) if not t.startswith("P")]
    og = O.Grid(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.xmin, g.ymin, g.zmin, KE_MAX)
    # the per-term cost does not depend on the potential's values
    pot = np.random.default_rng(seed).uniform(-1.5, 0.3, og.ngrid)
    t_pot = 0.0
    proj = _oracle_table(W, O, og, coords[core])
    sysm = O.System(og, pot, nspin=2, is_complex=True, so=True, nlflag=False, proj=proj)
    rng = np.random.default_rng(seed)
    psi = rng.uniform(-1, 1, 2 * og.ngrid) + 1j * rng.uniform(-1, 1, 2 * og.ngrid)
    acc = np.zeros((16, 2 * og.ngrid), np.complex128)
    t = time.time()
    for _ in range(sample_terms):
        psi = O.hnorm(psi, sysm, 0.15, -1.0, 0.3)
        acc += 0.01 * psi[None, :]
    t_term = (time.time() - t) / sample_terms
    return t_term, t_pot


def cpu_baseline(dot, args, n_conv, n_ritz, sample_states=1):
    """CPU restatement timed on the host (1 core): per-term cost of one start,
    extrapolated to the full stage (nstart x (nCheby-1) terms plus the 3n H psi
    of diag_H and calc_sigma_E, filter_mpi/Hmat.c, energy.c:383-539)."""
    t_term, _ = _cpu_sample(args.radius, args.ncheby, args.nstart, 1, 1)
    n = args.nstart * 16
    t_total = t_term * (args.nstart * (args.ncheby - 1) + 3 * n)
    return {"value": n_conv / t_total, "unit": "eigenpairs/s", "cores": 1, "kind": "port",
            "sample": f"1 Newton term (H psi + 16 axpys) of one spinor start on the full grid, {t_term:.2f} s; "
                      f"extrapolated to {args.nstart}x{args.ncheby - 1} terms + {3 * n} H psi; "
                      f"converged count {n_conv} of the FP64 pipeline on the same starts"}


def _worker(q, radius, ncheby, nstart, seed, nrep):
    """One host process: builds the workload once, then times nrep Newton terms
    (one per step of the arm) and reports each."""
    from filterbse_gb300 import workload as W
    from oracle import oracle as O
    types, coords = W.zincblende_dot(radius)
    g = W.reference_grid(coords, 0.5, KE_MAX)
    core = [i for i, t in enumerate(types) if not t.startswith("P")]
    og = O.Grid(g.nx, g.ny, g.nz, g.dx, g.dy, g.dz, g.xmin, g.ymin, g.zmin, KE_MAX)
    pot = np.random.default_rng(seed).uniform(-1.5, 0.3, og.ngrid)
    proj = _oracle_table(W, O, og, coords[core])
    sysm = O.System(og, pot, nspin=2, is_complex=True, so=True, nlflag=False, proj=proj)
    rng = np.random.default_rng(seed)
    psi = rng.uniform(-1, 1, 2 * og.ngrid) + 1j * rng.uniform(-1, 1, 2 * og.ngrid)
    acc = np.zeros((16, 2 * og.ngrid), np.complex128)
    q.put(("ready", seed))
    for _ in range(nrep):
        t = time.time()
        psi = O.hnorm(psi, sysm, 0.15, -1.0, 0.3)
        acc += 0.01 * psi[None, :]
        q.put(("term", time.time() - t))


def _cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def run_reference(args):
    """The CPU arm: the oracle's restatement of the reference's H psi and
    Newton term (FP64, numpy FFTs) on P = min(nproc, nstart) host processes of
    one thread each, one random start per process as the reference's ranks
    run them (filter_mpi/mod_filter.c:155-159).  A step is one Newton term of
    every process; the stage time is extrapolated from the mean term time:
    nstart / P rounds of nCheby - 1 terms plus the 3 n H psi of diag_H and
    calc_sigma_E spread over the processes."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[k] = "1"
    ctx = mp.get_context("spawn")
    ncores = os.cpu_count() or 1
    procs = max(1, min(ncores, args.nstart))
    nrep = args.warmup + args.steps
    q = ctx.Queue()
    ps = [ctx.Process(target=_worker, args=(q, args.radius, args.ncheby, args.nstart, 100 + i, nrep))
          for i in range(procs)]
    for p in ps:
        p.start()
    ready, terms = 0, []
    while ready < procs or len(terms) < procs * nrep:
        kind, v = q.get(timeout=1800)
        if kind == "ready":
            ready += 1
        else:
            terms.append(v)
    for p in ps:
        p.join()
    # per-step mean over the processes, warm-up steps dropped
    per_step = [float(np.mean(terms[i * procs:(i + 1) * procs])) for i in range(nrep)][args.warmup:]
    if not per_step:
        raise RuntimeError("reference arm: no timed steps")
    t_term = float(np.mean(per_step))
    n = args.nstart * 16
    t_total = t_term * (args.ncheby - 1) * np.ceil(args.nstart / procs) + t_term * 3 * n / procs
    n_conv = args.ref_converged
    val = n_conv / t_total
    out = {"metric": METRIC, "value": val, "unit": "eigenpairs/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_total * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": f"CdSe zincblende sphere r={args.radius}A spinor+SO, {args.nstart} starts x 16 "
                                  f"targets, nCheby {args.ncheby}", "cpu_model": _cpu_model(), "host_cores": ncores},
           "cpu_baseline": {"value": val, "unit": "eigenpairs/s", "cores": procs, "kind": "port",
                            "sample": f"{procs} processes x 1 thread, each timing {nrep} Newton terms (H psi + 16 "
                                      f"axpys) of one spinor start on the full grid, {args.warmup} dropped as "
                                      f"warm-up ({t_term:.3f} s/term); extrapolated to the full stage; converged "
                                      f"count {n_conv} as produced by the FP64 pipeline on this workload"},
           "e2e": {"value": val, "unit": "eigenpairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


# DRAM bytes read + written by one batched H psi of the 16 spinor starts of the
# 3 nm CdSe dot (the five kernels of one H psi, one ncu capture with cold
# caches: planes 1024 + 1038 + 1627 MB, projector gather 582 MB, scatter 761 MB)
HPSI_DRAM_BYTES = 5.032e9


def run_uneven(args):
    """Optional workload (--workload uneven): n uneven CdSe/InP spinor dots
    (diameters U(2, 4) nm, grids by the reference's rule capped at 160^3),
    4 starts x 16 targets each, filtered by one CUDA graph launch against the
    same contexts dot by dot.  Prints one JSON line with both rates."""
    import torch
    import filterbse_gb300 as F
    from filterbse_gb300 import workload as W
    log = lambda *a: print(*a, file=sys.stderr, flush=True)
    dev = torch.device("cuda", 0)
    t0 = time.time()
    dots = W.uneven_dots(args.ndots)
    log(f"[setup] {len(dots)} dots, grids {sorted(d.grid.nx for _, _, d in dots)}, {time.time() - t0:.1f}s")
    ns, m, nc = 4, 16, args.ncheby
    items, ctxs, bytes_h = [], [], 0
    for i, (mat, dia, dot) in enumerate(dots):
        g = dot.grid
        ctx = F.Context(g, dot.pot, nspin=2, is_complex=True, so=True, nl=False, proj=dot.proj, precision=F.MIXED)
        ctx.set_tuning(newton_ring=16)
        e0, e1, _ = ctx.energy_range(max_iter=1500)
        vmin, emax = e0 - 0.2 * abs(e0), e1 * 1.2
        de = emax - vmin
        zn, _ = F.samp_points(nc)
        an = F.newton_coeff(zn, ene_targets(**TARGETS), vmin, de, (nc / (2.5 * de)) ** 2)
        starts, _, _ = F.init_filter_states(ns, g.ngrid, 2, True, g.dv, -(SEED + 100 + i))
        items.append((ctx, zn, an, vmin, de, torch.tensor(starts, device=dev)))
        ctxs.append(ctx)
        t_proj = int(np.sum(dot.proj.nl)) * (4 + 6 * 4 + 5 * 4)
        bytes_h += (nc - 1) * (ns * 2 * g.ngrid * 16 + g.ngrid * 4 + t_proj)
    t1 = time.time()
    b = F.Batch(items)
    log(f"[graph] {b.nodes} nodes, captured and instantiated in {time.time() - t1:.1f}s (with one ordinary run)")
    res = {}
    for mode in ("graph", "sequential"):
        for _ in range(args.warmup):
            b.run(sequential=mode == "sequential")
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            t = time.perf_counter()
            b.run(sequential=mode == "sequential")
            ts.append(time.perf_counter() - t)
        res[mode] = float(np.mean(ts))
        log(f"[{mode}] {res[mode] * 1e3:.1f} ms per filter of all dots")
    nstates = len(dots) * ns * m
    out = {"metric": "filtered states/s, uneven multi-dot batch in one CUDA graph", "value": nstates / res["graph"],
           "unit": "states/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": res["graph"] * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 recursion/FFT, f64 accumulators",
           "data": "synthetic (seeded CdSe/InP dots, reference II-VI and InP potential tables)",
           "config": {"workload": f"{len(dots)} CdSe/InP spinor dots, diameters U(2,4) nm, {ns} starts x {m} "
                                  f"targets each, nCheby {nc}",
                      "grids": [d.grid.nx for _, _, d in dots], "graph_nodes": b.nodes,
                      "sequential_ms": res["sequential"] * 1e3,
                      "graph_over_sequential": res["sequential"] / res["graph"],
                      "hpsi_gbs_graph": bytes_h / res["graph"] / 1e9,
                      "hpsi_gbs_sequential": bytes_h / res["sequential"] / 1e9}}
    b.close()
    print(json.dumps(out), flush=True)


def run_bse(args):
    """Optional workload (--workload bse): the BSE stage on 40 hole and 40
    electron spinor states of the 3 nm dot (the mixed pipeline's Ritz vectors
    closest to the gap), n_xton = 1600, 128^3, epsilon = 6.  The kernel
    contraction runs on the FP64 SIMT path and on the mixed path (FP32 pair
    densities and convolutions, split-TF32 tcgen05 contraction); exciton
    energies and oscillator strengths of the mixed path are compared with the
    FP64 path's.  Prints one JSON line."""
    import torch
    import filterbse_gb300 as F
    from filterbse_gb300 import workload as W
    log = lambda *a: print(*a, file=sys.stderr, flush=True)
    dev = torch.device("cuda", 0)
    dot = W.cdse_dot(args.radius, d=0.5, ke_max=KE_MAX, spinor=True)
    g = dot.grid
    mk = lambda p: F.Context(g, dot.pot, nspin=2, is_complex=True, so=True, nl=False, proj=dot.proj, precision=p)
    cmx = mk(F.MIXED)
    e0, e1, _ = cmx.energy_range(max_iter=1500)
    vmin, emax = e0 - 0.2 * abs(e0), e1 * 1.2
    de = emax - vmin
    zn, _ = F.samp_points(args.ncheby)
    an = F.newton_coeff(zn, ene_targets(**TARGETS), vmin, de, (args.ncheby / (2.5 * de)) ** 2)
    starts, _, _ = F.init_filter_states(args.nstart, g.ngrid, 2, True, g.dv, -SEED)
    filt = cmx.newton_filter(zn, an, vmin, de, torch.tensor(starts, device=dev)).reshape(-1, 2 * 2 * g.ngrid)
    nk, ev, sg = cmx.ortho_diag_sigma(filt)
    # quasiparticle basis: the 40 highest states below the gap and the 40
    # lowest above it (the gap: the largest spacing between the VB and CB windows)
    gap_mid = 0.5 * (TARGETS["vbmax"] + TARGETS["cbmin"])
    order = np.argsort(ev)
    holes = [i for i in order if ev[i] < gap_mid][-40:]
    elecs = [i for i in order if ev[i] > gap_mid][:40]
    nh, ne = len(holes), len(elecs)
    idx = holes + elecs
    psi = filt[idx].contiguous().view(torch.complex128).reshape(nh + ne, -1).contiguous()
    eq = ev[idx]
    gx, gy, gz = g.axes()
    out = {"n_h": nh, "n_e": ne, "n_xton": nh * ne}
    res = {}
    for name, prec in (("fp64", F.FP64), ("mixed", F.MIXED)):
        ctx = mk(prec)
        bare, scr = ctx.bse_potentials(gx, gy, gz, g.xmin, g.ymin, g.zmin, eps=(6.0, 6.0, 6.0))
        ctx.bse_kernel(psi[:2], 1, 1, 1, bare, scr)  # warm-up of the kernels' scratch
        torch.cuda.synchronize()
        t = time.perf_counter()
        d, x = ctx.bse_kernel(psi, nh, ne, nh, bare, scr)
        torch.cuda.synchronize()
        tk = time.perf_counter() - t
        t = time.perf_counter()
        xe, coeff, *_ = ctx.bse_solve(eq, nh, ne, nh, d, x)
        mu = ctx.bse_dipoles(psi, gx, gy, gz, nh, ne, nh)
        mx = ctx.bse_optical(coeff, mu, nh, ne)
        torch.cuda.synchronize()
        ts = time.perf_counter() - t
        os_ = (2.0 / 3.0) * xe * np.sum(np.abs(mx) ** 2, axis=1)
        res[name] = (xe, os_)
        out[name] = {"kernel_s": tk, "solve_dipoles_s": ts}
        log(f"[bse {name}] kernel {tk:.2f}s, solve + dipoles {ts:.2f}s, lowest exciton {xe[0]:.8f}")
        ctx.close()
        del d, x, coeff
        torch.cuda.empty_cache()
    dxe = np.abs(res["mixed"][0] - res["fp64"][0])
    # oscillator strengths compared as sums over exciton clusters (levels within 1e-6 Ha mix freely)
    e64 = res["fp64"][0]
    cl, cur = [], [0]
    for i in range(1, len(e64)):
        if e64[i] - e64[i - 1] < 1e-6:
            cur.append(i)
        else:
            cl.append(cur)
            cur = [i]
    cl.append(cur)
    osd = max(abs(res["mixed"][1][c].sum() - res["fp64"][1][c].sum()) for c in cl)
    # FLOPs of the contraction (Hermitian halves of K^d and K^x): 8 N (n_e^2 n_h^2 + (n_e n_h)^2) / 2
    N = g.ngrid
    flops = 8.0 * N * (ne * ne * nh * nh + (ne * nh) ** 2) / 2
    out.update({"max_dE_mixed_vs_fp64": float(dxe.max()), "lowest_exciton_fp64": float(e64[0]),
                "max_cluster_OS_diff": float(osd), "max_OS": float(res["fp64"][1].max()),
                "contraction_tflops_fp64": flops / out["fp64"]["kernel_s"] / 1e12,
                "contraction_tflops_mixed": flops / out["mixed"]["kernel_s"] / 1e12})
    line = {"metric": "BSE kernel + solve, 40h x 40e spinor states of the 3 nm CdSe dot (n_xton 1600, 128^3)",
            "value": out["mixed"]["kernel_s"] + out["mixed"]["solve_dipoles_s"], "unit": "s",
            "higher_is_better": False, "n_gpus": 1, "dtype": "mixed: f32 densities/convolutions, split-tf32 "
            "tcgen05 contraction, f64 solve", "data": "synthetic", "config": out}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--radius", type=float, default=15.0)
    ap.add_argument("--ncheby", type=int, default=2048)
    ap.add_argument("--nstart", type=int, default=16)
    ap.add_argument("--workload", default="dot", choices=["dot", "uneven", "bse"],
                    help="dot: the 3 nm CdSe spinor dot (the headline); uneven: the multi-dot graph batch; "
                         "bse: the BSE stage on 40 + 40 states of the 3 nm dot")
    ap.add_argument("--ndots", type=int, default=24)
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip the learned-refinement leg (judge run, training, refinement)")
    ap.add_argument("--ref-converged", type=int, default=248,
                    help="eigenpairs an FP64 run of this workload converges to sigma <= 1e-2 (the "
                         "reference's sigmaECut): 248 for the default 3 nm dot, from the plain FP64 "
                         "GPU pipeline the gb300 arm runs on the same starts")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "uneven":
        run_uneven(args)
    elif args.workload == "bse":
        run_bse(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
