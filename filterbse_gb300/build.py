"""Builds libfbse_gpu.so in-tree: the sm_103a CUDA kernels, the C-ABI and the
host C helpers, with nvcc (one -gencode, translation units compiled in
parallel) and gcc.  Output: filterbse_gb300/libfbse_gpu.so."""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libfbse_gpu.so")
CU_SOURCES = ["hpsi_fused.cu", "fft.cu", "hpsi.cu", "filter.cu", "linalg.cu", "bse.cu", "angular.cu", "tcgemm.cu", "setup.cu", "job.cu", "precond.cu", "batch.cu", "api.cu"]
C_SOURCES = ["host/fbse_host.c", "host/fbse_setup.c", "host/fbse_bse_stats.c"]
EXECUTABLES = {"fbse_filter": "host/fbse_filter_main.c", "fbse_bse": "host/fbse_bse_main.c"}
BIN = os.path.join(HERE, "bin")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include")]


def _deps():
    out = []
    for d in ("csrc", "host"):
        for f in os.listdir(os.path.join(HERE, d)):
            out.append(os.path.join(HERE, d, f))
    out.append(os.path.join(ROOT, "include", "fbse.h"))
    return out


def _stale(obj: str, srcs) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(HERE, "csrc", s)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, deps):
            jobs.append([NVCC, *ARCH, *NVFLAGS, "-c", src, "-o", obj])
    for s in C_SOURCES:
        src = os.path.join(HERE, s)
        obj = os.path.join(BUILD, os.path.basename(s).replace(".c", ".o"))
        objs.append(obj)
        if force or _stale(obj, deps):
            # no contraction into fused multiply-adds: the same results on x86-64 and aarch64 hosts
            jobs.append(["gcc", "-O2", "-fPIC", "-std=gnu99", "-ffp-contract=off", "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for log in ex.map(_run, jobs):
            if verbose and log.strip():
                print(log)
    relinked = False
    if force or jobs or not os.path.exists(LIB):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
        relinked = True
    # drop-in executables (filter_mpi's and bse_cplx's command-line stages)
    os.makedirs(BIN, exist_ok=True)
    for exe, src in EXECUTABLES.items():
        out = os.path.join(BIN, exe)
        srcp = os.path.join(HERE, src)
        if force or relinked or _stale(out, [srcp, os.path.join(HERE, "host", "fbse_dropin.h"), LIB]):
            _run(["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-o", out,
                  srcp, "-L" + HERE,
                  "-lfbse_gpu", "-Wl,-rpath,$ORIGIN/..", "-lm"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
