"""One batched H psi on the benchmark workload (3 nm CdSe spinor dot, 128^3,
spin-orbit projectors, 16 seeded random starts), run three times.

This is the program the per-kernel ncu captures under profiles/ profile
(`python tests/hpsi_batch.py [mixed|fp64] [so|noso] [fused]`; "fused" runs
the mixed path's projectors fused into the FFT plane passes,
fbse_tuning.hpsi_fused = 1); pytest does not collect it.  It needs a GPU and the built
library."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    import torch
    import filterbse_gb300 as F
    from filterbse_gb300 import workload as W
    prec = F.FP64 if "fp64" in sys.argv[1:] else F.MIXED
    so = "noso" not in sys.argv[1:]
    dot = W.cdse_dot(15.0, d=0.5, ke_max=10.0, spinor=True)
    g = dot.grid
    c = F.Context(g, dot.pot, nspin=2, is_complex=True, so=so, nl=False, proj=dot.proj if so else None,
                  precision=prec)
    if "fused" in sys.argv[1:]:
        c.set_tuning(hpsi_fused=1)
    starts, _, _ = F.init_filter_states(16, g.ngrid, 2, True, g.dv, -777)
    dt = torch.complex64 if prec == F.MIXED else torch.complex128
    x = torch.tensor(starts.view(np.complex128), dtype=dt, device="cuda:0")
    y = torch.empty_like(x)
    for _ in range(3):
        c.hpsi(x, y)
    # the same H psi back to back, timed with CUDA events on the library's stream
    ext = torch.cuda.ExternalStream(c.stream_handle)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = F.launch_count()
    a.record(ext)
    for _ in range(20):
        c.hpsi(x, y, sync=False)
    b.record(ext)
    b.synchronize()
    print("H psi batch done:", g.nx, g.ny, g.nz, "FP64" if prec == F.FP64 else "mixed", "SO" if so else "no SO",
          f"{(F.launch_count() - l0) / 20:.0f} kernels", f"{a.elapsed_time(b) / 20:.4f} ms per H psi")
    for r in c.tuning_report():
        print("autotuner:", r)


if __name__ == "__main__":
    main()
