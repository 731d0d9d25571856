"""Study-compatible profiling driver.

    python -m pascal_btdma_gb300.study n1 n2 n3 m iters [--nseg P] [--workload diagonal|dominant]
                                       [--precision fp64] [--signature-out FILE]

Same arguments, same per-iteration flow and the same CSV schemas as the
reference's matched profiling driver (Study/example_cuda_cxx_btdma_profile.cu,
schemas in Study/README.md): nsys = n1*n2 systems of n3 block rows, block size
m; every iteration copies A, B, C, D from host memory to the device, solves
with solve_noncyclic_profiled and prints one timing row

    solver,variant,implementation,nranks,n1,n2,n3,m,nsys,nrow_min,nrow_max,iter,
    iterations,mpi_mode,total_s_max,total_s_avg,local_compute_s_max,
    forward_exchange_s_max,reduced_compute_s_max,backward_exchange_s_max,
    update_compute_s_max,compute_s_max,communication_s_max

and, on iteration 0, appends a solution-signature row to --signature-out (or
$PASCAL_BTDMA_SIGNATURE_OUT).  One process on one GPU: `nranks` is the number
of line segments (--nseg), nrow_min/nrow_max are the shortest and longest
segment, and `mpi_mode` reads "device" (the reduced rows never leave the GPU).
The default workload is the Study's diagonal one (A = 0.25 I, B = 2 I,
C = 0.25 I, d = 1); --workload dominant uses the seeded random generator.
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="Study-compatible profiling driver")
    ap.add_argument("n1", type=int, nargs="?", default=32)
    ap.add_argument("n2", type=int, nargs="?", default=32)
    ap.add_argument("n3", type=int, nargs="?", default=128)
    ap.add_argument("m", type=int, nargs="?", default=5)
    ap.add_argument("iters", type=int, nargs="?", default=10)
    ap.add_argument("--nseg", type=int, default=1)
    ap.add_argument("--workload", choices=["diagonal", "dominant"], default="diagonal")
    ap.add_argument("--delta", type=float, default=1.2)
    ap.add_argument("--precision", default="fp64")
    ap.add_argument("--signature-out", default=os.environ.get("PASCAL_BTDMA_SIGNATURE_OUT", ""))
    args = ap.parse_args(argv)

    import torch

    import pascal_btdma_gb300 as pbt
    from pascal_btdma_gb300 import synth

    n1, n2, n3, m, iters, nseg = args.n1, args.n2, args.n3, args.m, args.iters, args.nseg
    nsys = n1 * n2
    if n3 < 2:
        print("n3 must be >= 2", file=sys.stderr)
        return 2
    segs = [pbt.partition_1d(0, n3 - 1, nseg, r) for r in range(nseg)]
    nrow_min = min(l - f + 1 for f, l in segs)
    nrow_max = max(l - f + 1 for f, l in segs)
    if args.workload == "diagonal":
        w = synth.diagonal(m, nsys, n3)
    else:
        w = synth.dominant(m, nsys, n3, seed=12345, delta=args.delta)
    host = [torch.from_numpy(x).pin_memory() for x in w.arrays]
    dev = torch.device("cuda", torch.cuda.current_device())
    a, b, c, d = (torch.empty_like(h, device=dev) for h in host)
    plan = pbt.BtdmaGpuPlan().create(m, nsys, n3, nseg, precision=args.precision)

    print("solver,variant,implementation,nranks,n1,n2,n3,m,nsys,nrow_min,nrow_max,iter,iterations,mpi_mode,"
          "total_s_max,total_s_avg,local_compute_s_max,forward_exchange_s_max,reduced_compute_s_max,"
          "backward_exchange_s_max,update_compute_s_max,compute_s_max,communication_s_max", flush=True)
    for it in range(iters):
        for dst, src in zip((a, b, c, d), host):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        t = pbt.solve_noncyclic_profiled(plan, a, b, c, d, m, nsys, n3)
        fields = [t.total, t.local_compute, t.forward_exchange, t.reduced_compute, t.backward_exchange,
                  t.update_compute, t.computation(), t.communication()]
        row = ["btdma", "noncyclic", "gb300", nseg, n1, n2, n3, m, nsys, nrow_min, nrow_max, it, iters, "device",
               f"{fields[0]:.12g}", f"{fields[0]:.12g}"] + [f"{v:.12g}" for v in fields[1:]]
        print(",".join(map(str, row)), flush=True)
        if it == 0 and args.signature_out:
            x = d.cpu().numpy()
            xs = x.reshape(m, n3, nsys)
            exists = os.path.exists(args.signature_out) and os.path.getsize(args.signature_out) > 0
            with open(args.signature_out, "a") as f:
                if not exists:
                    f.write("solver,variant,implementation,nranks,n1,n2,n3,m,nsys,nrow_min,nrow_max,mpi_mode,"
                            "solution_sum,solution_l2,solution_linf,sample_z0,sample_zmid,sample_zlast\n")
                vals = [float(x.sum()), math.sqrt(float((x * x).sum())), float(np.abs(x).max()),
                        float(xs[0, 0, 0]), float(xs[0, n3 // 2, 0]), float(xs[0, n3 - 1, 0])]
                f.write(",".join(map(str, ["btdma", "noncyclic", "gb300", nseg, n1, n2, n3, m, nsys, nrow_min,
                                           nrow_max, "device"] + [repr(v) for v in vals])) + "\n")
    plan.destroy()
    return 0


if __name__ == "__main__":
    sys.exit(main())
