"""Sweeps of lines that live in an application's own arrays (pbt_solve_noncyclic_lines).

    python -m pascal_btdma_gb300.strided n m [--axis {x,y,z}] [--precision ff] [--sweeps 3]

The euler3d layout: U(n,n,n,m) and trA(n,n,n,m,m) in Fortran order, element e
of point (i, j, k) at i + n*(j + n*(k + n*e)), filled with the seeded
diagonally dominant generator.  A sweep along `axis` solves n*n lines of n
block rows in place in those arrays, with no transposes (x: lines along the
contiguous index, uncoalesced; y, z: coalesced).
"""
from __future__ import annotations

import argparse


def app_field(n: int, m: int, seed: int = 20240101, delta: float = 1.2, device: str = "cuda:0"):
    """A, B, C, D in the euler3d layout for the z sweep's systems: the reference
    layout [e, row=k, s_out=j, s_in=i] is exactly [e, k, j, i]."""
    import torch

    from . import synth

    w = synth.dominant(m, n * n, n, seed=seed, delta=delta)
    return [torch.from_numpy(x).to(device) for x in w.arrays]


def lines_of(n: int, axis: str):
    from . import Lines

    e = n * n * n
    if axis == "x":  # rows along i (stride 1), lines over (j, k)
        return Lines(n, n, n, n * n, 1, e)
    if axis == "y":  # rows along j (stride n), lines over (i, k)
        return Lines(n, n, 1, n * n, n, e)
    if axis == "z":  # rows along k (stride n*n), lines over (i, j)
        return Lines(n, n, 1, n, n * n, e)
    raise ValueError(f"axis {axis!r}: one of x, y, z")


def sweep(n: int, m: int, axis: str = "y", precision: str = "ff", sweeps: int = 3) -> float:
    """ms per sweep (CUDA events, after one untimed sweep); D is re-solved in
    place each time, which leaves the work per sweep unchanged."""
    import torch

    from . import BtdmaGpuPlan, solve_noncyclic_lines

    a, b, c, d = app_field(n, m)
    lines = lines_of(n, axis)
    with BtdmaGpuPlan() as plan:
        plan.create(m, n * n, n, 1, precision=precision)
        solve_noncyclic_lines(plan, a, b, c, d, lines)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(sweeps):
            solve_noncyclic_lines(plan, a, b, c, d, lines)
        e1.record()
        torch.cuda.synchronize()
        if plan.status() != 0:
            raise RuntimeError("strided sweep: zero pivot reported")
    return e0.elapsed_time(e1) / sweeps


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description="sweeps of lines in an application's own (euler3d) layout")
    ap.add_argument("n", type=int, help="points per axis")
    ap.add_argument("m", type=int, help="block size")
    ap.add_argument("--axis", default="y", choices=["x", "y", "z"])
    ap.add_argument("--precision", default="ff", choices=["fp64", "ff"])
    ap.add_argument("--sweeps", type=int, default=3)
    args = ap.parse_args(argv)
    ms = sweep(args.n, args.m, args.axis, args.precision, args.sweeps)
    rows = args.n ** 3
    print(f"n={args.n} m={args.m} axis={args.axis} precision={args.precision}: {ms:.3f} ms/sweep, "
          f"{rows / ms / 1e6:.2f} G block rows/s")


if __name__ == "__main__":
    main()
