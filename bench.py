#!/usr/bin/env python3
"""Benchmark of the batched block-tridiagonal solve on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (the production pencil batch): nsys = 65536 independent systems
(a 256 x 256 pencil batch) of N = 256 block rows, block size m = 5, seeded
synthetic diagonally dominant data (delta = 1.2, A_0 = C_{N-1} = 0), one line
per system (P = 1).  A "step" is one solve of the whole batch: 16.8 M block
rows, 11.4 GB of FP64 input (> L2, so no flush is needed between steps).

Metric: block-rows/s (higher is better).  `value` times K solves on
device-resident data with CUDA events on the launching stream; `e2e` times
the same K solves through the public API with the inputs copied from pinned
host memory each step and the solution copied back.

The timed method is the chosen one, float-float arithmetic (precision
"ff"); `plain_fp64` is the same batch with plain FP64 arithmetic, and
`rel_err_vs_fp64` the chosen result's distance from it.

Extra keys: `roofline` (algorithmic bytes 8*(3m^2+2m) per block row over the
kernel time, against the measured HBM copy bandwidth; `traffic` = ncu DRAM
bytes per launch), `plain_fp64` (also against the FP64 FMA rate, which is
what binds plain FP64 on GB300), `cpu_baseline` (the oracle port of the
reference CPU path on the host cores, on a bounded sample), `variants` (the
two-stage P = 16 split of the same batch, the long-line case m = 4,
nsys = 256, N = 32768, P = 128, the small case m = 3, nsys = 1024,
N = 128, P = 4 timed with L2 flushed, and the pencil batch as periodic lines,
P = 2), `mixed_precision`, `adjoint`,
`uneven_batch`, `shared_lines` (one heat3d ADI step, three sweeps of
shared-matrix lines in place in a 516^3 haloed field, against the general
solver with pack/unpack), `strided_lines` (the y sweep of a 256^3 euler3d
layout field at m = 5 solved in the application's arrays against
transpose-solve-transpose), `clocks` (nvidia-smi sampled during the timed
region).
`--sections` limits the extra sections (e.g. `--sections main`).

Under torchrun (N > 1) every rank solves its own full batch (weak scaling,
no collective on the data path); the time is the max over ranks.

`--impl reference` times the reference algorithm's CPU path (the oracle port
of Fortran_Original/src/mod_btdma_cpu.f90; the Fortran original cannot be
built here) on all host cores, on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

M, NSYS, NROW, NSEG, DELTA, SEED = 5, 65536, 256, 1, 1.2, 20240101
VARIANTS = [  # name, m, nsys, nrow, nseg, delta, cyclic
    ("pencil_P16", 5, 65536, 256, 16, 1.2, False),
    ("long_lines_P128", 4, 256, 32768, 128, 1.2, False),
    ("small_P4", 3, 1024, 128, 4, 2.0, False),  # 34.6 MB: fits in L2, timed with L2 flushed before each solve
    ("pencil_cyclic_P1", 5, 65536, 256, 1, 1.2, True),  # periodic lines, one pass per line (k_thomas_cyclic)
    ("pencil_cyclic_P2", 5, 65536, 256, 2, 1.2, True),  # periodic lines (btdma_many_cycl), two segments
]
L2_FIT_BYTES = 256 << 20  # inputs below this are timed with an L2 flush before every solve
# DRAM bytes (read + write) per block row of k_thomas<FF,5> from ncu
# (dram__bytes_read.sum + dram__bytes_write.sum on a 65536-system, 32-row
# batch: 2.349 GB / 2,097,152 rows).  The factor workspace round trip (C'
# written forward, read back backward) and y make the excess over the
# algorithmic 680 B; it scales with the rows, so a full launch moves
# rows * this.
TRAFFIC_BYTES_PER_ROW = {5: 1120.0}
# Mixed precision: the pencil batch with every block row scaled by a
# log-uniform factor in [1e-3, 1e3]; FP32 factorisation + FP64 residual
# refinement, and float-float, each against the plain FP64 solution.
MIXED = [(1.05, 1), (1.05, 16), (1.5, 1), (1.5, 16)]  # (delta, nseg)
# Adjoint: m=4, nsys=16384, N=512, delta=1.5, forward and adjoint at P=8 and
# P=1; memory-pressure variant: nsys=262144 (the 16384-system batch tiled 16x
# on the device), factors recomputed by the adjoint.
ADJ = dict(m=4, nsys=16384, nrow=512, delta=1.5, segs=(8, 1), pressure_tiles=16)
# Uneven batch: 32768 systems, N log-uniform in [16, 4096], m uniform in
# {2, 3, 4, 5}, delta = 1.5; one persistent launch per block size and sweep,
# 100 sweeps in a CUDA graph; tuning by the autotuner; against one uniform
# plan per (m, power-of-two N bucket) with the systems padded to the bucket.
UNEVEN = dict(nsys=32768, nmin=16, nmax=4096, mmin=2, mmax=5, delta=1.5, sweeps=100)
# heat3d-style ADI step: a 512^3 field with a halo of 2, lines of 256 blocks of 2 points
SHARED = dict(n=512, halo=2, sigma=0.05, steps=5)
METRIC = "block-rows/s (chosen method at <=1e-10 rel err vs plain FP64)"
DATA = "synthetic (seeded Philox4x32-10, diagonally dominant, delta=1.2)"


def workload_config(ws: int) -> dict:
    """The `config` of both arms' JSON lines (the same workload)."""
    return {"workload": f"pencil batch m={M}, nsys={NSYS}, N={NROW}, P={NSEG}", "m": M, "nsys": NSYS,
            "nrow": NROW, "nseg": NSEG, "l2": "inputs 11.4 GB > L2 (no flush needed)",
            "parallelism": f"replicas x{ws}"}


def run_shared(dev) -> dict:
    """Shared-matrix lines (include/pbt_shared.h): the three sweeps of one
    heat3d ADI step solved in place in the haloed field, against one sweep of
    the general solver on the same lines packed into the reference layout
    (matrix replicated per line; pack and unpack by PyTorch copies)."""
    import torch

    import pascal_btdma_gb300 as pbt
    from pascal_btdma_gb300 import shared

    cfg = SHARED
    n, h = cfg["n"], cfg["halo"]
    nblk, m = n // 2, 2
    field = torch.rand((n + 2 * h,) * 3, dtype=torch.float64, device=dev)
    interior = field[h:-h, h:-h, h:-h]
    st = interior.stride()
    a, b, c = shared.heat3d_blocks(nblk, cfg["sigma"])
    rows = n * n * nblk  # block rows per sweep
    sweeps = []
    for axis in (2, 1, 0):  # x, y, z as heat3d orders them
        outer, inner = [x for x in range(3) if x != axis]
        sweeps.append(shared.Lines(n, n, st[inner], st[outer], 2 * st[axis], st[axis]))
    s0 = torch.cuda.current_stream()
    out = {"field": [n + 2 * h] * 3, "halo": h, "m": m, "nblk": nblk, "lines_per_sweep": n * n,
           "bytes_per_block_row": 4 * m * 8,
           "bytes_note": "rhs read, y written and read back, x written: 4*m doubles per block row per sweep"}
    for prec in ("ff", "fp64"):
        with shared.SharedMatrix(m, nblk, a, b, c, precision=prec) as sm:
            for L in sweeps:
                sm.solve(interior, interior, L)
            per = []
            for L in sweeps:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s0)
                for _ in range(cfg["steps"]):
                    sm.solve(interior, interior, L)
                e1.record(s0)
                torch.cuda.synchronize()
                per.append(e0.elapsed_time(e1) / 1e3 / cfg["steps"])
        gbs = [rows * out["bytes_per_block_row"] / t / 1e9 for t in per]
        out[prec] = {"ms_per_adi_step": sum(per) * 1e3,
                     "ms_per_sweep_xyz": [t * 1e3 for t in per],
                     "block_rows_per_s": 3 * rows / sum(per),
                     "algorithmic_gbs_xyz": gbs}
    # General solver on the z sweep's lines: pack, solve (FF), unpack.
    nsys = n * n
    rep = [torch.from_numpy(x).to(dev).view(-1, 1).expand(-1, nsys).contiguous().view(-1) for x in (a, b, c)]
    d = torch.empty(m * nblk * nsys, dtype=torch.float64, device=dev)
    with pbt.BtdmaGpuPlan() as pl:
        pl.create(m, nsys, nblk, 1, precision="ff")

        def general_sweep():
            # field axis 0 -> (point = 2q + i, s_out, s_in) -> reference layout sys + nsys*(q + nblk*i)
            d.view(m, nblk, n, n).copy_(interior.unflatten(0, (nblk, m)).permute(1, 0, 2, 3))
            pbt.solve_noncyclic(pl, *rep, d, m, nsys, nblk)
            interior.unflatten(0, (nblk, m)).copy_(d.view(m, nblk, n, n).permute(1, 0, 2, 3))

        general_sweep()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s0)
        for _ in range(cfg["steps"]):
            general_sweep()
        e1.record(s0)
        torch.cuda.synchronize()
        gen = e0.elapsed_time(e1) / 1e3 / cfg["steps"]
    out["general_ff_pack_solve_unpack_ms_per_sweep"] = gen * 1e3
    out["speedup_ff_vs_general_ff"] = gen / (out["ff"]["ms_per_adi_step"] / 3e3)
    del field, interior, rep, d
    torch.cuda.empty_cache()
    return out


def run_lines(dev) -> dict:
    """Strided lines (pbt_solve_noncyclic_lines): the y sweep of an euler3d
    layout field, U(n1,n2,n3,m) and trA(n1,n2,n3,m,m) with n = 256, m = 5
    (the headline's 65536 lines of 256 rows), solved in the application's
    arrays, against the reference application's route: transpose A, B, C, D
    into the solver layout, solve, transpose D back (PyTorch copies)."""
    import torch

    import pascal_btdma_gb300 as pbt
    from pascal_btdma_gb300 import synth

    n, m = 256, 5
    nsys, nrow = n * n, n
    w = synth.dominant(m, nsys, nrow, seed=SEED, delta=DELTA)
    # packed [e, row = j, s_out = k, s_in = i] -> application [e, k, j, i]
    app = [torch.from_numpy(x).to(dev).view(-1, n, n, n).transpose(1, 2).contiguous() for x in w.arrays]
    lines = pbt.Lines(n, n, 1, n * n, n, n * n * n)
    out = {"field": [n, n, n], "m": m, "sweep": "y (lines over i, k; rows along j)", "lines": nsys, "rows": nrow}
    steps = 5
    for prec in ("ff", "fp64"):
        d0 = app[3].clone()
        with pbt.BtdmaGpuPlan() as pl:
            pl.create(m, nsys, nrow, 1, precision=prec)
            bufs = [d0.clone() for _ in range(steps + 1)]
            pbt.solve_noncyclic_lines(pl, *app[:3], bufs[-1], lines)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for k in range(steps):
                pbt.solve_noncyclic_lines(pl, *app[:3], bufs[k], lines)
            e1.record()
            torch.cuda.synchronize()
            t_lines = e0.elapsed_time(e1) / steps
            packed = [torch.empty(x.numel(), dtype=torch.float64, device=dev) for x in app]

            def transposed_sweep(dk):
                for src, dst in zip(app[:3] + [dk], packed):
                    dst.view(-1, n, n, n).copy_(src.transpose(1, 2))
                pbt.solve_noncyclic(pl, *packed, m, nsys, nrow)
                dk.copy_(packed[3].view(-1, n, n, n).transpose(1, 2))

            transposed_sweep(bufs[-1])
            torch.cuda.synchronize()
            e0.record()
            for k in range(steps):
                transposed_sweep(bufs[k])
            e1.record()
            torch.cuda.synchronize()
            t_tr = e0.elapsed_time(e1) / steps
            del packed
        out[prec] = {"lines_ms": t_lines, "transpose_solve_transpose_ms": t_tr, "speedup": t_tr / t_lines,
                     "block_rows_per_s": nsys * nrow / (t_lines / 1e3)}
        del bufs, d0
    del app
    torch.cuda.empty_cache()
    return out


def run_uneven(dev, log=None) -> dict:
    import torch

    import pascal_btdma_gb300 as pbt
    from pascal_btdma_gb300 import batch as B
    from pascal_btdma_gb300 import synth

    u = UNEVEN
    n, m = synth.uneven_shapes(SEED, u["nsys"], u["nmin"], u["nmax"], u["mmin"], u["mmax"])
    A, Bm, Cm, D, mo, vo = synth.fill_batch(m, n, seed=SEED, delta=u["delta"])
    user = tuple(torch.from_numpy(x).to(dev) for x in (A, Bm, Cm, D))
    rows = int(n.sum())
    out = {"nsys": u["nsys"], "block_rows": rows, "distinct_m_n": int(len(set(zip(m.tolist(), n.tolist()))))}
    for prec in ("fp64", "ff"):
        tuning = B.autotune(m, n, user, prec, log=log)
        plan = B.BatchPlan(m, n, prec, tuning)
        packed = plan.pack(*user)
        d0 = packed[3].clone()
        g = B.capture_sweeps(plan, packed, d0, sweeps=u["sweeps"])
        g.replay()  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        plan.status()
        t = e0.elapsed_time(e1) / 1e3 / u["sweeps"]
        # The same sweeps launched one by one (no graph).
        pa, pb, pc, pd = packed
        e0.record()
        for _ in range(5):
            pd.copy_(d0)
            plan.solve(pa, pb, pc, pd)
        e1.record()
        torch.cuda.synchronize()
        plan.status()
        te = e0.elapsed_time(e1) / 1e3 / 5
        out[prec] = {"block_rows_per_s": rows / t, "ms_per_sweep": t * 1e3, "ms_per_sweep_no_graph": te * 1e3,
                     "tuning": tuning, **plan.info()}
        plan.destroy()
        del packed, d0, g
    # The comparator a user of the plain plan API would build: one uniform plan
    # per (m, N bucket), N buckets of powers of two, every system padded to its
    # bucket's N with rows that decouple (B = I, A = C = 0, d = 0; the last
    # real row's C zeroed, as the non-cyclic solve treats it).  The groups'
    # solves run concurrently, one stream each, timed with CUDA events; one
    # segment per line, or segments of ~256 rows for the long buckets.
    import math

    groups = {}
    for s in range(u["nsys"]):
        nb = 1 << max(1, math.ceil(math.log2(int(n[s]))))
        groups.setdefault((int(m[s]), nb), []).append(s)
    padded = []
    for (mm, nb), idx in sorted(groups.items()):
        blocks = [[], [], [], []]
        for s in idx:
            ns = int(n[s])
            o, ov = int(mo[s]), int(vo[s])
            a_ = user[0][o:o + ns * mm * mm].view(mm * mm, ns)
            b_ = user[1][o:o + ns * mm * mm].view(mm * mm, ns)
            c_ = user[2][o:o + ns * mm * mm].view(mm * mm, ns).clone()
            d_ = user[3][ov:ov + ns * mm].view(mm, ns)
            c_[:, ns - 1] = 0.0
            pad = nb - ns
            eye = torch.zeros(mm * mm, pad, dtype=torch.float64, device=dev)
            eye[[i + mm * i for i in range(mm)], :] = 1.0
            z2 = torch.zeros(mm * mm, pad, dtype=torch.float64, device=dev)
            blocks[0].append(torch.cat([a_, z2], 1))
            blocks[1].append(torch.cat([b_, eye], 1))
            blocks[2].append(torch.cat([c_, z2], 1))
            blocks[3].append(torch.cat([d_, torch.zeros(mm, pad, dtype=torch.float64, device=dev)], 1))
        arrs = [torch.stack(bl, 2).contiguous().view(-1) for bl in blocks]  # (e, row, sys): reference layout
        padded.append((mm, nb, len(idx), arrs))
    torch.cuda.synchronize()
    padded_rows = sum(nb * k for _, nb, k, _ in padded)
    main = torch.cuda.current_stream()
    streams = [torch.cuda.Stream() for _ in padded]
    for prec in ("fp64", "ff"):
        for segmented in (False, True):
            plans, work = [], []
            for mm, nb, k, arrs in padded:
                P = max(1, nb // 256) if segmented else 1
                plans.append(pbt.BtdmaGpuPlan().create(mm, k, nb, P, precision=prec))
                work.append(arrs[3].clone())

            def sweep():
                for pl, (mm, nb, k, arrs), w_, st in zip(plans, padded, work, streams):
                    st.wait_stream(main)
                    with torch.cuda.stream(st):
                        w_.copy_(arrs[3])
                        pbt.solve_noncyclic(pl, arrs[0], arrs[1], arrs[2], w_, mm, k, nb, stream=st)
                for st in streams:
                    main.wait_stream(st)

            sweep()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = 5
            e0.record(main)
            for _ in range(reps):
                sweep()
            e1.record(main)
            torch.cuda.synchronize()
            for pl in plans:
                pl.status()
                pl.destroy()
            t = e0.elapsed_time(e1) / 1e3 / reps
            key = f"grouped_plans_{prec}" + ("_segmented" if segmented else "")
            out[key] = {"block_rows_per_s": rows / t, "ms_per_sweep": t * 1e3, "plans": len(padded),
                        "padded_block_rows": padded_rows, "streams": len(streams),
                        "nseg": "max(1, N_bucket // 256)" if segmented else 1}
            del work
    out["ff_over_fp64"] = out["fp64"]["ms_per_sweep"] / out["ff"]["ms_per_sweep"]
    del padded, user
    torch.cuda.empty_cache()
    return out


def bytes_per_row(m: int, width: int = 8) -> int:
    """Algorithmic bytes per block row: A, B, C, d read once, x written once."""
    return width * (3 * m * m + 2 * m)


def fp64_flops_per_row_thomas(m: int) -> float:
    """FP64 flops per block row of the plain block Thomas recurrence:
    R = B - A C' (2m^3), d - A y (2m^2), LU with partial pivoting
    (2m^3/3 - m^2/2 - m/6 ... ~2m^3/3), m+1 right-hand sides (2m^2(m+1)),
    back substitution x = y - C'x (2m^2)."""
    return 2 * m**3 + 2 * m**2 + (2 * m**3) / 3 + 2 * m**2 * (m + 1) + 2 * m**2


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int, dev) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port of the reference CPU path, bounded sample.
# ---------------------------------------------------------------------------
def cpu_baseline(m: int, nrow: int, nseg: int, delta: float, target_s: float = 12.0) -> dict:
    from oracle import oracle as O
    from pascal_btdma_gb300 import synth

    threads = O.default_threads()

    def run(nsys_s):
        w = synth.dominant(m, nsys_s, nrow, seed=SEED, delta=delta)
        c = [O.gpu_to_cpu(m, nsys_s, nrow, k < 3, x) for k, x in enumerate(w.arrays)]
        t0 = time.perf_counter()
        O.solve_noncyclic_cpu(m, nsys_s, nrow, nseg, *c, nthreads=threads)
        return time.perf_counter() - t0

    n = max(threads * 8, 256)
    dt = run(n)
    while dt < 0.5 and n < NSYS:
        n = min(NSYS, n * 4)
        dt = run(n)
    n_final = int(min(NSYS, max(n, n * target_s / max(dt, 1e-6))))
    dt = run(n_final)
    rows = n_final * nrow
    return {"value": rows / dt, "unit": "block-rows/s", "cores": threads, "kind": "port",
            "sample": f"{n_final} systems x {nrow} rows, m={m}, P={nseg}, oracle C port of mod_btdma_cpu "
                      f"(CPU layout), {dt:.2f} s on {threads} threads"}


# ---------------------------------------------------------------------------
# Our arm.
# ---------------------------------------------------------------------------
def residual_error(a, b, c, d, x, m, nsys, nrow) -> float:
    """max over systems of |d - M x|_inf / (|M|_inf |x|_inf + |d|_inf)."""
    import torch

    A = a.view(m, m, nrow, nsys)  # [j, i, row, sys]
    B = b.view(m, m, nrow, nsys)
    C = c.view(m, m, nrow, nsys)
    X = x.view(m, nrow, nsys)     # [j, row, sys]
    r = d.view(m, nrow, nsys).clone()
    for j in range(m):            # elementwise products: a handful of kernels, no per-system GEMV
        r -= B[j] * X[j].unsqueeze(0)
        r[:, 1:] -= A[j, :, 1:] * X[j, :-1].unsqueeze(0)
        r[:, :-1] -= C[j, :, :-1] * X[j, 1:].unsqueeze(0)
    rowabs = B.abs().sum(0) + A.abs().sum(0) + C.abs().sum(0)  # [i, row, sys]
    mnorm = rowabs.amax(dim=(0, 1))
    num = r.abs().amax(dim=(0, 1))
    den = mnorm * X.abs().amax(dim=(0, 1)) + d.view(m, nrow, nsys).abs().amax(dim=(0, 1))
    return float((num / den).max())


def make_workload(m, nsys, nrow, delta, dev, pinned=False, row_scale=False):
    import torch

    from pascal_btdma_gb300 import synth

    alloc = None
    keep = []
    if pinned:
        def alloc(n):
            t = torch.empty(n, dtype=torch.float64, pin_memory=True)
            keep.append(t)
            return t.numpy()
    w = synth.dominant(m, nsys, nrow, seed=SEED, delta=delta, alloc=alloc, row_scale=row_scale)
    return w, keep


def time_device(plan, arrs, dpool, m, nsys, nrow, steps, warmup, ws, dev, solve):
    """K solves on device-resident inputs; each step gets its own fresh RHS."""
    import torch

    a, b, c = arrs
    stream = torch.cuda.current_stream()
    for i in range(warmup):
        solve(plan, a, b, c, dpool[i % len(dpool)].clone(), m, nsys, nrow)
    work = [dpool[i % len(dpool)].clone() for i in range(steps)]
    torch.cuda.synchronize()
    barrier(ws)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for i in range(steps):
        solve(plan, a, b, c, work[i], m, nsys, nrow)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    ms = ev0.elapsed_time(ev1)
    return ms / 1e3


def time_device_flushed(plan, arrs, d0, m, nsys, nrow, steps, warmup, dev, solve):
    """Like time_device for inputs that fit in L2: before every solve a
    buffer larger than L2 is overwritten, and only the solve is timed (events
    around each solve, summed)."""
    import torch

    a, b, c = arrs
    scratch = torch.empty(L2_FIT_BYTES // 2, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        solve(plan, a, b, c, d0.clone(), m, nsys, nrow)
    work = [d0.clone() for _ in range(steps)]
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        scratch.fill_(float(i))
        evs[i][0].record(stream)
        solve(plan, a, b, c, work[i], m, nsys, nrow)
        evs[i][1].record(stream)
    torch.cuda.synchronize()
    return sum(e0.elapsed_time(e1) for e0, e1 in evs) / 1e3


def rel_err_vs(x, ref, m, nsys, nrow) -> float:
    """max over systems of max|x - ref| / max|ref| (GPU tensors)."""
    X = x.view(m, nrow, nsys)
    Rf = ref.view(m, nrow, nsys)
    return float(((X - Rf).abs().amax(dim=(0, 1)) / Rf.abs().amax(dim=(0, 1))).max())


def run_ours(args):
    import torch

    import pascal_btdma_gb300 as pbt
    from pascal_btdma_gb300 import synth

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)
    peaks = load_peaks()
    from pascal_btdma_gb300.peaks import fma_rates

    fma = fma_rates()
    m, nsys, nrow, nseg = M, NSYS, NROW, NSEG
    solve = pbt.solve_noncyclic
    rows = nsys * nrow

    # Inputs: pinned host copy (for e2e) and a device copy (for `value`).
    w, keep = make_workload(m, nsys, nrow, DELTA, dev, pinned=True)
    hA, hB, hC, hD = (torch.from_numpy(x) for x in w.arrays)
    a, b, c = (t.to(dev) for t in (hA, hB, hC))
    d0 = hD.to(dev)
    plans = {p: pbt.BtdmaGpuPlan().create(m, nsys, nrow, nseg, precision=p) for p in ("fp64", "ff")}

    # Accuracy on this very batch: FP64 (parity-tested against the oracle)
    # gives the reference solution; the chosen FF result is compared with it.
    x64 = d0.clone()
    solve(plans["fp64"], a, b, c, x64, m, nsys, nrow)
    xff = d0.clone()
    solve(plans["ff"], a, b, c, xff, m, nsys, nrow)
    rel_err = rel_err_vs(xff, x64, m, nsys, nrow)
    backward_err = residual_error(a, b, c, d0, x64, m, nsys, nrow)
    del x64, xff

    # Device-resident timing (`value`, the chosen FF method) with clocks
    # sampled during it; then plain FP64 the same way.
    clk = ClockSampler(local)
    clk.start()
    secs = time_device(plans["ff"], (a, b, c), [d0], m, nsys, nrow, args.steps, args.warmup, ws, dev, solve)
    clocks = clk.stop()
    secs = max_over_ranks(secs, ws, dev)
    secs64 = time_device(plans["fp64"], (a, b, c), [d0], m, nsys, nrow, args.steps, args.warmup, ws, dev, solve)
    secs64 = max_over_ranks(secs64, ws, dev)
    value = ws * rows * args.steps / secs
    kern_s = secs / args.steps          # one launch per solve at P = 1
    kern64_s = secs64 / args.steps
    achieved = rows * bytes_per_row(m) / kern_s / 1e9
    achieved64 = rows * bytes_per_row(m) / kern64_s / 1e9

    # End to end through the public API: every step copies its A, B, C, D from
    # pinned host memory, solves, and copies x back.  As a caller streaming
    # batches would, two plans and two device buffer sets alternate on two
    # streams, so one step's solve and D2H overlap the next step's H2D (the
    # host link, ~211 GB/s H2D on this system, is the bound).
    out_h = [torch.empty_like(hD).pin_memory() for _ in range(2)]
    dev_sets = [(a, b, c, d0)] + [tuple(torch.empty_like(t) for t in (a, b, c, d0))]
    e2e_plans = [plans["ff"], pbt.BtdmaGpuPlan().create(m, nsys, nrow, nseg, precision="ff")]
    e2e_streams = [torch.cuda.Stream(), torch.cuda.Stream()]

    def e2e_step(i):
        k = i % 2
        sa, sb, sc, sd = dev_sets[k]
        with torch.cuda.stream(e2e_streams[k]):
            sa.copy_(hA, non_blocking=True)
            sb.copy_(hB, non_blocking=True)
            sc.copy_(hC, non_blocking=True)
            sd.copy_(hD, non_blocking=True)
            solve(e2e_plans[k], sa, sb, sc, sd, m, nsys, nrow, stream=e2e_streams[k])
            out_h[k].copy_(sd, non_blocking=True)

    st = torch.cuda.current_stream()
    for i in range(2):
        e2e_step(i)
    torch.cuda.synchronize()
    barrier(ws)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for s_ in e2e_streams:
        s_.wait_event(e0)
    for i in range(args.steps):
        e2e_step(i)
    for s_ in e2e_streams:
        st.wait_stream(s_)
    e1.record(st)
    torch.cuda.synchronize()
    barrier(ws)
    e2e_s = max_over_ranks(e0.elapsed_time(e1) / 1e3, ws, dev)
    h2d = 3 * hA.numel() * 8 + hD.numel() * 8
    d2h = hD.numel() * 8
    e2e_plans[1].destroy()
    del dev_sets, e2e_streams

    # Variants: the two-stage split and the long lines, both arithmetics.
    variants = {}
    for p in plans.values():
        p.destroy()
    del a, b, c, d0, hA, hB, hC, hD, keep, w, out_h
    torch.cuda.empty_cache()
    for name, vm, vns, vn, vp, vdelta, vcyc in (VARIANTS if "variants" in args.sections else []):
        if vcyc:
            vw = synth.fill(synth.DOMINANT, vm, vns, vn, seed=SEED, delta=vdelta, flags=0)  # A_0, C_{N-1} couple the ends
        else:
            vw, _ = make_workload(vm, vns, vn, vdelta, dev)
        vsolve = pbt.solve_cyclic if vcyc else solve
        va, vb, vc, vd = (torch.from_numpy(x).to(dev) for x in vw.arrays)
        vrows = vns * vn
        fills = vns >= 128 * torch.cuda.get_device_properties(dev).multi_processor_count
        entry = {"m": vm, "nsys": vns, "nrow": vn, "nseg": vp, "cyclic": vcyc,
                 "default_plan_solves_as": (f"{vp} segments" if vp > 1 and not fills else "one segment per line"),
                 "l2": "flushed before each solve" if vrows * bytes_per_row(vm) < L2_FIT_BYTES else "inputs > L2"}
        xs = {}
        # With nseg > 1 a batch that fills the GPU is solved one segment per
        # line; "<prec>_segmented" keeps the nseg segments (the two-stage
        # method, PBT_FLAG_REFERENCE_METHOD).
        modes = [(p_, False) for p_ in ("ff", "fp64")] + ([(p_, True) for p_ in ("ff", "fp64")] if vp > 1 else [])
        for prec, segmented in modes:
            key = prec + ("_segmented" if segmented else "")
            vplan = pbt.BtdmaGpuPlan().create(vm, vns, vn, vp, precision=prec, cyclic=vcyc,
                                              reference_method=segmented)
            ksteps = max(3, args.steps // 2)
            small = vrows * bytes_per_row(vm) < L2_FIT_BYTES
            if small:
                vs = time_device_flushed(vplan, (va, vb, vc), vd, vm, vns, vn, ksteps, 3, dev, vsolve)
            else:
                vs = time_device(vplan, (va, vb, vc), [vd], vm, vns, vn, ksteps, 3, ws, dev, vsolve)
            vs = max_over_ranks(vs, ws, dev)
            xs[key] = vd.clone()
            if vcyc:
                vsolve(vplan, va, vb, vc, xs[key], vm, vns, vn)
                t = None
            else:
                t = pbt.solve_noncyclic_profiled(vplan, va, vb, vc, xs[key], vm, vns, vn)
            entry[key] = {
                "block_rows_per_s": ws * vrows * ksteps / vs,
                "ms_per_step": vs / ksteps * 1e3,
                "algorithmic_gbs": vrows * bytes_per_row(vm) / (vs / ksteps) / 1e9,
                "phases_ms": None if t is None else {"local": t.local_compute * 1e3,
                                                     "reduced": t.reduced_compute * 1e3,
                                                     "update": t.update_compute * 1e3},
            }
            vplan.destroy()
        entry["ff_rel_err_vs_fp64"] = rel_err_vs(xs["ff"], xs["fp64"], vm, vns, vn)
        if vp > 1:
            entry["ff_segmented_rel_err_vs_fp64"] = rel_err_vs(xs["ff_segmented"], xs["fp64"], vm, vns, vn)
        variants[name] = entry
        del va, vb, vc, vd, vw, xs
        torch.cuda.empty_cache()

    mixed = {}
    by_delta = {}
    for delta, nseg_m in (MIXED if "mixed" in args.sections else []):
        by_delta.setdefault(delta, []).append(nseg_m)
    for delta, segs in by_delta.items():
        mw, _ = make_workload(M, NSYS, NROW, delta, dev, row_scale=True)
        ma, mb, mc, md = (torch.from_numpy(x).to(dev) for x in mw.arrays)
        mrows = NSYS * NROW
        for nseg_m in segs:
            fills = NSYS >= 128 * torch.cuda.get_device_properties(dev).multi_processor_count
            entry = {"delta": delta, "nseg": nseg_m, "row_scale": "log-uniform [1e-3, 1e3]",
                     "default_plan_solves_as": (f"{nseg_m} segments" if nseg_m > 1 and not fills
                                                else "one segment per line")}
            ref = md.clone()
            with pbt.BtdmaGpuPlan() as p64:
                p64.create(M, NSYS, NROW, nseg_m, precision="fp64")
                solve(p64, ma, mb, mc, ref, M, NSYS, NROW)
            modes = [(p_, False) for p_ in ("fp32_refine", "ff")]
            if nseg_m > 1:
                modes += [(p_, True) for p_ in ("fp32_refine", "ff", "fp64")]
            for prec, segmented in modes:
                key = prec + ("_segmented" if segmented else "")
                with pbt.BtdmaGpuPlan() as pl:
                    pl.create(M, NSYS, NROW, nseg_m, precision=prec, tol=1e-12, max_iter=8,
                              reference_method=segmented)
                    ms = time_device(pl, (ma, mb, mc), [md], M, NSYS, NROW, 3, 3, ws, dev, solve)
                    ms = max_over_ranks(ms, ws, dev)
                    xo = md.clone()
                    solve(pl, ma, mb, mc, xo, M, NSYS, NROW)
                    info = pl.refine_info() if prec == "fp32_refine" else (None, None)
                entry[key] = {"block_rows_per_s": ws * mrows * 3 / ms, "ms_per_step": ms / 3 * 1e3,
                              "rel_err_vs_fp64": rel_err_vs(xo, ref, M, NSYS, NROW)}
                if prec == "fp32_refine":
                    entry[key]["fp32_solves"] = info[0]
                    entry[key]["last_correction"] = info[1]
                del xo
            mixed[f"delta{delta}_P{nseg_m}"] = entry
            del ref
        del ma, mb, mc, md, mw
        torch.cuda.empty_cache()

    adjoint = {}
    if "adjoint" in args.sections:
        aw, _ = make_workload(ADJ["m"], ADJ["nsys"], ADJ["nrow"], ADJ["delta"], dev)
        am, an, anr = ADJ["m"], ADJ["nsys"], ADJ["nrow"]
        A0, B0, C0, D0 = (torch.from_numpy(x).to(dev) for x in aw.arrays)

        def time_adjoint(plan, A_, B_, C_, D_, m_, ns_, nr_, k):
            x_ = D_.clone()
            solve(plan, A_, B_, C_, x_, m_, ns_, nr_)
            gsrc = torch.ones_like(D_)
            da_, db_, dc_ = torch.empty_like(A_), torch.empty_like(B_), torch.empty_like(C_)
            lam_ = gsrc.clone()
            for _ in range(2):
                lam_.copy_(gsrc)
                pbt.adjoint_noncyclic(plan, A_, B_, C_, x_, lam_, da_, db_, dc_)
            torch.cuda.synchronize()
            bufs = [gsrc.clone() for _ in range(k)]
            st_ = torch.cuda.current_stream()
            e0_, e1_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0_.record(st_)
            for i_ in range(k):
                pbt.adjoint_noncyclic(plan, A_, B_, C_, x_, bufs[i_], da_, db_, dc_)
            e1_.record(st_)
            torch.cuda.synchronize()
            return e0_.elapsed_time(e1_) / 1e3 / k

        for nseg_a in ADJ["segs"]:
            for prec in ("ff", "fp64"):
                with pbt.BtdmaGpuPlan() as pl:
                    pl.create(am, an, anr, nseg_a, precision=prec)
                    fs = time_device(pl, (A0, B0, C0), [D0], am, an, anr, 3, 3, ws, dev, solve) / 3
                    ad = time_adjoint(pl, A0, B0, C0, D0, am, an, anr, 3)
                adjoint[f"{prec}_P{nseg_a}"] = {"forward_ms": fs * 1e3, "adjoint_ms": ad * 1e3,
                                                "adjoint_over_forward": ad / fs,
                                                "fused": nseg_a == 1 and am <= 6}
        # memory pressure: 262144 systems, adjoint recomputes the factorisation
        tiles = ADJ["pressure_tiles"]
        ns_p = an * tiles

        def tile(t, w_):
            return t.view(-1, an).repeat(1, tiles).contiguous().view(-1)

        Ap, Bp, Cp, Dp = (tile(t, aw) for t in (A0, B0, C0, D0))
        del A0, B0, C0, D0
        with pbt.BtdmaGpuPlan() as pl:
            pl.create(am, ns_p, anr, 1, precision="ff")
            fs = time_device(pl, (Ap, Bp, Cp), [Dp], am, ns_p, anr, 2, 3, ws, dev, solve) / 2
            ad = time_adjoint(pl, Ap, Bp, Cp, Dp, am, ns_p, anr, 2)
        adjoint["ff_P1_nsys262144"] = {"forward_ms": fs * 1e3, "adjoint_ms": ad * 1e3,
                                       "adjoint_over_forward": ad / fs, "fused": True,
                                       "device_bytes_inputs": 8 * (3 * am * am + am) * ns_p * anr}
        del Ap, Bp, Cp, Dp, aw
        torch.cuda.empty_cache()
    uneven = run_uneven(dev) if "uneven" in args.sections else {}
    shared_lines = run_shared(dev) if "shared" in args.sections else {}
    strided_lines = run_lines(dev) if "lines" in args.sections else {}

    result = {
        "metric": METRIC,
        "value": value,
        "unit": "block-rows/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 data, float-float (2 x f32) arithmetic",
        "data": DATA,
        "config": workload_config(ws),
        "method": "block Thomas, pivoted LU, float-float arithmetic (precision='ff')",
        "rel_err_vs_fp64": rel_err,
        "fp64_backward_err": backward_err,
        "plain_fp64": {"value": ws * rows * args.steps / secs64, "ms_per_step": kern64_s * 1e3,
                       "algorithmic_gbs": achieved64, "hbm_frac": achieved64 / peaks["hbm_gbs"],
                       "fp64_tflops": rows * fp64_flops_per_row_thomas(m) / kern64_s / 1e12,
                       "fp64_pipe_frac": rows * fp64_flops_per_row_thomas(m) / kern64_s / (2 * fma["fp64_fma_per_s"])},
        "speedup_vs_plain_fp64": secs64 / secs,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"],
                     "traffic": TRAFFIC_BYTES_PER_ROW[m] * rows if m in TRAFFIC_BYTES_PER_ROW else None,
                     "traffic_note": "ncu dram bytes per row on a 65536 x 32 batch, scaled to this launch's rows",
                     "peak_source": peaks["source"], "bytes_per_row": bytes_per_row(m),
                     "kernel": f"k_thomas<FF,{m}>"},
        "fma_rates": fma,
        "e2e": {"value": ws * rows * args.steps / e2e_s, "unit": "block-rows/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_s / args.steps * 1e3,
                "pipelining": "2 streams, 2 plans, 2 device buffer sets; step i+1's H2D overlaps step i's solve + D2H"},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "variants": variants,
        "mixed_precision": mixed,
        "adjoint": adjoint,
        "uneven_batch": uneven,
        "shared_lines": shared_lines,
        "strided_lines": strided_lines,
    }
    if rank == 0:
        if "cpu" in args.sections:
            result["cpu_baseline"] = cpu_baseline(m, nrow, nseg, DELTA, target_s=args.cpu_seconds)
        print(json.dumps(result), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_case(args):
    """One workload, for profiler captures and size sweeps: --case
    m,nsys,nrow,nseg[,cyclic][,precision][,segmented] runs W + K solves of it on cuda:0
    (each on a fresh right-hand side) and prints ms per solve.  Not a bench
    line: the headline and its sections are run_ours."""
    import torch

    import pascal_btdma_gb300 as pbt
    from pascal_btdma_gb300 import synth

    parts = args.case.split(",")
    m, nsys, nrow, nseg = (int(x) for x in parts[:4])
    cyclic = len(parts) > 4 and parts[4] in ("1", "cyclic", "true")
    prec = parts[5] if len(parts) > 5 else "ff"
    segmented = len(parts) > 6 and parts[6] in ("1", "segmented", "true")
    dev = torch.device("cuda:0")
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=SEED, delta=DELTA, flags=0 if cyclic else synth.ZERO_ENDS)
    a, b, c, d = (torch.from_numpy(x).to(dev) for x in w.arrays)
    solve = pbt.solve_cyclic if cyclic else pbt.solve_noncyclic
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, nseg, precision=prec, cyclic=cyclic, reference_method=segmented)
        t = time_device(plan, (a, b, c), [d], m, nsys, nrow, args.steps, args.warmup, 1, dev, solve)
        plan.status()
    rows = nsys * nrow
    print(json.dumps({"case": {"m": m, "nsys": nsys, "nrow": nrow, "nseg": nseg, "cyclic": cyclic,
                               "precision": prec, "segmented": segmented}, "ms_per_solve": t / args.steps * 1e3,
                      "block_rows_per_s": rows * args.steps / t,
                      "algorithmic_gbs": rows * bytes_per_row(m) * args.steps / t / 1e9}), flush=True)


def run_batch_case(args):
    """The bench's uneven batch restricted to one block size, for profiler
    captures: --batch-case m,seg_len[,precision] runs W + K sweeps (D restored
    before each) and prints ms per sweep.  Not a bench line."""
    import torch

    from pascal_btdma_gb300 import batch as B
    from pascal_btdma_gb300 import synth

    parts = args.batch_case.split(",")
    mm, seg = int(parts[0]), int(parts[1])
    prec = parts[2] if len(parts) > 2 else "ff"
    u = UNEVEN
    n_all, m_all = synth.uneven_shapes(SEED, u["nsys"], u["nmin"], u["nmax"], u["mmin"], u["mmax"])
    sel = m_all == mm
    m, n = m_all[sel], n_all[sel]
    A, Bm, Cm, D, _, _ = synth.fill_batch(m, n, seed=SEED, delta=u["delta"])
    user = tuple(torch.from_numpy(x).to("cuda") for x in (A, Bm, Cm, D))
    plan = B.BatchPlan(m, n, prec, {"seg_len": {mm: seg}, "warps_per_cta": 4})
    pa, pb, pc, pd = plan.pack(*user)
    d0 = pd.clone()
    for _ in range(args.warmup):
        pd.copy_(d0)
        plan.solve(pa, pb, pc, pd)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        pd.copy_(d0)
        plan.solve(pa, pb, pc, pd)
    e1.record()
    torch.cuda.synchronize()
    plan.status()
    print(json.dumps({"batch_case": {"m": mm, "seg_len": seg, "precision": prec, "systems": int(sel.sum()),
                                     "block_rows": int(n.sum())}, **plan.info(),
                      "ms_per_sweep": e0.elapsed_time(e1) / args.steps}), flush=True)
    plan.destroy()


def run_reference(args):
    """The reference algorithm's CPU path on the host cores, a bounded sample per step."""
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle as O
    from pascal_btdma_gb300 import synth

    threads = O.default_threads()
    m, nrow, nseg = M, NROW, NSEG
    nsys_s = 16384
    w = synth.dominant(m, nsys_s, nrow, seed=SEED, delta=DELTA)
    cpu = [O.gpu_to_cpu(m, nsys_s, nrow, k < 3, x) for k, x in enumerate(w.arrays)]
    times = []
    for i in range(args.warmup + args.steps):
        arrs = [x.copy() for x in cpu]
        t0 = time.perf_counter()
        O.solve_noncyclic_cpu(m, nsys_s, nrow, nseg, *arrs, nthreads=threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    secs = sum(times)
    rows = nsys_s * nrow
    value = rows * args.steps / secs
    sample = (f"{nsys_s} of the {NSYS} systems per step (m={m}, N={nrow}, P={nseg}); oracle C port of "
              f"mod_btdma_cpu on {threads} threads")
    print(json.dumps({
        "impl": "reference",
        "metric": METRIC,
        "value": value, "unit": "block-rows/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": workload_config(ws),
        "method": "the reference's CPU path (oracle C port of mod_btdma_cpu: block Thomas, LAPACK-style dgesv), FP64",
        "cpu_baseline": {"value": value, "unit": "block-rows/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "block-rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--sections", default="all",
                    help="comma list of extra sections to run beside the headline: variants, mixed, adjoint, "
                         "uneven, shared, lines, cpu; 'all' (default) or 'main' (headline only)")
    ap.add_argument("--case", default="",
                    help="m,nsys,nrow,nseg[,cyclic][,precision][,segmented]: time one workload only (profiler captures)")
    ap.add_argument("--batch-case", default="",
                    help="m,seg_len[,precision]: the uneven batch's systems of block size m only (profiler captures)")
    args = ap.parse_args()
    if args.case:
        run_case(args)
        return
    if args.batch_case:
        run_batch_case(args)
        return
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    known = {"variants", "mixed", "adjoint", "uneven", "shared", "lines", "cpu"}
    if args.sections == "all":
        args.sections = known
    elif args.sections == "main":
        args.sections = set()
    else:
        args.sections = set(args.sections.split(","))
        if not args.sections <= known:
            ap.error(f"unknown sections {sorted(args.sections - known)}")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
