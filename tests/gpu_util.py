"""Helpers for the GPU parity tests: run the library on a workload through
the reference-style API (which calls the C ABI) and run the oracle on a copy."""
import numpy as np
import torch

import pascal_btdma_gb300 as pbt
from oracle import oracle as O


def to_dev(arrays, dev):
    return [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in arrays]


def gpu_solve(w, nseg=1, dev="cuda:0", cyclic=False, stream=None, **plan_kw):
    """Solve workload ``w`` on the GPU; returns (A, B, C, D) back on the host."""
    a, b, c, d = to_dev(w.arrays, dev)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(w.m, w.nsys, w.nrow, nseg, cyclic=cyclic, **plan_kw)
        fn = pbt.solve_cyclic if cyclic else pbt.solve_noncyclic
        fn(plan, a, b, c, d, w.m, w.nsys, w.nrow, stream=stream)
        singular = plan.status()
    return [t.cpu().numpy() for t in (a, b, c, d)], singular


def oracle_solve(w, nseg=1, cyclic=False):
    """The oracle on a copy of ``w``: the two-stage method, or for periodic
    lines in one segment, btdma_many_cycl on the whole line."""
    r = w.copy()
    if cyclic and nseg == 1:
        O.block_thomas_cyclic(w.m, w.nsys, w.nrow, *r.arrays)
        return r
    fn = O.solve_cyclic if cyclic else O.solve_noncyclic
    fn(w.m, w.nsys, w.nrow, nseg, *r.arrays)
    return r


def subset(w, systems):
    """The workload restricted to the given systems (systems are independent,
    so solving the subset is exactly solving those systems of the batch)."""
    from pascal_btdma_gb300.synth import Workload

    m, nsys, N = w.m, w.nsys, w.nrow
    sel = np.asarray(systems)

    def mat(x):
        return np.ascontiguousarray(x.reshape(m * m * N, nsys)[:, sel]).reshape(-1)

    def vec(x):
        return np.ascontiguousarray(x.reshape(m * N, nsys)[:, sel]).reshape(-1)

    return Workload(m, len(sel), N, mat(w.A), mat(w.B), mat(w.C), vec(w.D))


def column_subset(m, nsys, N, D, systems):
    return np.ascontiguousarray(D.reshape(m * N, nsys)[:, np.asarray(systems)]).reshape(-1)
