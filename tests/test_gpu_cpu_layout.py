"""Plans with PBT_FLAG_CPU_LAYOUT take A, B, C, D in the reference CPU
layout a(m, m, nsys, n), d(m, nsys, n) (Fortran_Original/src/mod_btdma_cpu.f90:18-19)
and must return exactly what the same plan without the flag returns on the
same systems in the GPU layout; the oracle's CPU-layout solve bounds both."""
import numpy as np
import pytest
import torch

import pascal_btdma_gb300 as pbt
from pascal_btdma_gb300 import synth
from conftest import per_system_relerr
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def run(w, arrays, nseg, **kw):
    a, b, c, d = (torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0") for x in arrays)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(w.m, w.nsys, w.nrow, nseg, **kw)
        fn = pbt.solve_cyclic if kw.get("cyclic") else pbt.solve_noncyclic
        fn(plan, a, b, c, d, w.m, w.nsys, w.nrow)
        assert plan.status() == 0
    return [t.cpu().numpy() for t in (a, b, c, d)]


@pytest.mark.parametrize("m,nsys,nrow,nseg,kw", [
    (3, 100, 40, 1, {}), (5, 70, 24, 1, {"precision": "ff"}), (4, 33, 48, 4, {}), (2, 64, 30, 3, {"precision": "ff"}),
    (10, 7, 12, 1, {}), (5, 64, 64, 1, {"precision": "fp32_refine", "tol": 1e-12}),
    (4, 40, 32, 4, {"cyclic": True}), (5, 40, 24, 1, {"cyclic": True, "precision": "ff"}),
])
def test_cpu_layout_equals_gpu_layout(cuda, m, nsys, nrow, nseg, kw):
    flags = 0 if kw.get("cyclic") else synth.ZERO_ENDS
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=40 + m, delta=1.5, flags=flags)
    cpu = [O.gpu_to_cpu(m, nsys, nrow, k < 3, x) for k, x in enumerate(w.arrays)]
    out_cpu = run(w, cpu, nseg, cpu_layout=True, **kw)
    out_gpu = run(w, w.arrays, nseg, **kw)
    assert np.array_equal(out_cpu[3], O.gpu_to_cpu(m, nsys, nrow, False, out_gpu[3]))
    for k in range(3):
        assert np.array_equal(out_cpu[k], cpu[k])  # A, B, C untouched
    ref = [x.copy() for x in cpu]
    if not kw.get("cyclic"):
        O.solve_noncyclic_cpu(m, nsys, nrow, nseg, *ref)
    elif nseg == 1:
        O.block_thomas_cyclic_cpu(m, nsys, nrow, *ref)
    else:
        O.solve_cyclic_cpu(m, nsys, nrow, nseg, *ref)
    ref_g = O.cpu_to_gpu(m, nsys, nrow, False, ref[3])
    tol = 1e-10 if kw.get("precision") == "fp32_refine" else 1e-12
    assert per_system_relerr(m, nsys, nrow, out_gpu[3], ref_g) <= tol


def test_cpu_layout_profiled_total_covers_conversion(cuda):
    m, nsys, nrow = 4, 256, 64
    w = synth.dominant(m, nsys, nrow, seed=3)
    cpu = [torch.from_numpy(O.gpu_to_cpu(m, nsys, nrow, k < 3, x)).to("cuda:0") for k, x in enumerate(w.arrays)]
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, cpu_layout=True)
        t = pbt.solve_noncyclic_profiled(plan, *cpu, m, nsys, nrow)
    assert t.total >= t.local_compute > 0


def test_cpu_layout_refuses_adjoint(cuda):
    m, nsys, nrow = 3, 32, 8
    a = torch.zeros(m * m * nsys * nrow, dtype=torch.float64, device="cuda:0")
    d = torch.zeros(m * nsys * nrow, dtype=torch.float64, device="cuda:0")
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, cpu_layout=True)
        with pytest.raises(NotImplementedError):
            pbt.adjoint_noncyclic(plan, a, a, a, d, d.clone())
