"""pbt_solve_noncyclic_noalloc: the entry point for callers that cannot
allocate device memory (their memory belongs to their own pool allocator, or
they must not call cudaMalloc/cudaFree, which can synchronise the device,
inside a time-stepping loop).  It keeps its reduced-system scratch in a fixed
32 MiB array inside libpbt.so instead of a plan's workspace.

Called here through the C ABI and compared with the plan-based entry point
(pbt_solve_noncyclic on a plan with PBT_FLAG_INPLACE | PBT_FLAG_REFERENCE_METHOD,
the same in-place two-stage method) on two calls in a row, at the tolerance of
the other GPU parity tests, and its solution directly with the oracle's.  This
file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest
import torch

from pascal_btdma_gb300 import _native as N
from pascal_btdma_gb300 import synth
from conftest import per_system_relerr
from gpu_util import oracle_solve

pytestmark = pytest.mark.gpu
TOL = 1e-12


def planned(w, nseg, dev):
    a, b, c, d = (torch.from_numpy(x).to(dev) for x in w.arrays)
    desc = N.PlanDesc()
    N.lib().pbt_plan_desc_init(C.byref(desc))
    desc.m, desc.nsys, desc.nrow, desc.nseg = w.m, w.nsys, w.nrow, nseg
    desc.flags = N.PBT_FLAG_INPLACE | N.PBT_FLAG_REFERENCE_METHOD
    h = C.c_void_p()
    assert N.lib().pbt_plan_create_ex(C.byref(h), C.byref(desc)) == N.PBT_OK, N.last_error()
    s = torch.cuda.current_stream().cuda_stream
    rc = N.lib().pbt_solve_noncyclic(h, a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(),
                                     w.m, w.nsys, w.nrow, C.c_void_p(s))
    assert rc == N.PBT_OK, N.last_error()
    torch.cuda.synchronize()
    N.lib().pbt_plan_destroy(h)
    return [t.cpu().numpy() for t in (a, c, d)]


def noalloc(w, nseg, dev):
    a, b, c, d = (torch.from_numpy(x).to(dev) for x in w.arrays)
    s = torch.cuda.current_stream().cuda_stream
    rc = N.lib().pbt_solve_noncyclic_noalloc(a.data_ptr(), b.data_ptr(), c.data_ptr(), d.data_ptr(),
                                             w.m, w.nsys, w.nrow, nseg, C.c_void_p(s))
    assert rc == N.PBT_OK, N.last_error()
    torch.cuda.synchronize()
    assert np.array_equal(b.cpu().numpy(), w.B)
    return [t.cpu().numpy() for t in (a, c, d)]


def test_noalloc_matches_plan_entry_twice(cuda):
    cases = [(5, 2048, 256, 4, 1.2, 11), (3, 777, 96, 1, 2.0, 12)]  # m, nsys, nrow, nseg, delta, seed
    for m, nsys, nrow, nseg, delta, seed in cases:
        w = synth.dominant(m, nsys, nrow, seed=seed, delta=delta)
        pa, pc, pd = planned(w, nseg, cuda)
        na, nc, nd = noalloc(w, nseg, cuda)
        assert per_system_relerr(m, nsys, nrow, nd, pd) <= TOL
        assert per_system_relerr(m, nsys, nrow, nd, oracle_solve(w, nseg).D) <= TOL
        scale = max(np.abs(pa).max(), np.abs(pc).max())
        assert np.abs(na - pa).max() <= TOL * scale and np.abs(nc - pc).max() <= TOL * scale


def test_noalloc_rejects_oversized_problem(cuda):
    m, nsys, nrow, nseg = 5, 65536, 256, 16  # reduced system ~ 115 M doubles > 4 Mi
    z = C.c_void_p(16)
    rc = N.lib().pbt_solve_noncyclic_noalloc(z, z, z, z, m, nsys, nrow, nseg, None)
    assert rc == N.PBT_EINVAL
    assert "static capacity" in N.last_error()
