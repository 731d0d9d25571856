"""The TMA-staged single-segment solve (k_thomas_staged, forced with
PBT_FLAG_STAGED_LOADS) against the oracle and against the direct-load kernel
(PBT_FLAG_DIRECT_LOADS).

The staged kernel does the same arithmetic in the same order as the direct
one, so the two must agree bit for bit; the oracle bounds both.  Shapes cover
every staged block size (1..6), the shortest lines (N = 2, 3), a last CTA
with only some lanes in the batch (nsys not a multiple of 32), and the cases
that must fall back to direct loads (odd nsys, an array not 16-byte aligned,
m > 6)."""
import numpy as np
import pytest
import torch

import pascal_btdma_gb300 as pbt
from pascal_btdma_gb300 import synth
from conftest import per_system_relerr
from gpu_util import gpu_solve, oracle_solve, to_dev

pytestmark = pytest.mark.gpu
TOL = 1e-12

SHAPES = [  # m, nsys, nrow
    (1, 64, 2), (1, 1000, 37), (2, 96, 3), (2, 2048, 64), (3, 40, 17), (3, 1024, 128),
    (4, 1000, 37), (4, 256, 300), (5, 64, 2), (5, 1000, 41), (5, 2048, 64), (6, 96, 3), (6, 130, 33),
]


@pytest.mark.parametrize("m,nsys,nrow", SHAPES)
@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_staged_matches_oracle_and_direct(cuda, m, nsys, nrow, prec):
    w = synth.dominant(m, nsys, nrow, seed=31 * m + nrow, delta=1.2)
    (_, B, _, D), singular = gpu_solve(w, 1, precision=prec, staged_loads=True)
    (_, _, _, Dd), singular_d = gpu_solve(w, 1, precision=prec, direct_loads=True)
    ref = oracle_solve(w, 1)
    assert singular == 0 and singular_d == 0
    assert per_system_relerr(m, nsys, nrow, D, ref.D) <= TOL
    assert np.array_equal(D, Dd)
    assert np.array_equal(B, w.B)


@pytest.mark.parametrize("m,nsys,nrow", [(3, 64, 24), (5, 1000, 40)])
@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_staged_in_place(cuda, m, nsys, nrow, prec):
    """In place the factors live in the caller's C as FP64 and the backward
    sweep converts them on its way out of shared memory."""
    w = synth.dominant(m, nsys, nrow, seed=7, delta=1.5)
    (_, _, C, D), _ = gpu_solve(w, 1, precision=prec, inplace=True, staged_loads=True)
    (_, _, Cd, Dd), _ = gpu_solve(w, 1, precision=prec, inplace=True, direct_loads=True)
    ref = oracle_solve(w, 1)
    assert per_system_relerr(m, nsys, nrow, D, ref.D) <= TOL
    assert np.array_equal(D, Dd) and np.array_equal(C, Cd)


def test_staged_refined_solve(cuda):
    m, nsys, nrow = 5, 2048, 64
    w = synth.dominant(m, nsys, nrow, seed=9, delta=1.05, row_scale=True)
    ref = oracle_solve(w, 1)
    for direct in (False, True):
        a, b, c, d = to_dev(w.arrays, "cuda:0")
        with pbt.BtdmaGpuPlan() as plan:
            plan.create(m, nsys, nrow, 1, precision="fp32_refine", tol=1e-12, max_iter=8, direct_loads=direct,
                        staged_loads=not direct)
            pbt.solve_noncyclic(plan, a, b, c, d, m, nsys, nrow)
            assert plan.status() == 0
        assert per_system_relerr(m, nsys, nrow, d.cpu().numpy(), ref.D) <= 1e-10


@pytest.mark.parametrize("nsys", [40, 1000])
def test_partial_last_cta_reports_no_false_pivots(cuda, nsys):
    """Lanes past nsys compute on the zero fill of the copies; they must not
    count as zero pivots, while a real singular system must."""
    m, nrow = 4, 16
    w = synth.dominant(m, nsys, nrow, seed=3, delta=1.5)
    _, singular = gpu_solve(w, 1, precision="ff", staged_loads=True)
    assert singular == 0
    B = w.B.reshape(m * m * nrow, nsys).copy()
    B[:, 5] = 0.0  # system 5: B_q = 0 and A_0 = 0 -> the first pivot is zero
    w2 = synth.Workload(m, nsys, nrow, w.A, B.reshape(-1), w.C, w.D)
    _, singular = gpu_solve(w2, 1, precision="fp64", staged_loads=True)
    assert singular >= 1


@pytest.mark.parametrize("case", ["odd_nsys", "unaligned", "m7"])
def test_fallbacks_stay_correct(cuda, case):
    if case == "odd_nsys":
        m, nsys, nrow = 4, 65, 20
    elif case == "m7":
        m, nsys, nrow = 7, 64, 12
    else:
        m, nsys, nrow = 3, 64, 20
    w = synth.dominant(m, nsys, nrow, seed=11, delta=1.5)
    ref = oracle_solve(w, 1)
    if case != "unaligned":
        (_, _, _, D), _ = gpu_solve(w, 1, precision="ff", staged_loads=True)
        assert per_system_relerr(m, nsys, nrow, D, ref.D) <= TOL
        return
    # Arrays that start 8 bytes past a 16-byte boundary: no tensor map, direct loads.
    dev = "cuda:0"
    bufs = []
    for x in w.arrays:
        t = torch.empty(x.size + 1, dtype=torch.float64, device=dev)
        v = t[1:]
        v.copy_(torch.from_numpy(x))
        assert v.data_ptr() % 16 == 8
        bufs.append(v)
    a, b, c, d = bufs
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, precision="ff", staged_loads=True)
        pbt.solve_noncyclic(plan, a, b, c, d, m, nsys, nrow)
        assert plan.status() == 0
    assert per_system_relerr(m, nsys, nrow, d.cpu().numpy(), ref.D) <= TOL


def test_staged_on_side_stream_and_repeated(cuda):
    m, nsys, nrow = 5, 512, 48
    w = synth.dominant(m, nsys, nrow, seed=21, delta=1.2)
    ref = oracle_solve(w, 1)
    a, b, c, d0 = to_dev(w.arrays, "cuda:0")
    s = torch.cuda.Stream()
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, precision="ff", staged_loads=True)
        outs = []
        with torch.cuda.stream(s):
            for _ in range(3):
                d = d0.clone()
                pbt.solve_noncyclic(plan, a, b, c, d, m, nsys, nrow, stream=s)
                outs.append(d)
        s.synchronize()
        assert plan.status() == 0
    for d in outs:
        assert per_system_relerr(m, nsys, nrow, d.cpu().numpy(), ref.D) <= TOL
    assert all(torch.equal(outs[0], o) for o in outs[1:])


def test_default_choice_matches_both(cuda):
    """Without a load flag the library picks a kernel per solve; whichever it
    picks, the bits are those of both forced variants (pencil-shaped batch
    large enough for the direct kernel to be picked)."""
    m, nsys, nrow = 3, 65536, 8
    w = synth.dominant(m, nsys, nrow, seed=4, delta=1.5)
    outs = [gpu_solve(w, 1, precision="ff", **kw)[0][3] for kw in ({}, {"direct_loads": True}, {"staged_loads": True})]
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
