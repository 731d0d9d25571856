"""Range of the float-float and FP32 arithmetics (pbt_precision in pbt.h).

Float-float carries FP32's exponent range.  Matrix entries outside 2^-96 <=
|v| < 2^96, right-hand-side entries at or above 2^128, overflows, and
solutions wholly below 2^-100 must end in a reported failure
(pbt_plan_status -> PBT_ERANGE), never in a silently wrong number; inside
those limits the result must match the oracle at 1e-12.  The rule every
case checks: either the status call raises a range (or convergence) error, or
the solution matches the oracle.  Plain FP64 has the reference's own range and
must match the oracle everywhere."""
import numpy as np
import pytest
import torch

import pascal_btdma_gb300 as pbt
from pascal_btdma_gb300 import batch as B
from pascal_btdma_gb300 import shared, synth
from conftest import per_system_relerr
from gpu_util import oracle_solve, to_dev

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-12, "ff": 1e-12, "fp32_refine": 1e-10}
FAILURES = (pbt.ArithmeticRangeError, pbt.RefinementNotConverged, pbt.SingularBlockError)


def scaled_rows(w, exps, seed=0):
    """Scale block rows by 2^e (e drawn from `exps` per (system, row)): every
    block row of A, B, C, d by one power of two, so x is unchanged."""
    m, nsys, N = w.m, w.nsys, w.nrow
    rng = np.random.default_rng(seed)
    f = np.exp2(rng.choice(np.asarray(exps, dtype=np.float64), size=(N, nsys)))
    out = w.copy()
    for X in (out.A, out.B, out.C):
        X.reshape(m * m, N, nsys)[:] *= f
    out.D.reshape(m, N, nsys)[:] *= f
    return out


def solve(w, nseg, prec, **kw):
    """(x, error or None): the GPU solution and the status call's exception."""
    a, b, c, d = to_dev(w.arrays, "cuda:0")
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(w.m, w.nsys, w.nrow, nseg, precision=prec, **kw)
        pbt.solve_noncyclic(plan, a, b, c, d, w.m, w.nsys, w.nrow)
        try:
            plan.status()
            err = None
        except FAILURES as e:
            err = e
    return d.cpu().numpy(), err


def reported_or_right(w, nseg, prec, expect_failure=None, **kw):
    x, err = solve(w, nseg, prec, **kw)
    if expect_failure is True:
        assert err is not None, f"{prec}: out-of-range input was not reported"
    if err is None:
        ref = oracle_solve(w, nseg)
        e = per_system_relerr(w.m, w.nsys, w.nrow, x, ref.D)
        assert e <= TOL[prec], f"{prec}: silent error {e:.3e}"
    if expect_failure is False:
        assert err is None, f"{prec}: false range report: {err}"
    return err


@pytest.mark.parametrize("nseg", [1, 4])
@pytest.mark.parametrize("exps", [(-110, 0), (0, 110), (-140, 0, 140), (-110, 110)], ids=str)
def test_rows_outside_the_window(cuda, exps, nseg):
    """Rows scaled by 2^+-110 and 2^+-140: FP64 matches the oracle; float-float
    reports PBT_ERANGE; the refined solve converges or reports."""
    w = scaled_rows(synth.dominant(5, 96, 48, seed=31, delta=1.5), exps, seed=len(exps))
    reported_or_right(w, nseg, "fp64", expect_failure=False)
    err = reported_or_right(w, nseg, "ff", expect_failure=True)
    assert isinstance(err, pbt.ArithmeticRangeError)
    reported_or_right(w, nseg, "fp32_refine")


@pytest.mark.parametrize("m,nseg", [(2, 1), (4, 1), (5, 1), (5, 6), (8, 1), (8, 3)])
def test_rows_inside_the_window(cuda, m, nseg):
    """Rows scaled by 2^+-60: no false report, oracle parity in every arithmetic
    and in both single-segment load paths."""
    w = scaled_rows(synth.dominant(m, 64, 36, seed=40 + m, delta=1.5), (-60, -20, 0, 30, 60), seed=m)
    for prec in ("fp64", "ff", "fp32_refine"):
        reported_or_right(w, nseg, prec, expect_failure=False)
    if nseg == 1 and m <= 6:
        reported_or_right(w, nseg, "ff", expect_failure=False, staged_loads=True)


@pytest.mark.parametrize("nseg", [1, 3])
def test_single_entries(cuda, nseg):
    """One matrix entry outside the window (B = 2^-100, a tiny coupling term;
    C = 2^100; A = NaN) or one right-hand side at 2^130: float-float and the
    refined solve must report each.  Right-hand-side entries far below the
    rest (2^-110, 2^-200) or large but representable (2^100) need no report
    and must come out right."""
    base = synth.dominant(4, 40, 30, seed=7, delta=1.5)
    bad = (("B", 5 + 40 * (7 + 30 * 1), 2.0 ** -100), ("C", 9 + 40 * (3 + 30 * 6), 2.0 ** 100),
           ("A", 3 + 40 * (12 + 30 * 5), float("nan")), ("D", 11 + 40 * 20, 2.0 ** 130))
    for arr, idx, val in bad:
        w = base.copy()
        getattr(w, arr)[idx] = val
        if arr in ("B", "D"):
            reported_or_right(w, nseg, "fp64", expect_failure=False)
        reported_or_right(w, nseg, "ff", expect_failure=True)
        reported_or_right(w, nseg, "fp32_refine", expect_failure=True)
    for val in (2.0 ** -110, 2.0 ** -200, 2.0 ** 100):
        w = base.copy()
        w.D[11 + 40 * 20] = val
        for prec in ("fp64", "ff", "fp32_refine"):
            reported_or_right(w, nseg, prec, expect_failure=False)


def test_tiny_solution_is_reported(cuda):
    """Inputs inside the window but a solution below 2^-100 (d ~ 2^-60, the
    blocks ~ 2^45): float-float cannot carry 47 bits there and must say so."""
    w = synth.dominant(3, 64, 20, seed=9, delta=1.5)
    w.A *= 2.0 ** 45
    w.B *= 2.0 ** 45
    w.C *= 2.0 ** 45
    w.D *= 2.0 ** -60
    reported_or_right(w, 1, "fp64", expect_failure=False)
    for nseg in (1, 4):
        reported_or_right(w, nseg, "ff", expect_failure=True)
        reported_or_right(w, nseg, "fp32_refine", expect_failure=True)


def test_cyclic_and_adjoint_report(cuda):
    w = synth.fill(synth.DOMINANT, 3, 50, 24, seed=3, delta=1.5, flags=0)
    w.C[7] = 2.0 ** 100
    for nseg in (1, 2):
        a, b, c, d = to_dev(w.arrays, cuda)
        with pbt.BtdmaGpuPlan() as plan:
            plan.create(3, 50, 24, nseg, cyclic=True, precision="ff")
            pbt.solve_cyclic(plan, a, b, c, d, 3, 50, 24)
            with pytest.raises(pbt.ArithmeticRangeError):
                plan.status()
    w = synth.dominant(3, 50, 24, seed=4, delta=1.5)
    a, b, c, d = to_dev(w.arrays, cuda)
    g = torch.ones_like(d)
    g[5] = 2.0 ** 130
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(3, 50, 24, 1, precision="ff")
        pbt.solve_noncyclic(plan, a, b, c, d, 3, 50, 24)
        assert plan.status() == 0
        pbt.adjoint_noncyclic(plan, a, b, c, d, g)
        with pytest.raises(pbt.ArithmeticRangeError):
            plan.status()


def test_batch_and_shared_report(cuda):
    m = np.array([2, 3, 5, 4], dtype=np.int32)
    n = np.array([40, 300, 70, 9], dtype=np.int32)
    systems = [synth.dominant(int(m[s]), 1, int(n[s]), seed=50 + s, delta=1.5) for s in range(4)]
    systems[2].B[13] = 2.0 ** 99
    user = [torch.from_numpy(np.concatenate([getattr(w, k) for w in systems])).to(cuda) for k in "ABCD"]
    plan = B.BatchPlan(m, n, "ff", {"seg_len": {k: 32 for k in range(1, 6)}, "warps_per_cta": 4})
    packed = plan.pack(*user)
    plan.solve(*packed)
    with pytest.raises(pbt.ArithmeticRangeError):
        plan.status()
    plan.destroy()

    w = synth.dominant(2, 1, 16, seed=5, delta=1.5)
    rhs = torch.from_numpy(np.random.default_rng(0).uniform(-1, 1, 33 * 16 * 2)).to(cuda)
    with shared.SharedMatrix(2, 16, w.A, w.B, w.C, precision="ff") as sm:
        sm.solve(rhs.clone())
        sm.status()  # in range: no report
        bad = rhs.clone()
        bad[40] = 2.0 ** 130
        sm.solve(bad)
        with pytest.raises(pbt.ArithmeticRangeError):
            sm.status()
