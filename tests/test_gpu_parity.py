"""GPU parity: the CUDA path, called through the C ABI, against the CPU
oracle on the same seeded inputs.  Plain FP64 must match within 1e-12
relative per system (max|x - x_oracle| / max|x_oracle|; the oracle pivots
like LAPACK, the GPU pivots the same way but fuses multiply-adds)."""
import numpy as np
import pytest
import torch

import pascal_btdma_gb300 as pbt
from pascal_btdma_gb300 import synth
from conftest import per_system_relerr
from gpu_util import column_subset, gpu_solve, oracle_solve, subset, to_dev

pytestmark = pytest.mark.gpu
TOL = 1e-12      # plain FP64 against the oracle
TOL_FF = 1e-12   # float-float (~47-bit arithmetic) against the oracle
PREC_TOL = [("fp64", TOL), ("ff", TOL_FF)]

GRID = [  # m, nsys, nrow, nseg
    (1, 37, 10, 1), (1, 37, 12, 4), (2, 65, 9, 1), (2, 65, 9, 3), (3, 33, 12, 4), (3, 129, 13, 2),
    (4, 31, 40, 8), (5, 70, 24, 3), (5, 64, 256, 16), (6, 17, 18, 6), (7, 9, 9, 3), (8, 20, 16, 5),
    (9, 11, 12, 4), (10, 7, 30, 3), (3, 40, 3, 1), (4, 5, 2, 1), (4, 300, 128, 1), (2, 1, 2, 1),
]


@pytest.mark.parametrize("m,nsys,nrow,nseg", GRID)
@pytest.mark.parametrize("delta", [1.05, 2.0])
@pytest.mark.parametrize("prec,tol", PREC_TOL)
def test_noncyclic_matches_oracle(cuda, m, nsys, nrow, nseg, delta, prec, tol):
    w = synth.dominant(m, nsys, nrow, seed=1000 * m + nseg, delta=delta)
    (_, B, _, D), singular = gpu_solve(w, nseg, precision=prec)
    ref = oracle_solve(w, nseg)
    assert singular == 0
    assert per_system_relerr(m, nsys, nrow, D, ref.D) <= tol
    assert np.array_equal(B, w.B)


def test_small_config(cuda):
    """m=3, nsys=1024, N=128 split into 4 segments of 32, delta=2.0."""
    w = synth.dominant(3, 1024, 128, seed=1, delta=2.0)
    (A, _, C, D), _ = gpu_solve(w, 4)
    ref = oracle_solve(w, 4)
    assert per_system_relerr(3, 1024, 128, D, ref.D) <= TOL
    assert np.array_equal(A, w.A) and np.array_equal(C, w.C)  # not in place by default


@pytest.mark.parametrize("nseg", [1, 2, 4])
@pytest.mark.parametrize("prec,tol", PREC_TOL)
def test_inplace_side_effects_match_reference(cuda, nseg, prec, tol):
    """PBT_FLAG_INPLACE + reference method: A and C receive the same A', C' as the reference."""
    m, nsys, nrow = 4, 96, 24
    w = synth.dominant(m, nsys, nrow, seed=77, delta=1.5)
    (A, _, C, D), _ = gpu_solve(w, nseg, inplace=True, reference_method=True, precision=prec)
    ref = oracle_solve(w, nseg)
    assert per_system_relerr(m, nsys, nrow, D, ref.D) <= tol
    scale = max(np.abs(ref.A).max(), np.abs(ref.C).max())
    assert np.abs(A - ref.A).max() <= 10 * tol * scale
    assert np.abs(C - ref.C).max() <= 10 * tol * scale


@pytest.mark.parametrize("m,nsys,nrow,nseg", [(3, 64, 40, 1), (5, 70, 24, 3)])
def test_ff_inplace_equals_workspace(cuda, m, nsys, nrow, nseg):
    w = synth.dominant(m, nsys, nrow, seed=78, delta=1.2)
    (_, _, _, D1), _ = gpu_solve(w, nseg, precision="ff")
    (_, _, _, D2), _ = gpu_solve(w, nseg, precision="ff", inplace=True)
    assert per_system_relerr(m, nsys, nrow, D1, D2) <= TOL_FF


@pytest.mark.parametrize("m,nsys,nrow,nseg", [(1, 33, 8, 2), (2, 40, 16, 4), (3, 70, 12, 3), (4, 64, 24, 6), (5, 31, 30, 5), (8, 9, 12, 2)])
@pytest.mark.parametrize("prec,tol", PREC_TOL)
def test_cyclic_matches_oracle(cuda, m, nsys, nrow, nseg, prec, tol):
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=5 + m, delta=1.5, flags=0)
    (_, _, _, D), _ = gpu_solve(w, nseg, cyclic=True, precision=prec)
    ref = oracle_solve(w, nseg, cyclic=True)
    assert per_system_relerr(m, nsys, nrow, D, ref.D) <= tol


CYCLIC_P1 = [  # m, nsys, nrow: periodic lines in one segment, m = 1..10, ragged warps, nrow down to 3
    (1, 33, 3), (1, 37, 10), (2, 65, 4), (2, 40, 16), (3, 70, 12), (3, 129, 5), (4, 64, 24), (4, 31, 40),
    (5, 31, 30), (5, 96, 64), (6, 17, 18), (7, 9, 9), (8, 20, 16), (9, 11, 12), (10, 7, 30),
]


@pytest.mark.parametrize("m,nsys,nrow", CYCLIC_P1)
@pytest.mark.parametrize("delta", [1.05, 1.5])
@pytest.mark.parametrize("prec,tol", PREC_TOL)
def test_cyclic_single_segment_matches_oracle(cuda, m, nsys, nrow, delta, prec, tol):
    """k_thomas_cyclic against btdma_many_cycl applied to the whole line."""
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=17 * m + nrow, delta=delta, flags=0)
    (A, B, C, D), singular = gpu_solve(w, 1, cyclic=True, precision=prec)
    assert singular == 0
    ref = oracle_solve(w, 1, cyclic=True)
    assert per_system_relerr(m, nsys, nrow, D, ref.D) <= tol
    # A, B and C are left untouched by a workspace plan.
    assert np.array_equal(A, w.A) and np.array_equal(B, w.B) and np.array_equal(C, w.C)


@pytest.mark.parametrize("m,nsys,nrow", [(2, 65, 9), (5, 70, 24), (8, 9, 12)])
@pytest.mark.parametrize("prec,tol", PREC_TOL)
def test_cyclic_single_segment_inplace_and_two_stage(cuda, m, nsys, nrow, prec, tol):
    """In place (C' into C, A untouched) it gives the workspace plan's x, and
    the single-segment solve agrees with the two-stage cyclic method."""
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=31 + m, delta=1.3, flags=0)
    (_, _, _, D1), _ = gpu_solve(w, 1, cyclic=True, precision=prec)
    (A2, _, C2, D2), _ = gpu_solve(w, 1, cyclic=True, precision=prec, inplace=True)
    (_, _, _, D3), _ = gpu_solve(w, 2, cyclic=True, precision=prec)
    assert per_system_relerr(m, nsys, nrow, D2, D1) <= tol
    assert per_system_relerr(m, nsys, nrow, D3, D1) <= tol
    assert np.array_equal(A2, w.A) and not np.array_equal(C2, w.C)


def test_cyclic_single_segment_singular_block_reported(cuda):
    """A zero diagonal block on a periodic line is counted, as in the other solves."""
    m, nsys, nrow = 3, 40, 8
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=4, delta=1.5, flags=0)
    B = w.B.reshape(m * m, nrow, nsys)
    B[:, 3, 5] = 0.0
    A = w.A.reshape(m * m, nrow, nsys)
    A[:, 3, 5] = 0.0
    (_, _, _, _), singular = gpu_solve(w, 1, cyclic=True)
    assert singular >= 1


def test_manufactured_solution(cuda):
    w = synth.manufactured(3, 256, 64, seed=2)
    (_, _, _, D), _ = gpu_solve(w, 4)
    ref = oracle_solve(w, 4)
    assert per_system_relerr(3, 256, 64, D, ref.D) <= 1e-10


def test_reference_signatures_on_gpu(cuda):
    """The reference's recorded first-solve signatures, full batch sizes."""
    import json
    from pathlib import Path

    rows = json.loads((Path(__file__).parent / "golden" / "signatures.json").read_text())["rows"]
    for row in rows:
        m, nsys, nrow, nseg = row["m"], row["nsys"], row["n3"], row["nseg"]
        nm = nsys * nrow * m * m
        if nm > 6e8:
            nsys = max(1, int(6e8 // (nrow * m * m)))
        dev = cuda
        eye = torch.eye(m, dtype=torch.float64, device=dev)
        blk = eye.T.reshape(m * m, 1).expand(m * m, nsys * nrow).reshape(-1)  # plane (i + m*j) = delta_ij
        a = (0.25 * blk).contiguous()
        b = (2.0 * blk).contiguous()
        c = (0.25 * blk).contiguous()
        d = torch.ones(nsys * nrow * m, dtype=torch.float64, device=dev)
        with pbt.BtdmaGpuPlan() as plan:
            plan.create(m, nsys, nrow, nseg)
            pbt.solve_noncyclic(plan, a, b, c, d, m, nsys, nrow)
        x = d.reshape(m, nrow, nsys)
        k = row["nsys"] / nsys
        assert float(d.sum()) * k == pytest.approx(row["solution_sum"], rel=1e-9)
        assert float(torch.sqrt((d * d).sum())) * np.sqrt(k) == pytest.approx(row["solution_l2"], rel=1e-9)
        assert float(d.abs().max()) == pytest.approx(row["solution_linf"], rel=1e-14)
        for z, key in ((0, "sample_z0"), (nrow // 2, "sample_zmid"), (nrow - 1, "sample_zlast")):
            assert float(x[0, z, 0]) == pytest.approx(row[key], rel=1e-14)
        del a, b, c, d


def test_singular_block_is_reported(cuda):
    m, nsys, nrow = 3, 64, 10
    w = synth.dominant(m, nsys, nrow, seed=3, delta=1.5)
    B = w.B.reshape(m, m, nrow, nsys)
    B[:, :, 4, 5] = 0.0  # system 5, row 4: B - A C' has a zero row/col -> zero pivot
    w.A.reshape(m, m, nrow, nsys)[:, :, 4, 5] = 0.0
    (_, _, _, D), singular = gpu_solve(w, 1)
    assert singular >= 1
    x = D.reshape(m, nrow, nsys)
    assert np.isfinite(np.delete(x, 5, axis=2)).all()  # other systems unaffected


def test_profiled_timings(cuda):
    w = synth.dominant(4, 4096, 64, seed=4, delta=1.5)
    a, b, c, d = to_dev(w.arrays, cuda)
    for nseg in (1, 4):
        with pbt.BtdmaGpuPlan() as plan:
            plan.create(4, 4096, 64, nseg)
            t = pbt.solve_noncyclic_profiled(plan, a, b, c, d.clone(), 4, 4096, 64)
        assert t.total > 0 and t.local_compute > 0
        assert t.computation() <= t.total * 1.001 + 1e-6
        if nseg > 1:
            assert t.reduced_compute > 0 and t.update_compute > 0


@pytest.mark.parametrize("cyclic", [False, True])
def test_batch_filling_the_gpu_runs_one_segment(cuda, cyclic):
    """A plan whose batch fills the GPU (at least 4 warps of systems per SM:
    19456 systems on 152 SMs; here 32768) solves one segment per line whatever
    nseg says: the same bits as an nseg = 1 plan, and the oracle's segmented x
    to rounding; PBT_FLAG_REFERENCE_METHOD keeps the segments."""
    m, nsys, nrow, nseg = 3, 32768, 24, 4
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=8, delta=1.5, flags=0 if cyclic else synth.ZERO_ENDS)
    for prec, tol in PREC_TOL:
        (_, _, _, D4), _ = gpu_solve(w, nseg, cyclic=cyclic, precision=prec)
        (_, _, _, D1), _ = gpu_solve(w, 1, cyclic=cyclic, precision=prec)
        (_, _, _, Dr), _ = gpu_solve(w, nseg, cyclic=cyclic, precision=prec, reference_method=True)
        assert np.array_equal(D4, D1)
        assert not np.array_equal(Dr, D1)
        sub = subset(w, np.arange(0, nsys, 1024))
        ref = oracle_solve(sub, nseg, cyclic=cyclic)
        for D in (D4, Dr):
            got = column_subset(m, nsys, nrow, D, np.arange(0, nsys, 1024))
            assert per_system_relerr(m, sub.nsys, nrow, got, ref.D) <= tol


def test_one_segment_threshold_is_four_warps_per_sm(cuda):
    """The switch to one segment per line happens at 4 warps of systems per SM
    (128 systems per SM): one warp below it the segments are kept."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    m, nrow, nseg = 2, 12, 3
    for nsys, one_segment in ((128 * sms - 32, False), (128 * sms, True)):
        w = synth.dominant(m, nsys, nrow, seed=9, delta=1.5)
        (_, _, _, D3), _ = gpu_solve(w, nseg, precision="ff")
        (_, _, _, D1), _ = gpu_solve(w, 1, precision="ff")
        assert np.array_equal(D3, D1) == one_segment


def test_plan_mismatch_and_reuse(cuda):
    w = synth.dominant(3, 64, 12, seed=5, delta=2.0)
    a, b, c, d = to_dev(w.arrays, cuda)
    plan = pbt.BtdmaGpuPlan().create(3, 64, 12, 2)
    with pytest.raises(ValueError, match="do not match"):
        pbt.solve_noncyclic(plan, a, b, c, d, 3, 64, 13)
    with pytest.raises(ValueError, match="PBT_FLAG_CYCLIC|cyclic"):
        pbt.solve_cyclic(plan, a, b, c, d, 3, 64, 12)
    # the same plan solves twice with the same result
    d1, d2 = d.clone(), d.clone()
    pbt.solve_noncyclic(plan, a, b, c, d1, 3, 64, 12)
    pbt.solve_noncyclic(plan, a, b, c, d2, 3, 64, 12)
    assert torch.equal(d1, d2)
    plan.destroy()
    with pytest.raises(RuntimeError, match="uncreated"):
        pbt.solve_noncyclic(plan, a, b, c, d, 3, 64, 12)


def test_side_stream(cuda):
    w = synth.dominant(5, 512, 32, seed=6, delta=1.2)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        (_, _, _, D), _ = gpu_solve(w, 2, stream=s)
    ref = oracle_solve(w, 2)
    assert per_system_relerr(5, 512, 32, D, ref.D) <= TOL


FULL = [  # the production-size configurations: m, nsys, nrow, nseg, delta, keep the segments
    (5, 65536, 256, 1, 1.2, False),
    (5, 65536, 256, 16, 1.2, False),  # fills the GPU: solved one segment per line
    (5, 65536, 256, 16, 1.2, True),   # the 16 segments kept (PBT_FLAG_REFERENCE_METHOD)
    (4, 256, 32768, 128, 1.2, False),
]


@pytest.mark.parametrize("m,nsys,nrow,nseg,delta,segmented", FULL,
                         ids=["pencil_P1", "pencil_P16", "pencil_P16_segmented", "long_lines_P128"])
def test_full_size_against_oracle_subset(cuda, m, nsys, nrow, nseg, delta, segmented):
    """Full batch on the GPU; 48 of its systems re-solved by the oracle.
    Systems are independent, so this checks those systems exactly."""
    w = synth.dominant(m, nsys, nrow, seed=2024, delta=delta)
    rng = np.random.default_rng(0)
    pick = np.unique(np.concatenate([[0, nsys - 1], rng.choice(nsys, size=min(nsys, 46), replace=False)]))
    ref = oracle_solve(subset(w, pick), nseg)
    for prec, tol in PREC_TOL:
        (_, _, _, D), singular = gpu_solve(w, nseg, precision=prec, reference_method=segmented)
        assert singular == 0
        got = column_subset(m, nsys, nrow, D, pick)
        err = per_system_relerr(m, len(pick), nrow, got, ref.D)
        print(f"{prec} m={m} nsys={nsys} nrow={nrow} nseg={nseg}: max rel err {err:.3e}")
        assert err <= tol
        assert np.isfinite(D).all()


@pytest.mark.parametrize("nseg,segmented", [(1, False), (2, False), (2, True)])
def test_full_size_cyclic_against_oracle_subset(cuda, nseg, segmented):
    """The pencil batch as periodic lines (m = 5, 65536 x 256, the bench's
    cyclic variant) on the GPU; 48 of its systems re-solved by the oracle's
    periodic solve (btdma_many_cycl restated)."""
    m, nsys, nrow = 5, 65536, 256
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=2025, delta=1.2, flags=0)
    rng = np.random.default_rng(1)
    pick = np.unique(np.concatenate([[0, nsys - 1], rng.choice(nsys, size=46, replace=False)]))
    ref = oracle_solve(subset(w, pick), nseg, cyclic=True)
    for prec, tol in PREC_TOL:
        (_, _, _, D), singular = gpu_solve(w, nseg, cyclic=True, precision=prec, reference_method=segmented)
        assert singular == 0
        got = column_subset(m, nsys, nrow, D, pick)
        err = per_system_relerr(m, len(pick), nrow, got, ref.D)
        print(f"cyclic {prec} m={m} nsys={nsys} nrow={nrow} nseg={nseg}: max rel err {err:.3e}")
        assert err <= tol
        assert np.isfinite(D).all()


@pytest.mark.parametrize("m,nsys,nrow,nseg,segmented,tpb,cyclic,prec", [
    (5, 39999, 16, 1, False, 0, False, "ff"),  # 250 CTAs of 160 threads, the last with 159 systems
    (6, 39999, 12, 1, False, 0, False, "ff"),
    (5, 39999, 16, 4, True, 0, False, "ff"),   # 179 x 4 CTAs of 224 threads, the last column with 127
    (6, 20001, 12, 3, True, 0, False, "ff"),   # 126 x 3 CTAs of 160 threads, the last column with 1
    (5, 1000, 20, 1, False, 96, False, "ff"),  # a CTA size fixed by the caller
    (5, 1000, 20, 4, True, 96, False, "ff"),
    (3, 39999, 16, 1, False, 0, False, "ff"),  # the fused forms, m <= 4
    (4, 39999, 16, 4, True, 0, False, "ff"),
    (5, 39999, 12, 1, False, 0, True, "ff"),   # the periodic solve
    (2, 39999, 9, 1, False, 0, True, "ff"),
    (5, 39999, 16, 4, True, 0, False, "fp32_refine"),  # the FP32 local stage of the refined solve
])
def test_rows_in_step_partial_cta(cuda, m, nsys, nrow, nseg, segmented, tpb, cyclic, prec):
    """The kernels that keep a CTA's warps in step (a barrier per row): the
    threads past the last system of a partial CTA take the barriers only.
    The systems of the partial CTA and a random sample are checked against
    the oracle."""
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=77, delta=1.2, flags=0 if cyclic else synth.ZERO_ENDS)
    rng = np.random.default_rng(3)
    pick = np.unique(np.concatenate([np.arange(nsys - 40, nsys), rng.choice(nsys, size=40, replace=False)]))
    ref = oracle_solve(subset(w, pick), nseg, cyclic=cyclic)
    (_, _, _, D), singular = gpu_solve(w, nseg, cyclic=cyclic, precision=prec, reference_method=segmented,
                                       threads_per_block=tpb)
    assert singular == 0
    err = per_system_relerr(m, len(pick), nrow, column_subset(m, nsys, nrow, D, pick), ref.D)
    assert err <= (REFINE_TOL if prec == "fp32_refine" else TOL_FF)
    assert np.isfinite(D).all()


REFINE_TOL = 1e-10  # the mixed-precision target: FP32 factorisation + FP64 residual refinement


@pytest.mark.parametrize("m,nsys,nrow,nseg", [(1, 37, 12, 4), (2, 65, 9, 1), (3, 33, 12, 4), (4, 31, 40, 8),
                                              (5, 70, 24, 3), (5, 64, 256, 16), (6, 17, 18, 6), (8, 20, 16, 5),
                                              (10, 7, 30, 3), (4, 300, 128, 1)])
@pytest.mark.parametrize("delta", [1.05, 2.0])
def test_refined_matches_oracle(cuda, m, nsys, nrow, nseg, delta):
    w = synth.dominant(m, nsys, nrow, seed=2000 * m + nseg, delta=delta)
    a, b, c, d = to_dev(w.arrays, cuda)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, nseg, precision="fp32_refine")
        pbt.solve_noncyclic(plan, a, b, c, d, m, nsys, nrow)
        iters, corr = plan.refine_info()
    ref = oracle_solve(w, nseg)
    err = per_system_relerr(m, nsys, nrow, d.cpu().numpy(), ref.D)
    assert err <= REFINE_TOL
    assert 2 <= iters <= 8 and corr <= 1e-5
    assert torch.equal(a.cpu(), torch.from_numpy(w.A)) and torch.equal(c.cpu(), torch.from_numpy(w.C))


@pytest.mark.parametrize("delta", [1.05, 1.5])
@pytest.mark.parametrize("nseg", [1, 16])
def test_refined_row_scaled(cuda, delta, nseg):
    """The mixed-precision configuration, fewer systems: m=5, N=256, each block
    row scaled by a log-uniform factor in [1e-3, 1e3]."""
    m, nsys, nrow = 5, 512, 256
    w = synth.dominant(m, nsys, nrow, seed=44, delta=delta, row_scale=True)
    a, b, c, d = to_dev(w.arrays, cuda)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, nseg, precision="fp32_refine")
        pbt.solve_noncyclic(plan, a, b, c, d, m, nsys, nrow)
        iters, corr = plan.refine_info()
    ref = oracle_solve(w, nseg)
    err = per_system_relerr(m, nsys, nrow, d.cpu().numpy(), ref.D)
    print(f"refined delta={delta} nseg={nseg}: {iters} FP32 solves, last correction {corr:.2e}, rel err {err:.2e}")
    assert err <= REFINE_TOL


@pytest.mark.parametrize("m,nsys,nrow", [(1, 64, 30), (2, 100, 50), (4, 96, 20), (5, 256, 128), (6, 64, 40)])
@pytest.mark.parametrize("delta", [1.05, 2.0])
def test_refine_fused_correction_matches_separate_passes(cuda, m, nsys, nrow, delta):
    """A single-segment refined plan whose first FP32 pass runs the staged
    kernel keeps that pass's factors and runs each correction as one fused
    pass (FP64 residual, FP32 substitution, accumulate); forcing direct loads
    leaves no factors, so the corrections run as residual, FP32 solve and
    accumulate.  They are the same operations: the same bits."""
    w = synth.dominant(m, nsys, nrow, seed=900 + m, delta=delta)
    outs = []
    for kw in ({}, {"direct_loads": True}):
        a, b, c, d = to_dev(w.arrays, cuda)
        with pbt.BtdmaGpuPlan() as plan:
            plan.create(m, nsys, nrow, 1, precision="fp32_refine", tol=1e-13, **kw)
            pbt.solve_noncyclic(plan, a, b, c, d, m, nsys, nrow)
            outs.append((d.cpu(), plan.refine_info()))
    assert outs[0][1][0] >= 2
    assert outs[0][1] == outs[1][1]
    assert torch.equal(outs[0][0], outs[1][0])
    ref = oracle_solve(w)
    assert per_system_relerr(m, nsys, nrow, outs[0][0].numpy(), ref.D) <= REFINE_TOL


def test_refine_stops_at_max_iter(cuda):
    w = synth.dominant(3, 64, 40, seed=5, delta=1.05)
    a, b, c, d = to_dev(w.arrays, cuda)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(3, 64, 40, 1, precision="fp32_refine", tol=1e-30, max_iter=3)
        pbt.solve_noncyclic(plan, a, b, c, d, 3, 64, 40)
        iters, corr = plan.refine_info()
    assert iters == 3 and corr > 0


@pytest.mark.parametrize("m,nsys,nrow,nseg", [(3, 64, 1024, 64), (4, 100, 600, 50), (5, 40, 4096, 256)])
@pytest.mark.parametrize("prec,tol", PREC_TOL)
def test_recursive_reduced_solve(cuda, m, nsys, nrow, nseg, prec, tol):
    """Few long lines: the plan solves its 2P-row reduced system with the
    two-stage method again (a reduced-system plan of 8-row segments, and for
    2P >= 512 one more level)."""
    w = synth.dominant(m, nsys, nrow, seed=300 + m, delta=1.5)
    (_, _, _, D), singular = gpu_solve(w, nseg, precision=prec)
    ref = oracle_solve(w, nseg)
    assert singular == 0
    assert per_system_relerr(m, nsys, nrow, D, ref.D) <= tol
