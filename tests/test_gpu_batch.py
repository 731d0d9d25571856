"""Uneven batches (include/pbt_batch.h): systems of mixed block size m and
length N in one persistent launch.  Every system is checked against the
oracle solving that system alone."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from pascal_btdma_gb300 import batch as B
from pascal_btdma_gb300 import synth

pytestmark = pytest.mark.gpu


def make_batch(nsys, nmin, nmax, seed, mmax=5):
    n, m = synth.uneven_shapes(seed, nsys, nmin, nmax, 1, mmax)
    systems = [synth.dominant(int(m[s]), 1, int(n[s]), seed=seed * 1000 + s, delta=1.5) for s in range(nsys)]
    ua = np.concatenate([w.A for w in systems])
    ub = np.concatenate([w.B for w in systems])
    uc = np.concatenate([w.C for w in systems])
    ud = np.concatenate([w.D for w in systems])
    return m, n, systems, (ua, ub, uc, ud)


def reference(systems):
    out = []
    for w in systems:
        r = w.copy()
        O.solve_noncyclic(w.m, 1, w.nrow, 1, *r.arrays)
        out.append(r.D)
    return np.concatenate(out)


def check(m, n, got, ref, tol):
    off = 0
    worst = 0.0
    for s in range(len(m)):
        k = int(m[s] * n[s])
        x, r = got[off:off + k], ref[off:off + k]
        worst = max(worst, float(np.abs(x - r).max() / np.abs(r).max()))
        off += k
    assert worst <= tol, worst


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("ff", 1e-12)])
@pytest.mark.parametrize("seg", [0, 32, 256])
@pytest.mark.parametrize("mmax", [5, 10])
def test_batch_matches_oracle(cuda, prec, tol, seg, mmax):
    """Every system against the oracle; block sizes 1..5, and 1..10."""
    m, n, systems, user = make_batch(300, 2, 700, seed=3 + mmax, mmax=mmax)
    plan = B.BatchPlan(m, n, prec, {"seg_len": {k: seg for k in range(1, 11)}, "warps_per_cta": 4})
    um, uv, pm, pv = plan.sizes()
    assert um == sum(int(mm * mm * nn) for mm, nn in zip(m, n)) and uv == sum(int(mm * nn) for mm, nn in zip(m, n))
    ua, ub, uc, ud = (torch.from_numpy(x).to(cuda) for x in user)
    pa, pb, pc, pd = plan.pack(ua, ub, uc, ud)
    plan.solve(pa, pb, pc, pd)
    assert plan.status() == (0, 0)
    got = plan.unpack(pd).cpu().numpy()
    check(m, n, got, reference(systems), tol)
    info = plan.info()
    assert info["tiles"] >= 300 // 32 and info["grid_ctas"] > 0
    assert set(np.unique(m)) == set(range(1, mmax + 1))
    if seg == 32:
        assert info["stage3_items"] > 0  # long lines were segmented
    plan.destroy()


def test_batch_user_offsets_and_layout(cuda):
    m = np.array([2, 3, 2, 1], dtype=np.int32)
    n = np.array([5, 4, 9, 3], dtype=np.int32)
    plan = B.BatchPlan(m, n, "fp64")
    mo, vo = plan.user_offsets()
    assert list(mo) == [0, 20, 56, 92] and list(vo) == [0, 10, 22, 40]
    plan.destroy()


def test_batch_graph_replay(cuda):
    m, n, systems, user = make_batch(200, 2, 400, seed=5)
    plan = B.BatchPlan(m, n, "fp64", {"seg_len": {k: 64 for k in range(1, 11)}, "warps_per_cta": 4})
    ua, ub, uc, ud = (torch.from_numpy(x).to(cuda) for x in user)
    packed = plan.pack(ua, ub, uc, ud)
    d0 = packed[3].clone()
    g = B.capture_sweeps(plan, packed, d0, sweeps=5)
    g.replay()
    torch.cuda.synchronize()
    assert plan.status() == (0, 0)
    got = plan.unpack(packed[3]).cpu().numpy()
    check(m, n, got, reference(systems), 1e-12)
    plan.destroy()


def test_batch_autotune(cuda, tmp_path):
    m, n, systems, user = make_batch(256, 16, 1024, seed=7)
    tensors = tuple(torch.from_numpy(x).to(cuda) for x in user)
    cache = tmp_path / "tune.json"
    best = B.autotune(m, n, tensors, "fp64", cache=cache)
    assert set(best) >= {"seg_len", "warps_per_cta", "ms"} and cache.exists()
    again = B.autotune(m, n, tensors, "fp64", cache=cache)
    assert again == best  # served from the cache
    plan = B.BatchPlan(m, n, "fp64", best)
    packed = plan.pack(*tensors)
    plan.solve(*packed)
    check(m, n, plan.unpack(packed[3]).cpu().numpy(), reference(systems), 1e-12)
    plan.destroy()


def test_batch_rejects_bad_shapes(cuda):
    with pytest.raises(ValueError, match="m=11"):
        B.BatchPlan([2, 11], [10, 10], "fp64")
    with pytest.raises(ValueError, match="nrow=1"):
        B.BatchPlan([2, 3], [10, 1], "fp64")
    with pytest.raises(NotImplementedError):
        B.BatchPlan([2, 3], [10, 10], "fp32_refine")
