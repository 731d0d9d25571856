"""Strided lines (pbt_solve_noncyclic_lines): the general solve run directly
in an application's own arrays, against the oracle on the same systems in
the reference layout.  The application layout is euler3d's: U(n1,n2,n3,m)
and trA(n1,n2,n3,m,m) in Fortran order, i.e. element e of point (i, j, k)
at i + n1*(j + n2*(k + n3*e))."""
import numpy as np
import pytest
import torch

import pascal_btdma_gb300 as pbt
from pascal_btdma_gb300 import synth
from conftest import per_system_relerr
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-12  # FP64 and float-float against the oracle, max-relative per system
SHAPE = (24, 20, 16)  # n1, n2, n3

# Per sweep: (rows axis, inner axis, outer axis) as indices into (i, j, k),
# and the axes of the C-order array [e, k, j, i] that give [e, row, s_out, s_in].
SWEEPS = {"x": ((0, 1, 2), (0, 3, 1, 2)), "y": ((1, 0, 2), (0, 2, 1, 3)), "z": ((2, 0, 1), (0, 1, 2, 3))}


def sweep_lines(sweep, shape, base_strides):
    (ra, ia, oa), _ = SWEEPS[sweep]
    st = base_strides  # element strides of i, j, k, e
    return pbt.Lines(shape[ia], shape[oa], st[ia], st[oa], st[ra], st[3])


def to_app(packed, E, sweep, shape):
    """Reference layout [e, row, s_out, s_in] -> application [e, k, j, i]."""
    (ra, ia, oa), perm = SWEEPS[sweep]
    P = packed.reshape(E, shape[ra], shape[oa], shape[ia])
    return np.ascontiguousarray(P.transpose(np.argsort(perm)))


def to_ref(app, sweep):
    _, perm = SWEEPS[sweep]
    return np.ascontiguousarray(app.transpose(perm)).reshape(-1)


def dense_strides(shape):
    n1, n2, n3 = shape
    return (1, n1, n1 * n2, n1 * n2 * n3)


@pytest.mark.parametrize("sweep", ["x", "y", "z"])
@pytest.mark.parametrize("m,prec,inplace", [(5, "ff", False), (5, "fp64", True), (3, "fp64", False),
                                            (4, "ff", True), (2, "ff", False), (6, "fp64", False)])
def test_euler3d_layout_sweeps(cuda, sweep, m, prec, inplace):
    (ra, ia, oa), _ = SWEEPS[sweep]
    nrow, nsys = SHAPE[ra], SHAPE[ia] * SHAPE[oa]
    w = synth.dominant(m, nsys, nrow, seed=31 * m + ord(sweep))
    ref = w.copy()
    O.solve_noncyclic(m, nsys, nrow, 1, *ref.arrays)
    app = [to_app(x, m * m if k < 3 else m, sweep, SHAPE) for k, x in enumerate(w.arrays)]
    a, b, c, d = (torch.from_numpy(x).to(cuda) for x in app)
    lines = sweep_lines(sweep, SHAPE, dense_strides(SHAPE))
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, precision=prec, inplace=inplace)
        pbt.solve_noncyclic_lines(plan, a, b, c, d, lines)
        assert plan.status() == 0
    got = to_ref(d.cpu().numpy(), sweep)
    assert per_system_relerr(m, nsys, nrow, got, ref.D) <= TOL
    assert np.array_equal(a.cpu().numpy(), app[0]) and np.array_equal(b.cpu().numpy(), app[1])
    if not inplace:
        assert np.array_equal(c.cpu().numpy(), app[2])


@pytest.mark.parametrize("m,prec", [(2, "fp64"), (5, "ff"), (6, "ff"), (3, "fp64")])
def test_packed_lines_are_the_plain_solve(cuda, m, prec):
    """Lines in the reference layout give the plain solve's bits."""
    nsys, nrow = 200, 33
    w = synth.dominant(m, nsys, nrow, seed=5 + m)
    arrs = [torch.from_numpy(x).to(cuda) for x in w.arrays]
    d2 = arrs[3].clone()
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, precision=prec, direct_loads=True)
        pbt.solve_noncyclic(plan, *arrs, m, nsys, nrow)
        pbt.solve_noncyclic_lines(plan, *arrs[:3], d2, pbt.Lines.packed(nsys, nrow))
        torch.cuda.synchronize()
    assert torch.equal(arrs[3], d2)


def test_haloed_arrays_need_an_inplace_plan(cuda):
    """Arrays with a halo of 2 around the interior: the lines span more than
    the plan's workspace, so only an in-place plan takes them; the halo stays
    untouched and the interior matches the oracle."""
    m, h, sweep = 3, 2, "y"
    (ra, ia, oa), _ = SWEEPS[sweep]
    nrow, nsys = SHAPE[ra], SHAPE[ia] * SHAPE[oa]
    w = synth.dominant(m, nsys, nrow, seed=77)
    ref = w.copy()
    O.solve_noncyclic(m, nsys, nrow, 1, *ref.arrays)
    n1, n2, n3 = SHAPE
    full_shape = (n1 + 2 * h, n2 + 2 * h, n3 + 2 * h)
    rng = np.random.default_rng(0)
    fulls, views = [], []
    for k, x in enumerate(w.arrays):
        E = m * m if k < 3 else m
        full = rng.uniform(-1, 1, (E, full_shape[2], full_shape[1], full_shape[0]))
        full[:, h:-h, h:-h, h:-h] = to_app(x, E, sweep, SHAPE)
        fulls.append(full)
        t = torch.from_numpy(full.copy()).to(cuda)
        views.append(t)
    F1, F2, F3 = full_shape
    strides = (1, F1, F1 * F2, F1 * F2 * F3)
    org = h * (1 + F1 + F1 * F2)  # the interior origin
    lines = sweep_lines(sweep, SHAPE, strides)
    interior = [t.view(-1)[org:] for t in views]
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, precision="ff")
        with pytest.raises(NotImplementedError):
            pbt.solve_noncyclic_lines(plan, *interior, lines)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, precision="ff", inplace=True)
        pbt.solve_noncyclic_lines(plan, *interior, lines)
        assert plan.status() == 0
    dfull = views[3].cpu().numpy()
    got = to_ref(dfull[:, h:-h, h:-h, h:-h], sweep)
    assert per_system_relerr(m, nsys, nrow, got, ref.D) <= TOL
    mask = np.ones(dfull.shape, bool)
    mask[:, h:-h, h:-h, h:-h] = False
    assert np.array_equal(dfull[mask], fulls[3][mask])


def test_lines_solve_refuses_other_plans(cuda):
    m, nsys, nrow = 3, 64, 12
    arrs = [torch.zeros(nsys * nrow * m * m, dtype=torch.float64, device=cuda) for _ in range(3)]
    arrs.append(torch.zeros(nsys * nrow * m, dtype=torch.float64, device=cuda))
    good = pbt.Lines.packed(nsys, nrow)
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1)
        with pytest.raises(ValueError):
            pbt.solve_noncyclic_lines(plan, *arrs, pbt.Lines.packed(nsys - 1, nrow))
        with pytest.raises(ValueError):
            pbt.solve_noncyclic_lines(plan, *arrs, pbt.Lines(nsys, 1, 1, 0, -nsys, nsys * nrow))
    for kw in ({"nseg": 2}, {"nseg": 2, "cyclic": True}, {"precision": "fp32_refine"}, {"cpu_layout": True},
               {"reference_method": True}):
        nseg = kw.pop("nseg", 1)
        with pbt.BtdmaGpuPlan() as plan:
            plan.create(m, nsys, nrow, nseg, **kw)
            with pytest.raises(NotImplementedError):
                pbt.solve_noncyclic_lines(plan, *arrs, good)


@pytest.mark.parametrize("shape", [SHAPE, (40, 7, 5)])  # (40, 7, 5): 35 lines of 40 rows, ragged 32-tiles
@pytest.mark.parametrize("m,prec,inplace", [(5, "ff", False), (3, "fp64", True), (2, "ff", True), (6, "fp64", False)])
def test_fast_axis_lines_are_the_plain_solve(cuda, m, prec, inplace, shape):
    """Lines along the contiguous index (the x sweep: row stride 1) go through
    tiled transposes into the reference layout and back: the plain solve's
    bits, and in place C' back in the application's layout."""
    sweep = "x"
    (ra, ia, oa), _ = SWEEPS[sweep]
    nrow, nsys = shape[ra], shape[ia] * shape[oa]
    w = synth.dominant(m, nsys, nrow, seed=90 + m)
    app = [to_app(x, m * m if k < 3 else m, sweep, shape) for k, x in enumerate(w.arrays)]
    a, b, c, d = (torch.from_numpy(x).to(cuda) for x in app)
    packed = [torch.from_numpy(x.copy()).to(cuda) for x in w.arrays]
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, precision=prec, inplace=inplace)
        pbt.solve_noncyclic_lines(plan, a, b, c, d, sweep_lines(sweep, shape, dense_strides(shape)))
    with pbt.BtdmaGpuPlan() as plan:
        plan.create(m, nsys, nrow, 1, precision=prec, inplace=inplace, direct_loads=True)
        pbt.solve_noncyclic(plan, *packed, m, nsys, nrow)
    torch.cuda.synchronize()
    assert np.array_equal(to_ref(d.cpu().numpy(), sweep), packed[3].cpu().numpy())
    if inplace:
        assert np.array_equal(to_ref(c.cpu().numpy(), sweep), packed[2].cpu().numpy())
    else:
        assert np.array_equal(c.cpu().numpy(), app[2])
