"""Lines sharing one matrix (include/pbt_shared.h): the solve straight from
and into a strided field against the oracle on the same systems packed in
the reference layout (the matrix replicated for every line)."""
import numpy as np
import pytest
import torch

from pascal_btdma_gb300 import shared, synth
from conftest import per_system_relerr
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def one_system(m, nrow, seed, delta=1.5):
    w = synth.dominant(m, 1, nrow, seed=seed, delta=delta)
    return w.A, w.B, w.C


def replicate(x, nsys):
    """One system's block array (nrow*m*m, layout q + nrow*e) -> nsys copies in
    the reference GPU layout sys + nsys*(q + nrow*e)."""
    return np.repeat(x[:, None], nsys, axis=1).reshape(-1)


TOL = 1e-12  # FP64 and float-float (~47-bit) solves against the oracle, max-relative per line
PRECS = ["fp64", "ff"]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("m,nrow,nsys", [(1, 9, 40), (2, 64, 300), (3, 17, 33), (4, 128, 1000), (5, 40, 64),
                                          (6, 10, 7), (7, 9, 45), (8, 12, 50), (9, 5, 31), (10, 6, 33),
                                          (2, 2, 1), (3, 1000, 65)])
def test_packed_lines_match_oracle(cuda, m, nrow, nsys, prec):
    a, b, c = one_system(m, nrow, seed=10 * m + nrow)
    rng = np.random.default_rng(m)
    d = rng.uniform(-1, 1, nsys * nrow * m)
    ref = d.copy()
    O.solve_noncyclic(m, nsys, nrow, 1, replicate(a, nsys), replicate(b, nsys), replicate(c, nsys), ref)
    rhs = torch.from_numpy(d).to(cuda)
    with shared.SharedMatrix(m, nrow, a, b, c, precision=prec) as sm:
        x = torch.empty_like(rhs)
        sm.solve(rhs, x)
        sm.solve(rhs)  # in place
        torch.cuda.synchronize()
    assert torch.equal(x, rhs)
    assert per_system_relerr(m, nsys, nrow, x.cpu().numpy(), ref) <= TOL


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_heat3d_sweeps_in_a_haloed_field(cuda, axis, prec):
    """The heat3d matrix (m = 2) solved along each axis of a field with a halo
    of 2, in place in the interior, against packing the same lines for the
    oracle; the halo stays untouched."""
    n, h, sigma = (24, 20, 16), 2, 0.05
    rng = np.random.default_rng(axis)
    full = rng.uniform(-1, 1, tuple(k + 2 * h for k in n))
    nblk = n[axis] // 2
    a, b, c = shared.heat3d_blocks(nblk, sigma)
    field = torch.from_numpy(full.copy()).to(cuda)
    interior = field[h:-h, h:-h, h:-h]  # a view: data_ptr at the interior origin, strides of the full array
    st = [s for s in interior.stride()]
    others = [ax for ax in range(3) if ax != axis]
    outer, inner = others
    lines = shared.Lines(n[inner], n[outer], st[inner], st[outer], 2 * st[axis], st[axis])
    with shared.SharedMatrix(2, nblk, a, b, c, precision=prec) as sm:
        sm.solve(interior, interior, lines)
        torch.cuda.synchronize()
    got = field.cpu().numpy()
    # Oracle: pack every line in the reference layout, sys + nsys*(q + nblk*i)
    # with sys = s_in + n_inner*s_out and point 2q + i of the line, solve, unpack.
    core = full[h:-h, h:-h, h:-h]
    nsys = n[inner] * n[outer]
    L = np.moveaxis(core, [axis, outer, inner], [0, 1, 2])  # [point, s_out, s_in]
    packed = np.ascontiguousarray(L.reshape(nblk, 2, nsys).transpose(1, 0, 2)).reshape(-1)
    O.solve_noncyclic(2, nsys, nblk, 1, replicate(a, nsys), replicate(b, nsys), replicate(c, nsys), packed)
    sol = packed.reshape(2, nblk, nsys).transpose(1, 0, 2).reshape(n[axis], n[outer], n[inner])
    want = full.copy()
    want_core = np.moveaxis(sol, [0, 1, 2], [axis, outer, inner])
    want[h:-h, h:-h, h:-h] = want_core
    assert np.max(np.abs(got - want)) <= TOL * np.max(np.abs(want_core))
    assert np.array_equal(got[:h], full[:h]) and np.array_equal(got[-h:], full[-h:])


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("m,nrow,nsys", [(2, 13, 35), (3, 7, 70), (5, 4, 33), (1, 40, 5), (10, 3, 64)])
def test_contiguous_lines(cuda, m, nrow, nsys, prec):
    """Lines stored one after another (a line's rows and unknowns contiguous,
    the staging by half-warps along each line), with a ragged last warp and
    a ragged last chunk of rows, out of place, against the oracle."""
    a, b, c = one_system(m, nrow, seed=7 * m + nrow)
    rng = np.random.default_rng(100 + m)
    lines_major = rng.uniform(-1, 1, (nsys, nrow, m))  # [line][row][unknown]
    packed = np.ascontiguousarray(lines_major.transpose(2, 1, 0)).reshape(-1)  # sys + nsys*(row + nrow*i)
    O.solve_noncyclic(m, nsys, nrow, 1, replicate(a, nsys), replicate(b, nsys), replicate(c, nsys), packed)
    want = packed.reshape(m, nrow, nsys).transpose(2, 1, 0)
    rhs = torch.from_numpy(lines_major.copy()).to(cuda)
    x = torch.full_like(rhs, 7.0)
    lines = shared.Lines(nsys, 1, nrow * m, 0, m, 1)
    with shared.SharedMatrix(m, nrow, a, b, c, precision=prec) as sm:
        sm.solve(rhs, x, lines)
        torch.cuda.synchronize()
    assert torch.equal(rhs.cpu(), torch.from_numpy(lines_major))  # out of place: rhs untouched
    got = x.cpu().numpy()
    err = np.abs(got - want).max(axis=(1, 2)) / np.abs(want).max(axis=(1, 2))
    assert err.max() <= TOL
