"""Pins the CPU oracle (a restatement of Fortran_Original/src/mod_btdma_cpu.f90)
before it is trusted as the GPU checker (CPU only):
  * the reference's own recorded first-solve signatures (tests/golden/signatures.json),
  * LAPACK dgesv (scipy) for the block solves,
  * a dense numpy solve of the assembled matrix (non-cyclic and cyclic),
  * the reference partition rule and the manufactured-solution workload.
"""
import json
from pathlib import Path

import numpy as np
import pytest
import scipy.linalg as sla

from oracle import oracle as O
from pascal_btdma_gb300 import synth
from conftest import per_system_relerr

GOLDEN = json.loads((Path(__file__).parent / "golden" / "signatures.json").read_text())


def mpiutil_para(sta_g, end_g, myrank, nprocs):
    """Restated from Fortran_Original/src/mpiutil.f90:27-48 (1-based)."""
    n = end_g - sta_g + 1
    tmp1, tmp2 = n // nprocs, n % nprocs
    aa, bb = (myrank, 1) if myrank < tmp2 else (tmp2, 0)
    a = myrank * tmp1 + aa + sta_g
    return a, a + tmp1 + bb - 1


@pytest.mark.parametrize("n,p", [(128, 4), (10, 3), (7, 7), (2048, 8), (1000, 7), (5, 1)])
def test_partition_matches_mpiutil_para(n, p):
    for r in range(p):
        f, l = O.partition(n, p, r)
        a, b = mpiutil_para(1, n, r, p)
        assert (f + 1, l + 1) == (a, b)


@pytest.mark.parametrize("m", range(1, 11))
def test_dgesv_matches_lapack(m):
    rng = np.random.default_rng(m)
    for _ in range(20):
        a = rng.uniform(-1, 1, (m, m))
        b = rng.uniform(-1, 1, (m, 2 * m + 1))
        x, info = O.dgesv(a, b)
        lu, piv, xl, infol = sla.lapack.dgesv(a, b)
        assert info == infol == 0
        assert np.abs(x - xl).max() <= 1e-12 * max(1.0, np.abs(xl).max())


def test_dgesv_reports_singular_like_lapack():
    a = np.array([[1.0, 2.0], [2.0, 4.0]])
    b = np.array([[1.0], [3.0]])
    x, info = O.dgesv(a, b)
    assert info == 2
    assert np.array_equal(x, b)  # dgesv leaves b untouched when info > 0


CASES = [  # m, nsys, nrow, nseg
    (1, 7, 10, 1), (1, 7, 10, 3), (2, 5, 9, 1), (2, 5, 9, 3), (3, 6, 12, 4), (3, 6, 13, 2),
    (4, 3, 40, 8), (5, 4, 24, 3), (6, 2, 18, 6), (7, 2, 9, 3), (8, 3, 16, 5), (9, 2, 12, 4), (10, 2, 30, 3),
    (3, 4, 3, 1), (4, 2, 2, 1),
]


@pytest.mark.parametrize("m,nsys,nrow,nseg", CASES)
@pytest.mark.parametrize("delta", [1.05, 2.0])
def test_noncyclic_matches_dense_solve(m, nsys, nrow, nseg, delta):
    w = synth.dominant(m, nsys, nrow, seed=m * 100 + nseg, delta=delta)
    got = w.copy()
    assert O.solve_noncyclic(m, nsys, nrow, nseg, *got.arrays) == 0
    for s in range(nsys):
        M, rhs = O.assemble_dense(m, nsys, nrow, *w.arrays, s)
        x = np.linalg.solve(M, rhs)
        xo = O.solution_of(m, nsys, nrow, got.D, s)
        assert np.abs(xo - x).max() <= 1e-12 * np.abs(x).max()
    assert np.array_equal(got.B, w.B)  # B is read only


@pytest.mark.parametrize("m,nsys,nrow,nseg", [(1, 3, 8, 2), (2, 3, 16, 4), (3, 4, 12, 3), (4, 2, 24, 6), (5, 2, 30, 5), (8, 2, 12, 2)])
def test_cyclic_matches_dense_solve(m, nsys, nrow, nseg):
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=3 + m, delta=1.5, flags=0)  # A_0, C_{N-1} kept: periodic
    got = w.copy()
    assert O.solve_cyclic(m, nsys, nrow, nseg, *got.arrays) == 0
    for s in range(nsys):
        M, rhs = O.assemble_dense(m, nsys, nrow, *w.arrays, s, cyclic=True)
        x = np.linalg.solve(M, rhs)
        xo = O.solution_of(m, nsys, nrow, got.D, s)
        assert np.abs(xo - x).max() <= 1e-12 * np.abs(x).max()


@pytest.mark.parametrize("m,nsys,nrow", [(1, 3, 3), (1, 5, 8), (2, 3, 4), (3, 4, 12), (4, 2, 24), (5, 3, 30),
                                         (6, 2, 7), (8, 2, 12), (10, 2, 9)])
def test_whole_line_cyclic_matches_dense_solve(m, nsys, nrow):
    """btdma_many_cycl applied to a whole periodic line (one segment)."""
    w = synth.fill(synth.DOMINANT, m, nsys, nrow, seed=11 + m, delta=1.5, flags=0)
    got = w.copy()
    assert O.block_thomas_cyclic(m, nsys, nrow, *got.arrays) == 0
    for s in range(nsys):
        M, rhs = O.assemble_dense(m, nsys, nrow, *w.arrays, s, cyclic=True)
        x = np.linalg.solve(M, rhs)
        xo = O.solution_of(m, nsys, nrow, got.D, s)
        assert np.abs(xo - x).max() <= 1e-12 * np.abs(x).max()
    # The CPU-layout entry gives the same bits.
    c = [O.gpu_to_cpu(m, nsys, nrow, i < 3, v) for i, v in enumerate(w.arrays)]
    assert O.block_thomas_cyclic_cpu(m, nsys, nrow, *c) == 0
    assert np.array_equal(O.cpu_to_gpu(m, nsys, nrow, False, c[3]), got.D)


def test_whole_line_cyclic_needs_three_rows():
    w = synth.fill(synth.DOMINANT, 2, 2, 2, seed=1, delta=1.5, flags=0)
    with pytest.raises(ValueError):
        O.block_thomas_cyclic(2, 2, 2, *w.copy().arrays)


def test_matches_banded_lapack():
    m, nsys, nrow, nseg = 3, 4, 128, 4  # the small config, 4 systems
    w = synth.dominant(m, nsys, nrow, seed=1, delta=2.0)
    got = w.copy()
    O.solve_noncyclic(m, nsys, nrow, nseg, *got.arrays)
    for s in range(nsys):
        M, rhs = O.assemble_dense(m, nsys, nrow, *w.arrays, s)
        bw = 2 * m - 1
        ab = np.zeros((2 * bw + 1, M.shape[0]))
        for i in range(M.shape[0]):
            for j in range(max(0, i - bw), min(M.shape[0], i + bw + 1)):
                ab[bw + i - j, j] = M[i, j]
        x = sla.solve_banded((bw, bw), ab, rhs)
        xo = O.solution_of(m, nsys, nrow, got.D, s)
        assert np.abs(xo - x).max() <= 1e-12 * np.abs(x).max()


def test_side_effects_like_reference():
    """A <- A', C <- C' (modified factors), D <- x, B untouched."""
    m, nsys, nrow, nseg = 3, 4, 12, 2
    w = synth.dominant(m, nsys, nrow, seed=2, delta=2.0)
    got = w.copy()
    O.solve_noncyclic(m, nsys, nrow, nseg, *got.arrays)
    assert not np.array_equal(got.A, w.A) and not np.array_equal(got.C, w.C)
    assert np.array_equal(got.B, w.B)


def test_two_row_segments_are_wrong_in_the_reference_method():
    """With a 2-row segment (nseg > 1) the reference's reduced row 1 couples to
    the next segment's first row instead of its own last row; the oracle keeps
    that behaviour, the library refuses such plans (see test_abi)."""
    m, nsys, nrow, nseg = 3, 3, 12, 6
    w = synth.dominant(m, nsys, nrow, seed=4, delta=1.2)
    got = w.copy()
    O.solve_noncyclic(m, nsys, nrow, nseg, *got.arrays)
    M, rhs = O.assemble_dense(m, nsys, nrow, *w.arrays, 0)
    x = np.linalg.solve(M, rhs)
    assert np.abs(O.solution_of(m, nsys, nrow, got.D, 0) - x).max() > 1e-6 * np.abs(x).max()


def test_manufactured_solution():
    m, nsys, nrow, nseg = 3, 8, 40, 4
    w = synth.manufactured(m, nsys, nrow, seed=6)
    got = w.copy()
    O.solve_noncyclic(m, nsys, nrow, nseg, *got.arrays)
    for s in range(nsys):
        M, rhs = O.assemble_dense(m, nsys, nrow, *w.arrays, s)
        xd = np.linalg.solve(M, rhs)
        xo = O.solution_of(m, nsys, nrow, got.D, s)
        xr = O.solution_of(m, nsys, nrow, w.x_ref, s)
        cond = np.linalg.cond(M)
        assert np.abs(xo - xd).max() <= 1e-13 * cond * np.abs(xd).max()
        assert np.abs(xo - xr).max() <= 1e-14 * cond * np.abs(xr).max()


def test_thread_count_does_not_change_bits():
    m, nsys, nrow, nseg = 4, 33, 20, 3
    w = synth.dominant(m, nsys, nrow, seed=8, delta=1.5)
    a, b = w.copy(), w.copy()
    O.solve_noncyclic(m, nsys, nrow, nseg, *a.arrays, nthreads=1)
    O.solve_noncyclic(m, nsys, nrow, nseg, *b.arrays, nthreads=5)
    assert np.array_equal(a.D, b.D) and np.array_equal(a.A, b.A)


def test_cpu_layout_entry_equals_gpu_layout_entry():
    m, nsys, nrow, nseg = 3, 5, 18, 3
    w = synth.dominant(m, nsys, nrow, seed=10, delta=1.5)
    g = w.copy()
    O.solve_noncyclic(m, nsys, nrow, nseg, *g.arrays)
    c = [O.gpu_to_cpu(m, nsys, nrow, k < 3, x) for k, x in enumerate(w.arrays)]
    O.solve_noncyclic_cpu(m, nsys, nrow, nseg, *c)
    assert np.array_equal(O.gpu_to_cpu(m, nsys, nrow, False, g.D), c[3])


def signature(m, nsys, nrow, D):
    x = D.reshape(m, nrow, nsys)
    return {
        "solution_sum": float(D.sum()), "solution_l2": float(np.sqrt((D * D).sum())),
        "solution_linf": float(np.abs(D).max()), "sample_z0": float(x[0, 0, 0]),
        "sample_zmid": float(x[0, nrow // 2, 0]), "sample_zlast": float(x[0, nrow - 1, 0]),
    }


def check_signature(sig, row, nsys_run):
    """Sums over nsys_run identical systems, scaled to the recorded nsys.  The
    recorded sums are sequential sums of up to 5e7 terms; the reference's own
    sums for the same case at different rank counts differ by up to 3e-10
    relative, so sums are compared at 1e-9 and the samples at 1e-14."""
    k = row["nsys"] / nsys_run
    assert sig["solution_sum"] * k == pytest.approx(row["solution_sum"], rel=1e-9)
    assert sig["solution_l2"] * np.sqrt(k) == pytest.approx(row["solution_l2"], rel=1e-9)
    for key in ("solution_linf", "sample_z0", "sample_zmid", "sample_zlast"):
        assert sig[key] == pytest.approx(row[key], rel=1e-14, abs=1e-15)


@pytest.mark.parametrize("row", GOLDEN["rows"], ids=lambda r: f"m{r['m']}_n{r['n3']}_P{r['nseg']}_ns{r['nsys']}")
def test_reference_signatures(row):
    """The diagonal workload's systems are all identical, so a few systems
    reproduce the reference's whole-batch signature after scaling."""
    m, nrow, nseg = row["m"], row["n3"], row["nseg"]
    nsys = min(row["nsys"], 32)
    w = synth.diagonal(m, nsys, nrow)
    O.solve_noncyclic(m, nsys, nrow, nseg, *w.arrays)
    check_signature(signature(m, nsys, nrow, w.D), row, nsys)
