"""ctypes wrapper of the CPU oracle (liboracle.so).  TEST INFRASTRUCTURE ONLY.

A restatement of the reference MPI CPU path (Fortran_Original/src/mod_btdma_cpu.f90)
in C; see pbt_oracle.c for the line-by-line correspondence.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may use it, as the
checker or the timed CPU baseline, never as part of the solver.

Arrays are numpy float64 vectors in the reference GPU layout unless the
function name ends in ``_cpu`` (block-fastest layout X(m, m, nsys, nrow)).
All functions work in place like the reference: D <- x, A <- A', C <- C'.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        from . import build as _build  # noqa: F401  (package-relative when imported as oracle.oracle)

        path = _build.build()
        _lib = C.CDLL(str(path))
        P, I = C.c_void_p, C.c_int
        for name in ("pbto_solve_noncyclic", "pbto_solve_cyclic", "pbto_solve_noncyclic_cpu", "pbto_solve_cyclic_cpu"):
            getattr(_lib, name).argtypes = [I, I, I, I, P, P, P, P, I]
            getattr(_lib, name).restype = I
        for name in ("pbto_block_thomas", "pbto_block_thomas_cpu", "pbto_block_thomas_cyclic",
                     "pbto_block_thomas_cyclic_cpu"):
            getattr(_lib, name).argtypes = [I, I, I, P, P, P, P, I]
            getattr(_lib, name).restype = I
        _lib.pbto_dgesv.argtypes = [I, I, P, I, P, I]
        _lib.pbto_dgesv.restype = I
        _lib.pbto_partition.argtypes = [I, I, I, C.POINTER(I), C.POINTER(I)]
        _lib.pbto_partition.restype = None
        _lib.pbto_default_threads.argtypes = []
        _lib.pbto_default_threads.restype = I
        for name in ("pbto_gpu_to_cpu", "pbto_cpu_to_gpu"):
            getattr(_lib, name).argtypes = [I, I, I, I, P, P]
            getattr(_lib, name).restype = None
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError("oracle arrays must be contiguous float64")
    return C.c_void_p(a.ctypes.data)


def _check(rc: int, what: str) -> int:
    if rc < 0:
        raise ValueError(f"{what}: oracle rejected its arguments (rc={rc})")
    return rc


def solve_noncyclic(m, nsys, nrow, nseg, A, B, Cm, D, nthreads=0) -> int:
    """Reference non-cyclic two-stage solve; returns the number of singular dgesv calls."""
    return _check(lib().pbto_solve_noncyclic(m, nsys, nrow, nseg, _p(A), _p(B), _p(Cm), _p(D), nthreads),
                  "solve_noncyclic")


def solve_cyclic(m, nsys, nrow, nseg, A, B, Cm, D, nthreads=0) -> int:
    return _check(lib().pbto_solve_cyclic(m, nsys, nrow, nseg, _p(A), _p(B), _p(Cm), _p(D), nthreads),
                  "solve_cyclic")


def block_thomas(m, nsys, nrow, A, B, Cm, D, nthreads=0) -> int:
    return _check(lib().pbto_block_thomas(m, nsys, nrow, _p(A), _p(B), _p(Cm), _p(D), nthreads), "block_thomas")


def block_thomas_cyclic(m, nsys, nrow, A, B, Cm, D, nthreads=0) -> int:
    """A whole periodic line as one segment: btdma_many_cycl on the original rows (nrow >= 3)."""
    return _check(lib().pbto_block_thomas_cyclic(m, nsys, nrow, _p(A), _p(B), _p(Cm), _p(D), nthreads),
                  "block_thomas_cyclic")


def solve_noncyclic_cpu(m, nsys, nrow, nseg, A, B, Cm, D, nthreads=0) -> int:
    return _check(lib().pbto_solve_noncyclic_cpu(m, nsys, nrow, nseg, _p(A), _p(B), _p(Cm), _p(D), nthreads),
                  "solve_noncyclic_cpu")


def solve_cyclic_cpu(m, nsys, nrow, nseg, A, B, Cm, D, nthreads=0) -> int:
    return _check(lib().pbto_solve_cyclic_cpu(m, nsys, nrow, nseg, _p(A), _p(B), _p(Cm), _p(D), nthreads),
                  "solve_cyclic_cpu")


def block_thomas_cyclic_cpu(m, nsys, nrow, A, B, Cm, D, nthreads=0) -> int:
    return _check(lib().pbto_block_thomas_cyclic_cpu(m, nsys, nrow, _p(A), _p(B), _p(Cm), _p(D), nthreads),
                  "block_thomas_cyclic_cpu")


def gpu_to_cpu(m, nsys, nrow, is_matrix, g: np.ndarray) -> np.ndarray:
    out = np.empty_like(g)
    lib().pbto_gpu_to_cpu(m, nsys, nrow, int(is_matrix), _p(g), _p(out))
    return out


def cpu_to_gpu(m, nsys, nrow, is_matrix, c: np.ndarray) -> np.ndarray:
    out = np.empty_like(c)
    lib().pbto_cpu_to_gpu(m, nsys, nrow, int(is_matrix), _p(c), _p(out))
    return out


def dgesv(a: np.ndarray, b: np.ndarray) -> tuple[np.ndarray, int]:
    """dgesv on a column-major (Fortran-ordered) m x m matrix and m x nrhs rhs."""
    a = np.asfortranarray(a, dtype=np.float64).copy(order="F")
    b = np.asfortranarray(b, dtype=np.float64).copy(order="F")
    if b.ndim == 1:
        b = b.reshape(-1, 1, order="F")
    m, nrhs = a.shape[0], b.shape[1]
    info = lib().pbto_dgesv(m, nrhs, C.c_void_p(a.ctypes.data), m, C.c_void_p(b.ctypes.data), m)
    return b, info


def partition(n: int, p: int, seg: int) -> tuple[int, int]:
    f, l = C.c_int(), C.c_int()
    lib().pbto_partition(n, p, seg, C.byref(f), C.byref(l))
    return f.value, l.value


def default_threads() -> int:
    return lib().pbto_default_threads()


# --------------------------------------------------------------------------
# Dense cross-check (numpy): assemble one system's block-tridiagonal matrix.
# --------------------------------------------------------------------------
def assemble_dense(m, nsys, nrow, A, B, Cm, D, sys, cyclic=False):
    """Dense (nrow*m) x (nrow*m) matrix and rhs of system ``sys`` from the
    reference GPU layout; A_0 / C_{nrow-1} are dropped unless ``cyclic``."""
    n = nrow * m
    M = np.zeros((n, n))
    rhs = np.zeros(n)
    a4 = A.reshape(m, m, nrow, nsys)  # [j, i, row, sys] since index = sys + nsys*(row + nrow*(i + m*j))
    b4 = B.reshape(m, m, nrow, nsys)
    c4 = Cm.reshape(m, m, nrow, nsys)
    d3 = D.reshape(m, nrow, nsys)
    for q in range(nrow):
        r = slice(q * m, (q + 1) * m)
        M[r, r] = b4[:, :, q, sys].T
        if q > 0:
            M[r, (q - 1) * m:q * m] = a4[:, :, q, sys].T
        elif cyclic:
            M[r, (nrow - 1) * m:] += a4[:, :, q, sys].T
        if q < nrow - 1:
            M[r, (q + 1) * m:(q + 2) * m] = c4[:, :, q, sys].T
        elif cyclic:
            M[r, 0:m] += c4[:, :, q, sys].T
        rhs[r] = d3[:, q, sys]
    return M, rhs


def solution_of(m, nsys, nrow, D, sys):
    """x of system ``sys`` as a (nrow*m,) vector from the reference GPU layout."""
    return D.reshape(m, nrow, nsys)[:, :, sys].T.reshape(-1)
