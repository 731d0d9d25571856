"""Seeded synthetic workloads (libpbt_synth.so, include/pbt_synth.h) as numpy arrays.

Arrays come back in the reference GPU layout, flattened:
A, B, C of nsys*nrow*m*m doubles and D of nsys*nrow*m doubles,
element (sys, row, i, j) at sys + nsys*(row + nrow*(i + m*j)).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N

DOMINANT = 0
DIAGONAL = 1
MANUFACTURED = 2
ZERO_ENDS = 0x1
ROW_SCALE = 0x2


@dataclass
class Workload:
    m: int
    nsys: int
    nrow: int
    A: np.ndarray
    B: np.ndarray
    C: np.ndarray
    D: np.ndarray
    x_ref: np.ndarray | None = None

    @property
    def arrays(self):
        return self.A, self.B, self.C, self.D

    def copy(self) -> "Workload":
        return Workload(self.m, self.nsys, self.nrow, self.A.copy(), self.B.copy(), self.C.copy(), self.D.copy(),
                        None if self.x_ref is None else self.x_ref.copy())


def _p(a: np.ndarray) -> C.c_void_p:
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return C.c_void_p(a.ctypes.data)


def fill(kind: int, m: int, nsys: int, nrow: int, seed: int = 0, delta: float = 2.0, flags: int = ZERO_ENDS,
         nthreads: int = 0, out: tuple | None = None, alloc=None) -> Workload:
    """Generate one workload.  ``alloc(n)`` may supply the buffers (e.g. pinned
    host memory as numpy views); ``out`` may pass (A, B, C, D) to fill."""
    nm, nv = nsys * nrow * m * m, nsys * nrow * m
    if out is not None:
        A, B, Cc, D = out
    else:
        mk = alloc or (lambda n: np.empty(n, dtype=np.float64))
        A, B, Cc, D = mk(nm), mk(nm), mk(nm), mk(nv)
    x = np.empty(nv, dtype=np.float64) if kind == MANUFACTURED else None
    rc = N.synth_lib().pbt_synth_fill(
        int(kind), int(flags), int(m), int(nsys), int(nrow), C.c_uint64(seed), float(delta),
        _p(A), _p(B), _p(Cc), _p(D), _p(x) if x is not None else None, int(nthreads),
    )
    if rc != 0:
        raise ValueError("pbt_synth_fill rejected its arguments")
    return Workload(m, nsys, nrow, A, B, Cc, D, x)


def dominant(m, nsys, nrow, seed=0, delta=2.0, row_scale=False, **kw) -> Workload:
    """A, C, d, R iid U[-1,1); B = R + diag(delta*rowsum(|A|+|C|+|R|)); A_0 = C_{N-1} = 0."""
    return fill(DOMINANT, m, nsys, nrow, seed, delta, ZERO_ENDS | (ROW_SCALE if row_scale else 0), **kw)


def diagonal(m, nsys, nrow, **kw) -> Workload:
    """The reference Study workload A = 0.25 I, B = 2 I, C = 0.25 I, d = 1."""
    return fill(DIAGONAL, m, nsys, nrow, 0, 0.0, 0, **kw)


def manufactured(m, nsys, nrow, seed=0, **kw) -> Workload:
    """Known solution x(row, i) = 100*(row+1) + (i+1) with A, C ~ U(-0.4, 0.4), B = I - (A + C)."""
    return fill(MANUFACTURED, m, nsys, nrow, seed, 0.0, ZERO_ENDS, **kw)


def uniform(seed: int, stream: int, sys: int, row: int, elem: int) -> float:
    return N.synth_lib().pbt_synth_uniform(C.c_uint64(seed), stream, sys, row, elem)


def philox4x32_10(ctr, key) -> tuple[int, int, int, int]:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    N.synth_lib().pbt_philox4x32_10(c, k, o)
    return tuple(o)


def uneven_shapes(seed: int, nsys: int, nmin=16, nmax=4096, mmin=2, mmax=5) -> tuple[np.ndarray, np.ndarray]:
    n = np.empty(nsys, dtype=np.int32)
    m = np.empty(nsys, dtype=np.int32)
    rc = N.synth_lib().pbt_synth_uneven_shapes(C.c_uint64(seed), nsys, nmin, nmax, mmin, mmax,
                                               C.c_void_p(n.ctypes.data), C.c_void_p(m.ctypes.data))
    if rc != 0:
        raise ValueError("pbt_synth_uneven_shapes rejected its arguments")
    return n, m


def fill_batch(m_per_sys, n_per_sys, seed=0, delta=1.5, kind=DOMINANT, flags=ZERO_ENDS, nthreads=0, alloc=None):
    """An uneven batch in the per-system layout of include/pbt_batch.h.
    Returns (A, B, C, D, mat_off, vec_off) as flat numpy arrays."""
    m = np.ascontiguousarray(m_per_sys, dtype=np.int32)
    n = np.ascontiguousarray(n_per_sys, dtype=np.int32)
    mo = np.concatenate([[0], np.cumsum(n.astype(np.int64) * m * m)[:-1]]).astype(np.int64)
    vo = np.concatenate([[0], np.cumsum(n.astype(np.int64) * m)[:-1]]).astype(np.int64)
    nm = int((n.astype(np.int64) * m * m).sum())
    nv = int((n.astype(np.int64) * m).sum())
    mk = alloc or (lambda k: np.empty(k, dtype=np.float64))
    A, B, Cc, D = mk(nm), mk(nm), mk(nm), mk(nv)
    rc = N.synth_lib().pbt_synth_fill_batch(int(kind), int(flags), int(m.size), m.ctypes.data, n.ctypes.data,
                                            mo.ctypes.data, vo.ctypes.data, C.c_uint64(seed), float(delta),
                                            _p(A), _p(B), _p(Cc), _p(D), int(nthreads))
    if rc != 0:
        raise ValueError("pbt_synth_fill_batch rejected its arguments")
    return A, B, Cc, D, mo, vo
