"""Lines that share one block-tridiagonal matrix, solved in place in a
strided field (include/pbt_shared.h).

The constant-coefficient ADI sweeps of the reference's heat3d example build
the same blocks for every line (Fortran_Original/examples/heat3d/
heat3d_mpi_gpu.f90:439-509) and pack / unpack the field around each solve.
`SharedMatrix` factorises the matrix once and solves every line straight
from a right-hand-side field into a solution field, addressed by strides
(`Lines`); `Lines.packed` gives the reference GPU layout, `Lines.axis` the
lines of a 3-D field along one axis with blocks of m consecutive points.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from . import _raise


_LinesC = N.Lines

_P = C.c_void_p
SHARED_SIGNATURES = {
    "pbt_shared_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int, _P, _P, _P, C.c_int]),
    "pbt_shared_solve": (C.c_int, [_P, _P, _P, C.POINTER(_LinesC), _P]),
    "pbt_shared_shape": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pbt_shared_status": (C.c_int, [_P, _P]),
    "pbt_shared_destroy": (C.c_int, [_P]),
}
_bound = False


def _lib():
    global _bound
    lib = N.lib()
    if not _bound:
        for name, (res, args) in SHARED_SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _bound = True
    return lib


@dataclass
class Lines:
    """Where line s = s_in + nsys_inner * s_out, row q, unknown i lives:
    element s_in*stride_inner + s_out*stride_outer + q*row_stride + i*elem_stride."""

    nsys_inner: int
    nsys_outer: int
    stride_inner: int
    stride_outer: int
    row_stride: int
    elem_stride: int

    @classmethod
    def packed(cls, nsys: int, nrow: int) -> "Lines":
        """The reference GPU layout D[sys + nsys*(row + nrow*i)]."""
        return cls(nsys, 1, 1, 0, nsys, nsys * nrow)

    @classmethod
    def axis(cls, shape, axis: int, m: int) -> "Lines":
        """Lines of a C-ordered 3-D array `shape` (slowest first) along `axis`,
        each block row m consecutive points of the line; the lines run over the
        other two axes, the faster one innermost."""
        if len(shape) != 3 or shape[axis] % m:
            raise ValueError("need a 3-D shape whose axis length is a multiple of m")
        strides = [shape[1] * shape[2], shape[2], 1]
        others = [a for a in range(3) if a != axis]
        outer, inner = others  # C order: the later axis is the faster one
        return cls(shape[inner], shape[outer], strides[inner], strides[outer], m * strides[axis], strides[axis])

    def c(self) -> _LinesC:
        return _LinesC(self.nsys_inner, self.nsys_outer, self.stride_inner, self.stride_outer, self.row_stride,
                       self.elem_stride)


class SharedMatrix:
    """One block-tridiagonal matrix (nrow block rows of size m) shared by
    every line.  a, b, c: host arrays of one system, element (i, j) of row q
    at q + nrow*(i + m*j) (A_0 and C_{nrow-1} are ignored).  precision:
    "fp64" or "ff" (float-float on the FP32 pipes), the arithmetic of the
    solve; the factorisation is FP64 on the host either way."""

    def __init__(self, m: int, nrow: int, a, b, c, precision: str = "fp64"):
        from . import PRECISIONS

        if precision not in ("fp64", "ff"):
            raise ValueError(f"precision {precision!r}: SharedMatrix solves in 'fp64' or 'ff'")
        arrs = [np.ascontiguousarray(x, dtype=np.float64).reshape(-1) for x in (a, b, c)]
        for x in arrs:
            if x.size != nrow * m * m:
                raise ValueError(f"each block array needs nrow*m*m = {nrow * m * m} values")
        h = _P()
        _raise(_lib().pbt_shared_create(C.byref(h), int(m), int(nrow), *(x.ctypes.data for x in arrs),
                                        PRECISIONS[precision]), "SharedMatrix")
        self._h = h
        self.m, self.nrow, self.precision = int(m), int(nrow), precision

    def solve(self, rhs, x=None, lines: Lines | None = None, stream=None):
        """x <- M^{-1} rhs on every line (CUDA float64 tensors; x defaults to
        rhs, in place).  `lines` defaults to the packed layout of rhs."""
        import torch

        if x is None:
            x = rhs
        if lines is None:
            nsys = rhs.numel() // (self.nrow * self.m)
            lines = Lines.packed(nsys, self.nrow)
        s = torch.cuda.current_stream().cuda_stream if stream is None else stream.cuda_stream
        lc = lines.c()
        _raise(_lib().pbt_shared_solve(self._h, C.c_void_p(rhs.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(lc),
                                       C.c_void_p(s)), "SharedMatrix.solve")
        return x

    def status(self, stream=None) -> None:
        """Synchronise and raise ArithmeticRangeError if a float-float solve
        since the last call left the arithmetic's range (pbt_shared_status)."""
        import torch

        s = torch.cuda.current_stream().cuda_stream if stream is None else stream.cuda_stream
        _raise(_lib().pbt_shared_status(self._h, C.c_void_p(s)), "SharedMatrix.status")

    def destroy(self) -> None:
        if getattr(self, "_h", None):
            _raise(_lib().pbt_shared_destroy(self._h), "SharedMatrix.destroy")
            self._h = None

    def __enter__(self) -> "SharedMatrix":
        return self

    def __exit__(self, *exc) -> None:
        self.destroy()

    def __del__(self) -> None:
        try:
            self.destroy()
        except Exception:
            pass


def heat3d_blocks(nblk: int, sigma: float, is_first: bool = True, is_last: bool = True):
    """The 2x2 blocks the reference's heat3d builds for every line of a sweep
    (build_matrix_kernel, Fortran_Original/examples/heat3d/heat3d_mpi_gpu.f90:439-509),
    as (a, b, c) arrays of one system in the layout SharedMatrix takes."""
    m = 2
    A = np.zeros((m, m, nblk))
    B = np.zeros((m, m, nblk))
    Cc = np.zeros((m, m, nblk))
    A[0, 0], A[0, 1], A[1, 0], A[1, 1] = sigma, -16.0 * sigma, 0.0, sigma
    B[0, 0], B[0, 1], B[1, 0], B[1, 1] = 1.0 + 30.0 * sigma, -16.0 * sigma, -16.0 * sigma, 1.0 + 30.0 * sigma
    Cc[0, 0], Cc[0, 1], Cc[1, 0], Cc[1, 1] = sigma, 0.0, -16.0 * sigma, sigma
    if is_first:
        A[:, :, 0] = 0.0
        B[:, :, 0] = [[1.0 + 20.0 * sigma, -6.0 * sigma], [-16.0 * sigma, 1.0 + 30.0 * sigma]]
        Cc[:, :, 0] = [[-4.0 * sigma, sigma], [-16.0 * sigma, sigma]]
    if is_last:
        A[:, :, -1] = [[sigma, -16.0 * sigma], [sigma, -4.0 * sigma]]
        B[:, :, -1] = [[1.0 + 30.0 * sigma, -16.0 * sigma], [-6.0 * sigma, 1.0 + 20.0 * sigma]]
        Cc[:, :, -1] = 0.0
    # element (i, j) of row q at q + nblk*(i + m*j): axis order (j, i, q) in C order
    return tuple(np.ascontiguousarray(x.transpose(1, 0, 2)).reshape(-1) for x in (A, B, Cc))


def sweep_field(n: int, axis: int, precision: str = "ff", sweeps: int = 3, halo: int = 2, sigma: float = 0.05,
                device: str = "cuda:0") -> float:
    """Solve the heat3d lines (m = 2, n/2 blocks) along `axis` of a random
    (n + 2*halo)^3 field in place, `sweeps` times; returns ms per sweep
    (CUDA events, after one untimed sweep)."""
    import torch

    if n % 2:
        raise ValueError("n must be even (blocks of two points)")
    field = torch.rand((n + 2 * halo,) * 3, dtype=torch.float64, device=device)
    interior = field[halo:-halo, halo:-halo, halo:-halo]
    st = interior.stride()
    outer, inner = [x for x in range(3) if x != axis]
    lines = Lines(n, n, st[inner], st[outer], 2 * st[axis], st[axis])
    a, b, c = heat3d_blocks(n // 2, sigma)
    with SharedMatrix(2, n // 2, a, b, c, precision=precision) as sm:
        sm.solve(interior, interior, lines)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(sweeps):
            sm.solve(interior, interior, lines)
        e1.record()
        torch.cuda.synchronize()
    return e0.elapsed_time(e1) / sweeps


def main(argv=None) -> None:
    import argparse

    ap = argparse.ArgumentParser(description="heat3d-style sweeps of shared-matrix lines in a haloed field")
    ap.add_argument("n", type=int, help="interior points per axis (even)")
    ap.add_argument("--axis", type=int, default=0, choices=[0, 1, 2], help="0 = slowest (z), 2 = fastest (x)")
    ap.add_argument("--precision", default="ff", choices=["fp64", "ff"])
    ap.add_argument("--sweeps", type=int, default=3)
    args = ap.parse_args(argv)
    ms = sweep_field(args.n, args.axis, args.precision, args.sweeps)
    rows = args.n * args.n * (args.n // 2)
    print(f"n={args.n} axis={args.axis} precision={args.precision}: {ms:.3f} ms/sweep, "
          f"{rows / ms / 1e6:.2f} G block rows/s")


if __name__ == "__main__":
    main()
