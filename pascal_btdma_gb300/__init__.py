"""pascal_btdma_gb300 -- GB300-native batched block-tridiagonal solver.

Host-side mirror of PaScaL_BTDMA's CUDA C++ API
(CUDA_CXX_Port/include/pascal_btdma_cuda.hpp) over the C ABI of
``include/pbt.h``:

    reference (namespace pascal_btdma)        here
    -----------------------------------       -----------------------------------
    BtdmaGpuPlan::create(m, nsys, nrow, comm) BtdmaGpuPlan.create(m, nsys, nrow, nseg)
    BtdmaGpuPlan::destroy()                   BtdmaGpuPlan.destroy()
    solve_noncyclic(plan, a, b, c, d, m,      solve_noncyclic(plan, a, b, c, d, m,
                    nsys, nrow, stream)                       nsys, nrow, stream)
    solve_noncyclic_profiled(..., timings,    solve_noncyclic_profiled(..., timings,
                             stream)                                   stream)
    solve_cyclic(...)                         solve_cyclic(...)
    BtdmaSolveTimings                         BtdmaSolveTimings
    partition_1d(start, end, n, r, f, l)      partition_1d(start, end, n, r) -> (f, l)
    matrix_index / vector_index               matrix_index / vector_index
    CudaError                                 CudaError
    std::invalid_argument                     ValueError
    std::runtime_error (uncreated plan)       RuntimeError
    std::logic_error (not implemented)        NotImplementedError

One GPU replaces the MPI communicator: ``nseg`` is the number of segments P
each line is split into (the reference's ranks along the line) and ``nrow``
is the full line length.  Arrays are CUDA float64 tensors (or raw device
addresses) in the reference GPU layout; D is overwritten with the solution.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

from . import _native as N

__all__ = [
    "BtdmaGpuPlan",
    "BtdmaSolveTimings",
    "CudaError",
    "SingularBlockError",
    "solve_noncyclic",
    "solve_noncyclic_profiled",
    "solve_cyclic",
    "adjoint_noncyclic",
    "BlockTridiagonalSolve",
    "partition_1d",
    "matrix_index",
    "vector_index",
    "K_MAX_BLOCK_SIZE",
]

K_MAX_BLOCK_SIZE = N.PBT_MAX_BLOCK

PRECISIONS = {"fp64": N.PBT_PREC_FP64, "ff": N.PBT_PREC_FF, "fp32_refine": N.PBT_PREC_FP32_REFINE}


class CudaError(RuntimeError):
    """A CUDA runtime call failed (the reference's pascal_btdma::CudaError)."""


class SingularBlockError(ArithmeticError):
    """A zero pivot was met in some m x m block."""


class DeviceWaitTimeout(RuntimeError):
    """A kernel's bounded wait for its staged input ran out; the solve's result is not valid."""


class ArithmeticRangeError(ArithmeticError):
    """A float-float or FP32 solve left its arithmetic's range (an input outside
    2^-96 <= |x| < 2^96, an overflow, or a solution below 2^-100); the solution
    is not valid -- solve with precision "fp64"."""


class RefinementNotConverged(ArithmeticError):
    """The FP32-refined solve did not reach its tolerance in max_iter FP32 solves."""


def _raise(code: int, where: str) -> None:
    if code == N.PBT_OK:
        return
    msg = f"{where}: {N.last_error()}"
    if code == N.PBT_EINVAL:
        raise ValueError(msg)
    if code == N.PBT_ECUDA:
        raise CudaError(msg)
    if code == N.PBT_ESTATE:
        raise RuntimeError(msg)
    if code == N.PBT_EUNSUPPORTED:
        raise NotImplementedError(msg)
    if code == N.PBT_ENOMEM:
        raise MemoryError(msg)
    if code == N.PBT_ESINGULAR:
        raise SingularBlockError(msg)
    if code == N.PBT_ETIMEOUT:
        raise DeviceWaitTimeout(msg)
    if code == N.PBT_ERANGE:
        raise ArithmeticRangeError(msg)
    if code == N.PBT_ENOCONV:
        raise RefinementNotConverged(msg)
    raise RuntimeError(f"{where}: status {code}: {N.last_error()}")


@dataclass
class BtdmaSolveTimings:
    """Phase times in seconds (pascal_btdma_cuda.hpp:24-39)."""

    total: float = 0.0
    local_compute: float = 0.0
    forward_exchange: float = 0.0
    reduced_compute: float = 0.0
    backward_exchange: float = 0.0
    update_compute: float = 0.0

    def computation(self) -> float:
        return self.local_compute + self.reduced_compute + self.update_compute

    def communication(self) -> float:
        return self.forward_exchange + self.backward_exchange


@dataclass
class BtdmaGpuPlan:
    """Plan for ``nsys`` systems of ``nrow`` block rows of size ``m``, each line
    split into ``nseg`` segments.  Owns its device workspace; not safe for
    overlapping solves (pascal_btdma_cuda.hpp:88-135)."""

    m: int = 0
    nsys: int = 0
    nrow: int = 0
    nseg: int = 1
    precision: str = "fp64"
    cyclic: bool = False
    inplace: bool = False
    reference_method: bool = False
    direct_loads: bool = False
    staged_loads: bool = False
    cpu_layout: bool = False
    created: bool = False
    _handle: C.c_void_p = field(default_factory=C.c_void_p, repr=False)

    def create(
        self,
        m: int,
        nsys: int,
        nrow: int,
        nseg: int = 1,
        *,
        precision: str = "fp64",
        cyclic: bool = False,
        inplace: bool = False,
        reference_method: bool = False,
        direct_loads: bool = False,
        staged_loads: bool = False,
        cpu_layout: bool = False,
        tol: float = 1e-12,
        max_iter: int = 8,
        threads_per_block: int = 0,
    ) -> "BtdmaGpuPlan":
        self.destroy()
        if precision not in PRECISIONS:
            raise ValueError(f"unknown precision {precision!r}; expected one of {sorted(PRECISIONS)}")
        d = N.PlanDesc()
        N.lib().pbt_plan_desc_init(C.byref(d))
        d.m, d.nsys, d.nrow, d.nseg = int(m), int(nsys), int(nrow), int(nseg)
        d.precision = PRECISIONS[precision]
        d.flags = (
            (N.PBT_FLAG_CYCLIC if cyclic else 0)
            | (N.PBT_FLAG_INPLACE if inplace else 0)
            | (N.PBT_FLAG_REFERENCE_METHOD if reference_method else 0)
            | (N.PBT_FLAG_DIRECT_LOADS if direct_loads else 0)
            | (N.PBT_FLAG_STAGED_LOADS if staged_loads else 0)
            | (N.PBT_FLAG_CPU_LAYOUT if cpu_layout else 0)
        )
        d.tol = float(tol)
        d.max_iter = int(max_iter)
        d.threads_per_block = int(threads_per_block)
        h = C.c_void_p()
        _raise(N.lib().pbt_plan_create_ex(C.byref(h), C.byref(d)), "BtdmaGpuPlan.create")
        self._handle = h
        self.m, self.nsys, self.nrow, self.nseg = d.m, d.nsys, d.nrow, d.nseg
        self.precision, self.cyclic, self.inplace = precision, cyclic, inplace
        self.reference_method = reference_method
        self.direct_loads, self.staged_loads, self.cpu_layout = direct_loads, staged_loads, cpu_layout
        self.created = True
        return self

    def destroy(self) -> None:
        if self.created and self._handle:
            _raise(N.lib().pbt_plan_destroy(self._handle), "BtdmaGpuPlan.destroy")
        self._handle = C.c_void_p()
        self.created = False

    @property
    def handle(self) -> C.c_void_p:
        return self._handle

    def workspace_bytes(self) -> int:
        return int(N.lib().pbt_plan_workspace_bytes(self._handle)) if self.created else 0

    def status(self) -> int:
        """Synchronise and return the number of zero pivots met since the last
        call; raises DeviceWaitTimeout, ArithmeticRangeError or
        RefinementNotConverged for those outcomes (pbt_plan_status)."""
        n = C.c_longlong(0)
        code = N.lib().pbt_plan_status(self._handle, C.byref(n))
        if code not in (N.PBT_OK, N.PBT_ESINGULAR):
            _raise(code, "BtdmaGpuPlan.status")
        return int(n.value)

    def refine_info(self) -> tuple[int, float]:
        """(FP32 solves run, last correction size) of the last refined solve."""
        it, corr = C.c_int(0), C.c_double(0.0)
        _raise(N.lib().pbt_plan_refine_info(self._handle, C.byref(it), C.byref(corr)), "refine_info")
        return it.value, corr.value

    def __enter__(self) -> "BtdmaGpuPlan":
        return self

    def __exit__(self, *exc) -> None:
        self.destroy()

    def __del__(self) -> None:
        try:
            self.destroy()
        except Exception:
            pass


def _ptr(x) -> int:
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        if not x.is_cuda:
            raise ValueError("arrays must be CUDA device tensors")
        import torch

        if x.dtype != torch.float64:
            raise ValueError(f"arrays must be float64, got {x.dtype}")
        if not x.is_contiguous():
            raise ValueError("arrays must be contiguous")
        return x.data_ptr()
    raise TypeError(f"expected a CUDA tensor or a device address, got {type(x).__name__}")


def _stream(stream, arrays) -> int:
    if stream is None:
        if any(hasattr(a, "data_ptr") for a in arrays):
            import torch

            return torch.cuda.current_stream().cuda_stream
        return 0
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _check_sizes(plan: BtdmaGpuPlan, arrays) -> None:
    need_m = plan.nsys * plan.nrow * plan.m * plan.m
    need_v = plan.nsys * plan.nrow * plan.m
    for name, a, need in zip("abcd", arrays, (need_m, need_m, need_m, need_v)):
        if hasattr(a, "numel") and a.numel() < need:
            raise ValueError(f"array {name} holds {a.numel()} elements, the plan needs {need}")


def _solve(fn, where, plan, a, b, c, d, m, nsys, nrow, stream, extra=()):
    if not isinstance(plan, BtdmaGpuPlan) or not plan.created:
        raise RuntimeError(f"{where} called with an uncreated BtdmaGpuPlan")
    arrays = (a, b, c, d)
    _check_sizes(plan, arrays)
    s = _stream(stream, arrays)
    code = fn(plan.handle, *(C.c_void_p(_ptr(x)) for x in arrays), int(m), int(nsys), int(nrow), *extra, C.c_void_p(s))
    _raise(code, where)


def solve_noncyclic(plan, a, b, c, d, m, nsys, nrow, stream=None) -> None:
    """Solve every system in place: D <- x (pascal_btdma_cuda.hpp:137-145)."""
    _solve(N.lib().pbt_solve_noncyclic, "solve_noncyclic", plan, a, b, c, d, m, nsys, nrow, stream)


def solve_noncyclic_profiled(plan, a, b, c, d, m, nsys, nrow, timings=None, stream=None) -> BtdmaSolveTimings:
    """As solve_noncyclic, filling per-phase times (pascal_btdma_cuda.hpp:147-156)."""
    t = N.Timings()
    _solve(
        N.lib().pbt_solve_noncyclic_profiled,
        "solve_noncyclic_profiled",
        plan, a, b, c, d, m, nsys, nrow, stream,
        extra=(C.byref(t),),
    )
    out = timings if timings is not None else BtdmaSolveTimings()
    for f in ("total", "local_compute", "forward_exchange", "reduced_compute", "backward_exchange", "update_compute"):
        setattr(out, f, getattr(t, f))
    return out


def solve_cyclic(plan, a, b, c, d, m, nsys, nrow, stream=None) -> None:
    """Periodic lines (mod_btdma_gpu_v2.f90:200-239); needs a plan created with
    ``cyclic=True``; ``nseg = 1`` (``nrow >= 3``) solves each periodic line in
    one pass, ``nseg >= 2`` by the two-stage method."""
    _solve(N.lib().pbt_solve_cyclic, "solve_cyclic", plan, a, b, c, d, m, nsys, nrow, stream)


def solve_noncyclic_lines(plan, a, b, c, d, lines, stream=None) -> None:
    """Solve lines that live in the caller's own arrays, addressed by
    ``lines`` (a ``Lines``; the same strides for A, B, C and D, which may be
    strided views): D <- x.  Replaces the transposes the reference's
    applications run around each solve (euler3d_mpi_gpu.f90:931-1017).  The
    plan: single segment, non-cyclic, FP64 or "ff", ``nsys`` lines; an
    ``inplace`` plan writes C' into C, any other needs a dense layout."""
    if not isinstance(plan, BtdmaGpuPlan) or not plan.created:
        raise RuntimeError("solve_noncyclic_lines called with an uncreated BtdmaGpuPlan")
    import torch

    arrays = (a, b, c, d)
    for x in arrays:
        if not (hasattr(x, "data_ptr") and x.is_cuda and x.dtype == torch.float64):
            raise ValueError("arrays must be float64 CUDA tensors (strided views allowed)")
    lc = lines.c() if hasattr(lines, "c") else lines
    s = _stream(stream, arrays)
    _raise(N.lib().pbt_solve_noncyclic_lines(plan.handle, *(C.c_void_p(x.data_ptr()) for x in arrays), C.byref(lc),
                                             C.c_void_p(s)), "solve_noncyclic_lines")


def partition_1d(start: int, end: int, nprocs: int, rank: int) -> tuple[int, int]:
    """(first, last) of part ``rank`` of [start, end] (pascal_btdma_cuda.cu:921-930)."""
    f, l = C.c_int(), C.c_int()
    N.lib().pbt_partition_1d(int(start), int(end), int(nprocs), int(rank), C.byref(f), C.byref(l))
    return f.value, l.value


def matrix_index(sys: int, row: int, p: int, q: int, nsys: int, nrow: int, m: int) -> int:
    """Element (p, q) of block (sys, row) (pascal_btdma_cuda.hpp:46-56)."""
    return sys + nsys * (row + nrow * (p + m * q))


def vector_index(sys: int, row: int, p: int, nsys: int, nrow: int) -> int:
    """Element p of vector (sys, row) (pascal_btdma_cuda.hpp:58-65)."""
    return sys + nsys * (row + nrow * p)


def cpu_matrix_index(sys: int, row: int, p: int, q: int, nsys: int, m: int) -> int:
    """Element (p, q) of block (sys, row) in the reference CPU layout a(m, m, nsys, n)
    (Fortran_Original/src/mod_btdma_cpu.f90:18), used by plans with cpu_layout=True."""
    return p + m * (q + m * (sys + nsys * row))


def cpu_vector_index(sys: int, row: int, p: int, nsys: int, m: int) -> int:
    """Element p of vector (sys, row) in the reference CPU layout d(m, nsys, n)."""
    return p + m * (sys + nsys * row)


def adjoint_noncyclic(plan, a, b, c, x, g, da=None, db=None, dc=None, m=None, nsys=None, nrow=None, stream=None) -> None:
    """Adjoint of the non-cyclic solve: g (dL/dx) <- lambda = dL/dd; da, db, dc
    (optional) <- dL/dA, dL/dB, dL/dC.  a, b, c, x are the forward blocks and
    solution, unchanged."""
    if not isinstance(plan, BtdmaGpuPlan) or not plan.created:
        raise RuntimeError("adjoint_noncyclic called with an uncreated BtdmaGpuPlan")
    m = plan.m if m is None else m
    nsys = plan.nsys if nsys is None else nsys
    nrow = plan.nrow if nrow is None else nrow
    arrays = (a, b, c, x, g) + tuple(t for t in (da, db, dc) if t is not None)
    s = _stream(stream, arrays)
    opt = [C.c_void_p(_ptr(t)) if t is not None else None for t in (da, db, dc)]
    code = N.lib().pbt_adjoint_noncyclic(plan.handle, *(C.c_void_p(_ptr(t)) for t in (a, b, c, x, g)), *opt,
                                         int(m), int(nsys), int(nrow), C.c_void_p(s))
    _raise(code, "adjoint_noncyclic")


def _autograd_function():
    import torch

    class _Solve(torch.autograd.Function):
        """x = M^{-1} d for the batched block-tridiagonal M given by (A, B, C),
        differentiable in A, B, C and d through the hand-written adjoint."""

        @staticmethod
        def forward(ctx, A, B, C, d, plan):
            x = d.detach().clone()
            solve_noncyclic(plan, A.detach(), B.detach(), C.detach(), x, plan.m, plan.nsys, plan.nrow)
            ctx.plan = plan
            ctx.save_for_backward(A, B, C, x)
            return x

        @staticmethod
        def backward(ctx, grad_x):
            A, B, C, x = ctx.saved_tensors
            plan = ctx.plan
            lam = grad_x.detach().clone().contiguous()
            need = ctx.needs_input_grad
            dA = torch.empty_like(A) if need[0] else None
            dB = torch.empty_like(B) if need[1] else None
            dC = torch.empty_like(C) if need[2] else None
            adjoint_noncyclic(plan, A.detach(), B.detach(), C.detach(), x, lam, dA, dB, dC)
            return dA, dB, dC, (lam if need[3] else None), None

    return _Solve


class _LazySolve:
    _fn = None

    def apply(self, A, B, C, d, plan):
        if _LazySolve._fn is None:
            _LazySolve._fn = _autograd_function()
        return _LazySolve._fn.apply(A, B, C, d, plan)


BlockTridiagonalSolve = _LazySolve()

from .shared import Lines  # noqa: E402  (shared imports _raise from this module)
