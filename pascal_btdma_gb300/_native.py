"""ctypes binding of libpbt.so (include/pbt.h) and libpbt_synth.so (include/pbt_synth.h).

The libraries are built in tree by ``pascal_btdma_gb300.build``.  Nothing here
falls back to another implementation: a missing library is an error.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libpbt.so"
SYNTH_PATH = PKG / "libpbt_synth.so"

PBT_OK = 0
PBT_EINVAL = 1
PBT_ECUDA = 2
PBT_ESTATE = 3
PBT_EUNSUPPORTED = 4
PBT_ENOMEM = 5
PBT_ESINGULAR = 6
PBT_ETIMEOUT = 7
PBT_ERANGE = 8
PBT_ENOCONV = 9

PBT_PREC_FP64 = 0
PBT_PREC_FF = 1
PBT_PREC_FP32_REFINE = 2

PBT_FLAG_CYCLIC = 0x1
PBT_FLAG_INPLACE = 0x2
PBT_FLAG_REFERENCE_METHOD = 0x4
PBT_FLAG_DIRECT_LOADS = 0x8
PBT_FLAG_STAGED_LOADS = 0x10
PBT_FLAG_CPU_LAYOUT = 0x20

PBT_MAX_BLOCK = 10


class PlanDesc(C.Structure):
    _fields_ = [
        ("m", C.c_int),
        ("nsys", C.c_int),
        ("nrow", C.c_int),
        ("nseg", C.c_int),
        ("precision", C.c_int),
        ("flags", C.c_uint),
        ("tol", C.c_double),
        ("max_iter", C.c_int),
        ("threads_per_block", C.c_int),
        ("reserved", C.c_int * 7),
    ]


class Timings(C.Structure):
    _fields_ = [
        ("total", C.c_double),
        ("local_compute", C.c_double),
        ("forward_exchange", C.c_double),
        ("reduced_compute", C.c_double),
        ("backward_exchange", C.c_double),
        ("update_compute", C.c_double),
    ]


class Lines(C.Structure):
    """pbt_lines: line s = s_in + nsys_inner*s_out, row q, element e at
    s_in*stride_inner + s_out*stride_outer + q*row_stride + e*elem_stride."""

    _fields_ = [("nsys_inner", C.c_int), ("nsys_outer", C.c_int), ("stride_inner", C.c_longlong),
                ("stride_outer", C.c_longlong), ("row_stride", C.c_longlong), ("elem_stride", C.c_longlong)]


# Every function include/pbt.h declares, with its ctypes signature.
_P = C.c_void_p
_D = C.c_void_p  # device pointer to double
SIGNATURES = {
    "pbt_plan_desc_init": (None, [C.POINTER(PlanDesc)]),
    "pbt_plan_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int, C.c_int, C.c_int]),
    "pbt_plan_create_ex": (C.c_int, [C.POINTER(_P), C.POINTER(PlanDesc)]),
    "pbt_plan_destroy": (C.c_int, [_P]),
    "pbt_solve_noncyclic": (C.c_int, [_P, _D, _D, _D, _D, C.c_int, C.c_int, C.c_int, _P]),
    "pbt_solve_noncyclic_profiled": (
        C.c_int,
        [_P, _D, _D, _D, _D, C.c_int, C.c_int, C.c_int, C.POINTER(Timings), _P],
    ),
    "pbt_solve_cyclic": (C.c_int, [_P, _D, _D, _D, _D, C.c_int, C.c_int, C.c_int, _P]),
    "pbt_solve_noncyclic_lines": (C.c_int, [_P, _D, _D, _D, _D, C.POINTER(Lines), _P]),
    "pbt_adjoint_noncyclic": (
        C.c_int,
        [_P, _D, _D, _D, _D, _D, _D, _D, _D, C.c_int, C.c_int, C.c_int, _P],
    ),
    "pbt_solve_noncyclic_noalloc": (C.c_int, [_D, _D, _D, _D, C.c_int, C.c_int, C.c_int, C.c_int, _P]),
    "pbt_plan_status": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "pbt_plan_refine_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "pbt_plan_get_desc": (C.c_int, [_P, C.POINTER(PlanDesc)]),
    "pbt_plan_workspace_bytes": (C.c_size_t, [_P]),
    "pbt_last_error_string": (C.c_char_p, []),
    "pbt_partition_1d": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pbt_version": (C.c_int, []),
}

SYNTH_SIGNATURES = {
    "pbt_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "pbt_synth_uniform": (C.c_double, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
    "pbt_synth_fill": (
        C.c_int,
        [C.c_int, C.c_uint, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_double, _P, _P, _P, _P, _P, C.c_int],
    ),
    "pbt_synth_uneven_shapes": (
        C.c_int,
        [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _P, _P],
    ),
    "pbt_synth_exp2": (C.c_double, [C.c_double]),
    "pbt_synth_fill_batch": (
        C.c_int,
        [C.c_int, C.c_uint, C.c_int, _P, _P, _P, _P, C.c_uint64, C.c_double, _P, _P, _P, _P, C.c_int],
    ),
}

_lib = None
_synth = None


def _bind(path: Path, sigs: dict) -> C.CDLL:
    if not path.exists():
        raise RuntimeError(
            f"{path.name} is not built; run `python -m pascal_btdma_gb300.build` "
            "(or __graft_entry__.build()) first"
        )
    lib = C.CDLL(str(path))
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def lib() -> C.CDLL:
    """The loaded libpbt.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        _lib = _bind(LIB_PATH, SIGNATURES)
    return _lib


def synth_lib() -> C.CDLL:
    global _synth
    if _synth is None:
        _synth = _bind(SYNTH_PATH, SYNTH_SIGNATURES)
    return _synth


def last_error() -> str:
    msg = lib().pbt_last_error_string()
    return msg.decode() if msg else ""


def loaded_paths() -> list[str]:
    """Paths of the native libraries this process has loaded."""
    out = []
    if _lib is not None:
        out.append(os.fspath(LIB_PATH))
    if _synth is not None:
        out.append(os.fspath(SYNTH_PATH))
    return out
