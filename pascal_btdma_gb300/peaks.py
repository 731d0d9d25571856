"""Measure the FP64, FP32 and packed FP32x2 FMA rates of the current GPU with the
benchmark's probe library (libpbt_probe.so, built from probe/fma_probe.cu).

    python -m pascal_btdma_gb300.peaks
"""
from __future__ import annotations

import ctypes as C
import json

_probe = None


def probe_lib() -> C.CDLL:
    global _probe
    if _probe is None:
        from . import build as B

        if not B.PROBE.exists():
            raise RuntimeError(f"{B.PROBE.name} is not built; run `python -m pascal_btdma_gb300.build` first")
        _probe = C.CDLL(str(B.PROBE))
        _probe.pbt_probe_fma_rates.restype = C.c_int
        _probe.pbt_probe_fma_rates.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _probe.pbt_probe_fma2_rate.restype = C.c_int
        _probe.pbt_probe_fma2_rate.argtypes = [C.POINTER(C.c_double)]
    return _probe


def fma_rates() -> dict:
    f64, f32 = C.c_double(), C.c_double()
    rc = probe_lib().pbt_probe_fma_rates(C.byref(f64), C.byref(f32))
    if rc != 0:
        raise RuntimeError(f"pbt_probe_fma_rates failed (CUDA error, code {rc})")
    f2 = C.c_double()
    if probe_lib().pbt_probe_fma2_rate(C.byref(f2)) != 0:
        raise RuntimeError("pbt_probe_fma2_rate failed (CUDA error)")
    return {"fp64_fma_per_s": f64.value, "fp32_fma_per_s": f32.value, "fp32x2_fma_per_s": f2.value,
            "fp64_tflops": 2 * f64.value / 1e12, "fp32_tflops": 2 * f32.value / 1e12}


if __name__ == "__main__":
    print(json.dumps(fma_rates()))
