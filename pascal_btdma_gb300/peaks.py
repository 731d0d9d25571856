"""Measure the FP64 and FP32 FMA rates of the current GPU (include/pbt_probe.h).

    python -m pascal_btdma_gb300.peaks
"""
from __future__ import annotations

import ctypes as C
import json


def fma_rates() -> dict:
    from . import _native as N

    f64, f32 = C.c_double(), C.c_double()
    rc = N.lib().pbt_probe_fma_rates(C.byref(f64), C.byref(f32))
    if rc != 0:
        raise RuntimeError(f"pbt_probe_fma_rates failed: {N.last_error() or rc}")
    return {"fp64_fma_per_s": f64.value, "fp32_fma_per_s": f32.value,
            "fp64_tflops": 2 * f64.value / 1e12, "fp32_tflops": 2 * f32.value / 1e12}


if __name__ == "__main__":
    print(json.dumps(fma_rates()))
