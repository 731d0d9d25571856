"""Build the native libraries of the package, in tree.

    python -m pascal_btdma_gb300.build        # or pascal_btdma_gb300.build.build()

Outputs (git-ignored, rebuilt on the GPU host because it is a different CPU
architecture):
    pascal_btdma_gb300/libpbt.so        CUDA kernels + C ABI (include/pbt.h), sm_103a
    pascal_btdma_gb300/libpbt_synth.so  synthetic workload generator (include/pbt_synth.h)
    pascal_btdma_gb300/libpbt_probe.so  FMA-rate probe of the benchmark (probe/fma_probe.cu;
                                        measurement tooling, not part of libpbt.so)

The FP64 kernel file is compiled once per block size (-DPBT_M=1..10) so the
unrolled variants compile in parallel; objects are cached under _build/ and
rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libpbt.so"
SYNTH = PKG / "libpbt_synth.so"
PROBE = PKG / "libpbt_probe.so"
PROBE_SRC = PKG / "probe" / "fma_probe.cu"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"] + ARCH
MAX_BLOCK = 10

# Families of kernels instantiated per block size: (source, object stem).
PER_M_SOURCES = [("pbt_inst.cu", "F64"), ("pbt_inst.cu", "FF"), ("pbt_inst.cu", "F32")]
HOST_SOURCES = ["pbt_api.cpp", "pbt_noalloc.cu", "pbt_batch.cpp", "pbt_batch_pack.cu", "pbt_layout.cu",
                "pbt_shared.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpbt.so")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [INCLUDE / "pbt.h"])


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build command failed ({res.returncode}):\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build_probe() -> Path:
    """Compile libpbt_probe.so (the benchmark's FMA-rate probe) if its source changed."""
    if _stale(PROBE, [PROBE_SRC]):
        _run([_nvcc(), *NVCC_FLAGS, "-shared", "-o", str(PROBE), str(PROBE_SRC), "-cudart", "static"])
    return PROBE


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile libpbt.so, libpbt_synth.so and libpbt_probe.so if any input changed."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    hdrs = _headers()
    tasks: list[tuple[Path, list[str]]] = []
    objs: list[Path] = []
    for src, stem in PER_M_SOURCES:
        for m in range(1, MAX_BLOCK + 1):
            obj = BUILD / f"{stem.lower()}_m{m}.o"
            objs.append(obj)
            if _stale(obj, [CSRC / src] + hdrs):
                extra = {"F64": ["-DPBT_NUM_IS_F64"], "FF": ["-DPBT_NUM_IS_FF"]}.get(stem, [])
                tasks.append((obj, [nvcc, *NVCC_FLAGS, f"-DPBT_M={m}", f"-DPBT_NUM=pbt::{stem}", *extra, "-c",
                                    str(CSRC / src), "-o", str(obj)]))
    for src in HOST_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        if _stale(obj, [CSRC / src] + hdrs + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))):
            tasks.append((obj, [nvcc, *NVCC_FLAGS, "-x", "cu", "-c", str(CSRC / src), "-o", str(obj)]))
    jobs = jobs or max(2, os.cpu_count() or 2)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = {ex.submit(_run, cmd): obj for obj, cmd in tasks}
        futs[ex.submit(build_probe)] = PROBE
        for f in cf.as_completed(futs):
            f.result()
            if verbose:
                print("built", futs[f].name, flush=True)
    if tasks or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-cudart", "static"])
    synth_src = CSRC / "pbt_synth.c"
    if _stale(SYNTH, [synth_src, INCLUDE / "pbt_synth.h"]):
        cc = shutil.which("gcc") or "cc"
        _run([cc, "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", str(synth_src), "-o", str(SYNTH), "-lm"])
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    print(LIB)
    sys.exit(0)
