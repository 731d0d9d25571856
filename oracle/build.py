"""Build the CPU oracle (test infrastructure only): oracle/liboracle.so.

    python oracle/build.py

The oracle is plain C (pbt_oracle.c, a restatement of the reference CPU path
Fortran_Original/src/mod_btdma_cpu.f90), compiled with -ffp-contract=off so
x86-64 and AArch64 hosts give identical results.

The reference's own CPU path cannot be compiled here: it is Fortran 90 that
needs an MPI Fortran compiler (mpifort) and a BLAS/LAPACK library
(Fortran_Original/Makefile.inc:27-29), and neither a Fortran compiler nor MPI
is installed.  Its CUDA C++ port (CUDA_CXX_Port/) needs <mpi.h> and an MPI
library as well.  So oracle/_ref/ stays empty and the restatement is the CPU
baseline ("kind": "port").
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "pbt_oracle.c"
HDR = HERE / "pbt_oracle.h"
LIB = HERE / "liboracle.so"


def build() -> Path:
    if not LIB.exists() or max(SRC.stat().st_mtime, HDR.stat().st_mtime) > LIB.stat().st_mtime:
        cc = shutil.which("gcc") or "cc"
        cmd = [cc, "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread", str(SRC), "-o", str(LIB), "-lm"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{res.stderr}")
    return LIB


if __name__ == "__main__":
    print(build())
