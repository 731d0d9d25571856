"""The C++ layer (include/pbt.hpp) over the C ABI: compiles against the
header, links libpbt.so, and maps status codes to the reference C++ port's
exception types (CUDA_CXX_Port/include/pascal_btdma_cuda.hpp:20-22 and
pascal_btdma_cuda.cu:862-870, 956-967).  CPU only: no call reaches a kernel."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

PROGRAM = r"""
#include "pbt.hpp"
#include <cstdio>
#include <utility>

template <class E, class F>
static void expect(const char* name, F f) {
    try {
        f();
        std::printf("%s: no exception\n", name);
    } catch (const E&) {
        std::printf("%s: ok\n", name);
    } catch (const std::exception& e) {
        std::printf("%s: wrong exception %s\n", name, e.what());
    }
}

int main() {
    expect<std::invalid_argument>("m11", [] { pbt::BtdmaGpuPlan p(11, 4, 4, 1); });
    expect<std::invalid_argument>("nseg0", [] { pbt::BtdmaGpuPlan p(3, 4, 8, 0); });
    expect<std::invalid_argument>("two_row_segments", [] { pbt::BtdmaGpuPlan p(3, 4, 8, 4); });
    expect<std::runtime_error>("uncreated", [] {
        pbt::BtdmaGpuPlan p;
        pbt::solve_noncyclic(p, nullptr, nullptr, nullptr, nullptr, 3, 4, 8);
    });
    expect<std::logic_error>("unknown_precision", [] {
        pbt_plan_desc d;
        pbt_plan_desc_init(&d);
        d.m = 3; d.nsys = 4; d.nrow = 8; d.precision = 9;
        pbt::BtdmaGpuPlan p(d);
    });
    pbt::BtdmaGpuPlan a;
    pbt::BtdmaGpuPlan b(std::move(a));
    b = pbt::BtdmaGpuPlan();
    std::printf("moves: ok %d\n", (int)b.created());
    auto r = pbt::partition_1d(0, 9, 3, 0);
    std::printf("partition: %d %d\n", r.first, r.second);
    return 0;
}
"""


def test_cpp_layer_compiles_and_maps_errors(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    from pascal_btdma_gb300 import _native as N

    lib = Path(N.LIB_PATH)
    src = tmp_path / "probe.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "probe"
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(src), f"-L{lib.parent}",
                    "-lpbt", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    assert out == ["m11: ok", "nseg0: ok", "two_row_segments: ok", "uncreated: ok", "unknown_precision: ok",
                   "moves: ok 0", "partition: 0 3"], out
