// pbt_layout.cu -- conversion between the reference CPU layout and the
// reference GPU layout, for plans created with PBT_FLAG_CPU_LAYOUT.
//
//   CPU layout (Fortran_Original/src/mod_btdma_cpu.f90:18-19): a(m, m, nsys, n),
//     d(m, nsys, n): element e of (sys, row) at e + E*(sys + nsys*row),
//     E = m*m for the blocks (e = i + m*j) and E = m for d (e = i).
//   GPU layout (CUDA_CXX_Port/include/pascal_btdma_cuda.hpp:46-65):
//     element e of (sys, row) at sys + nsys*(row + n*e).
//
// One CTA moves one tile of 32 systems of one row: the tile is one contiguous
// run of 32*E doubles in the CPU layout and E runs of 32 doubles in the GPU
// layout, so both sides are read and written in full 256-byte segments; the
// tile is turned around in shared memory (stride 33 against bank conflicts).
#include <cuda_runtime.h>

#include "pbt_internal.h"
#include "pbt_num.cuh"

namespace pbt {

namespace {

constexpr int kTile = 32;
constexpr int kThreads = 256;

// dir 0: CPU layout (src) -> GPU layout (dst); dir 1: GPU -> CPU.
__global__ void __launch_bounds__(kThreads) k_layout(const double* __restrict__ src, double* __restrict__ dst,
                                                      int E, int nsys, int nrow, int dir) {
    extern __shared__ double tile[];  // [E][33]
    const int s0 = blockIdx.x * kTile;
    const int cnt = min(kTile, nsys - s0);
    const size_t plane = (size_t)nsys * nrow;
    for (int row = blockIdx.y; row < nrow; row += gridDim.y) {
    const size_t cpu0 = (size_t)E * ((size_t)s0 + (size_t)nsys * row);  // first element of the tile, CPU layout
    const size_t gpu0 = (size_t)s0 + (size_t)nsys * row;                // (sys s0, row, e = 0), GPU layout
    const int total = cnt * E;
    if (dir == 0) {
        for (int t = threadIdx.x; t < total; t += kThreads) {
            const int s = t / E, e = t - s * E;
            tile[e * (kTile + 1) + s] = src[cpu0 + t];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < E * kTile; t += kThreads) {
            const int e = t / kTile, s = t - e * kTile;
            if (s < cnt) dst[gpu0 + s + plane * e] = tile[e * (kTile + 1) + s];
        }
    } else {
        for (int t = threadIdx.x; t < E * kTile; t += kThreads) {
            const int e = t / kTile, s = t - e * kTile;
            if (s < cnt) tile[e * (kTile + 1) + s] = src[gpu0 + s + plane * e];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < total; t += kThreads) {
            const int s = t / E, e = t - s * E;
            dst[cpu0 + t] = tile[e * (kTile + 1) + s];
        }
    }
    __syncthreads();  // the tile is reused by the next row
    }
}

// In place: raw float-float pairs (8-byte slots, as the kernels keep their
// intermediates) <-> FP64 values.  The pair (h, l) has |l| <= ulp(h)/2, so
// h + l is exact in FP64; back, FF::split keeps 47 bits.
__global__ void k_ff_raw_f64(double* x, size_t n, int to_f64) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (to_f64) {
            x[i] = FF::join(FF::lds(x + i));
        } else {
            const double v = x[i];
            FF::sts(x + i, FF::split(v));
        }
    }
}

}  // namespace

cudaError_t launch_ff_raw_f64(double* x, size_t n, int to_f64, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const size_t blocks = (n + kThreads - 1) / kThreads;
    k_ff_raw_f64<<<(unsigned)(blocks < 4096 ? blocks : 4096), kThreads, 0, s>>>(x, n, to_f64);
    return cudaGetLastError();
}

cudaError_t launch_layout(const double* src, double* dst, int E, int nsys, int nrow, int dir, cudaStream_t s) {
    if (E <= 0 || nsys <= 0 || nrow <= 0) return cudaSuccess;
    const dim3 grid((unsigned)((nsys + kTile - 1) / kTile), (unsigned)(nrow < 65535 ? nrow : 65535));
    const size_t smem = (size_t)E * (kTile + 1) * sizeof(double);  // <= 26.4 KB for m <= 10
    k_layout<<<grid, kThreads, smem, s>>>(src, dst, E, nsys, nrow, dir);
    return cudaGetLastError();
}

}  // namespace pbt
