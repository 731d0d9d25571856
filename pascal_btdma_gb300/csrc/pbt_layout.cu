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
constexpr int kBatch = 4;  // loads a thread has in flight in k_layout

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
    // Loads go out kBatch at a time before any of them is waited on.
    if (dir == 0) {
        for (int t0 = threadIdx.x; t0 < total; t0 += kBatch * kThreads) {
            double v[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                const int t = t0 + u * kThreads;
                v[u] = t < total ? src[cpu0 + t] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                const int t = t0 + u * kThreads;
                if (t < total) {
                    const int s = t / E, e = t - s * E;
                    tile[e * (kTile + 1) + s] = v[u];
                }
            }
        }
        __syncthreads();
        for (int t = threadIdx.x; t < E * kTile; t += kThreads) {
            const int e = t / kTile, s = t - e * kTile;
            if (s < cnt) dst[gpu0 + s + plane * e] = tile[e * (kTile + 1) + s];
        }
    } else {
        for (int t0 = threadIdx.x; t0 < E * kTile; t0 += kBatch * kThreads) {
            double v[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                const int t = t0 + u * kThreads;
                const int e = t / kTile, s = t - e * kTile;
                v[u] = (t < E * kTile && s < cnt) ? src[gpu0 + s + plane * e] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kBatch; ++u) {
                const int t = t0 + u * kThreads;
                const int e = t / kTile, s = t - e * kTile;
                if (t < E * kTile && s < cnt) tile[e * (kTile + 1) + s] = v[u];
            }
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
// h + l is exact in FP64; back, FF::split_wide keeps 47 bits (these are the
// library's own intermediates: no input window).
// to_f64 = 2 also sets values below the float-float input window (|v| <
// 2^-96) to zero: used on the reduced system's blocks before a float-float
// sub-plan reads them as its matrix, where such entries are negligible next
// to the identity diagonal blocks (A' and C' decay along long segments).
__global__ void k_ff_raw_f64(double* x, size_t n, int to_f64) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (to_f64) {
            const double v = FF::join(FF::lds(x + i));
            const unsigned e = ((unsigned)__double2hiint(v) >> 20) & 0x7ffu;
            x[i] = (to_f64 == 2 && e < kFFExpLo) ? 0.0 : v;
        } else {
            const double v = x[i];
            FF::sts(x + i, FF::split_wide(v));
        }
    }
}

// Lines whose rows are contiguous (row stride 1: a sweep along an array's
// fast index) <-> the reference GPU layout.  One CTA moves a tile of 32 rows
// x 32 systems of one element plane: the lines side is read (or written) along
// the rows, the reference side along the systems, both in 256-byte runs, and
// the tile turns around in shared memory (stride 33).  dir 0: lines (src) ->
// reference (dst); dir 1: reference (src) -> lines (dst).
__global__ void __launch_bounds__(256) k_lines_layout(const double* __restrict__ src, double* __restrict__ dst,
                                                      LineStrides ls, int nsys, int nrow, int dir) {
    __shared__ double tile[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8 threads, 4 tile rows each
    const int r0 = blockIdx.x * 32, e = blockIdx.z;
    const int nsb = (nsys + 31) / 32;
    auto app = [&](int s, int r) {
        return (size_t)(s % ls.lin) * (size_t)ls.in + (size_t)(s / ls.lin) * (size_t)ls.out + (size_t)r +
               (size_t)e * (size_t)ls.elem;
    };
    auto ref = [&](int s, int r) { return (size_t)s + (size_t)nsys * ((size_t)r + (size_t)nrow * e); };
    for (int sb = blockIdx.y; sb < nsb; sb += gridDim.y) {
        const int s0 = sb * 32;
        if (dir == 0) {
#pragma unroll
            for (int j = 0; j < 32; j += 8) {
                const int r = r0 + tx, sy = s0 + ty + j;
                if (r < nrow && sy < nsys) tile[ty + j][tx] = src[app(sy, r)];
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 32; j += 8) {
                const int sx = s0 + tx, r = r0 + ty + j;
                if (r < nrow && sx < nsys) dst[ref(sx, r)] = tile[tx][ty + j];
            }
        } else {
#pragma unroll
            for (int j = 0; j < 32; j += 8) {
                const int sx = s0 + tx, r = r0 + ty + j;
                if (r < nrow && sx < nsys) tile[tx][ty + j] = src[ref(sx, r)];
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < 32; j += 8) {
                const int r = r0 + tx, sy = s0 + ty + j;
                if (r < nrow && sy < nsys) dst[app(sy, r)] = tile[ty + j][tx];
            }
        }
        __syncthreads();  // the tile is reused by the next system block
    }
}

}  // namespace

cudaError_t launch_lines_layout(const double* src, double* dst, const LineStrides& ls, int E, int nsys, int nrow,
                                int dir, cudaStream_t s) {
    if (E <= 0 || nsys <= 0 || nrow <= 0) return cudaSuccess;
    const int nsb = (nsys + 31) / 32;
    const dim3 grid((unsigned)((nrow + 31) / 32), (unsigned)(nsb < 65535 ? nsb : 65535), (unsigned)E);
    k_lines_layout<<<grid, dim3(32, 8), 0, s>>>(src, dst, ls, nsys, nrow, dir);
    return cudaGetLastError();
}

// The reduced solution of a float-float plan after its FP64 sub-solve, back
// to raw pairs (rd[sys + nsys*(r + rows*i)]).  A CTA is 32 systems x 32
// threads along their values, so that the line's range check (range_bits: a
// non-finite value, or the whole reduced solution below the float-float
// limit) sees all of a system's values after one shared-memory reduction.
__global__ void __launch_bounds__(1024) k_reduced_to_ff(double* rd, int nsys, int rows, int m,
                                                       unsigned long long* status) {
    __shared__ unsigned red[32][33];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int sys = blockIdx.x * 32 + tx;
    unsigned amax = 0;
    if (sys < nsys) {
        const size_t n = (size_t)rows * m;
        for (size_t k = ty; k < n; k += 32) {
            double* p = rd + sys + (size_t)nsys * k;
            const FF::T v = FF::split_wide(*p);
            amax = max(amax, FF::mag(v));
            FF::sts(p, v);
        }
    }
    red[ty][tx] = amax;
    __syncthreads();
    if (ty == 0 && sys < nsys) {
        for (int k = 1; k < 32; ++k) amax = max(amax, red[k][tx]);
        report_status(status, range_bits<FF>(amax, true));
    }
}

cudaError_t launch_reduced_to_ff(double* rd, int nsys, int rows, int m, unsigned long long* status, cudaStream_t s) {
    k_reduced_to_ff<<<(unsigned)((nsys + 31) / 32), dim3(32, 32), 0, s>>>(rd, nsys, rows, m, status);
    return cudaGetLastError();
}

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
