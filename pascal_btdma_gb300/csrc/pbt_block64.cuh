// pbt_block64.cuh -- per-thread m x m FP64 block arithmetic held in registers.
//
// Everything is templated on the block size M so that every loop unrolls and
// every block lives in registers (up to M = 5 without spills; larger M spill
// to thread-local memory).  The FP64 pipe is the bottleneck of this path on
// GB300, so the helpers keep FP64 instructions to the FMAs the mathematics
// needs: pivot search and |x| tests are integer compares on the bit pattern,
// row swaps are predicated selects, and each pivot's reciprocal is formed
// once and reused by the multipliers and the back substitution.
//
// The dense kernels restate the block operations of the reference GPU path
// (gesv / gesv_mrhs2 / gesv_mrhs3 / gemm / gemv,
// Fortran_Original/src/mod_btdma_gpu_v2.f90:921-1123), but with partial
// pivoting as in the reference CPU path's LAPACK dgesv
// (Fortran_Original/src/mod_btdma_cpu.f90:339,357,381,421).
#pragma once

#include <cstddef>
#include <cstdint>

namespace pbt {

// Predicated select kept opaque to the compiler: written as plain C++, the
// select-based row swaps below are turned into a dynamically indexed array,
// which moves the whole block to thread-local memory.
__device__ __forceinline__ double sel(unsigned s, double x, double y) {
    double r;
    asm("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %3, 0;\n\tselp.f64 %0, %1, %2, p;\n\t}"
        : "=d"(r)
        : "d"(x), "d"(y), "r"(s));
    return r;
}

// Hides a value from the optimiser.  Called once per row iteration on the
// plane stride, it stops the compiler from hoisting the m*m 64-bit element
// addresses of a block out of the row loop, where they would hold ~2*m*m
// registers for the whole kernel and force the blocks themselves to spill.
__device__ __forceinline__ size_t opaque(size_t v) {
    asm volatile("" : "+l"(v));
    return v;
}

// Compiler barrier for memory operations: loads after it are not hoisted above
// it.  Placed between forming a row's right-hand sides and loading its C
// block, it caps the number of live blocks (and so the register pressure).
__device__ __forceinline__ void mem_fence_compiler() { asm volatile("" ::: "memory"); }

// |x| as an unsigned integer: orders like |x| for every non-NaN double.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return static_cast<unsigned long long>(__double_as_longlong(x)) & 0x7fffffffffffffffull;
}

// Gaussian elimination with partial pivoting on the augmented system
// [a | b] (a: M x M, b: M x NR right-hand sides), leaving the solution
// a^{-1} b in b.  Pivot = first row of maximal |a(i,k)| (LAPACK idamax
// rule); the multipliers are a(i,k) * (1/a(k,k)) as in dgetf2.  A zero pivot
// sets `bad` and the arithmetic goes on (Inf/NaN), like the reference.
template <int M, int NR>
__device__ __forceinline__ void gesv_pp(double (&a)[M][M], double (&b)[M][NR], bool& bad) {
    double rinv[M];
#pragma unroll
    for (int k = 0; k < M; ++k) {
        if (k + 1 < M) {
            int p = k;
            unsigned long long best = abs_bits(a[k][k]);
#pragma unroll
            for (int i = k + 1; i < M; ++i) {
                const unsigned long long v = abs_bits(a[i][k]);
                const bool gt = v > best;
                best = gt ? v : best;
                p = gt ? i : p;
            }
#pragma unroll
            for (int i = k + 1; i < M; ++i) {
                const unsigned s = (p == i);
#pragma unroll
                for (int c = k; c < M; ++c) {
                    const double t = a[k][c];
                    a[k][c] = sel(s, a[i][c], t);
                    a[i][c] = sel(s, t, a[i][c]);
                }
#pragma unroll
                for (int c = 0; c < NR; ++c) {
                    const double t = b[k][c];
                    b[k][c] = sel(s, b[i][c], t);
                    b[i][c] = sel(s, t, b[i][c]);
                }
            }
        }
        bad |= (abs_bits(a[k][k]) == 0ull);
        const double r = __drcp_rn(a[k][k]);
        rinv[k] = r;
#pragma unroll
        for (int i = k + 1; i < M; ++i) {
            const double l = a[i][k] * r;
#pragma unroll
            for (int c = k + 1; c < M; ++c) a[i][c] = fma(-l, a[k][c], a[i][c]);
#pragma unroll
            for (int c = 0; c < NR; ++c) b[i][c] = fma(-l, b[k][c], b[i][c]);
        }
    }
#pragma unroll
    for (int k = M - 1; k >= 0; --k) {
#pragma unroll
        for (int c = 0; c < NR; ++c) {
            const double x = b[k][c] * rinv[k];
            b[k][c] = x;
#pragma unroll
            for (int i = 0; i < k; ++i) b[i][c] = fma(-a[i][k], x, b[i][c]);
        }
    }
}

// ---------------------------------------------------------------------------
// Loads and stores in the reference GPU layout: element (i, j) of the block of
// (sys, row) sits at base[(i + M*j) * plane], base = X + sys + nsys*row,
// plane = nsys * nrow.  Consecutive threads own consecutive systems, so each
// warp-wide access is one contiguous 256-byte segment.
// ---------------------------------------------------------------------------
template <int M>
__device__ __forceinline__ void ld_blk(double (&x)[M][M], const double* __restrict__ base, size_t plane) {
#pragma unroll
    for (int j = 0; j < M; ++j)
#pragma unroll
        for (int i = 0; i < M; ++i) x[i][j] = __ldg(base + (size_t)(i + M * j) * plane);
}

// Same, from memory this kernel also writes (no read-only cache path).
template <int M>
__device__ __forceinline__ void ld_blk_rw(double (&x)[M][M], const double* base, size_t plane) {
#pragma unroll
    for (int j = 0; j < M; ++j)
#pragma unroll
        for (int i = 0; i < M; ++i) x[i][j] = base[(size_t)(i + M * j) * plane];
}

template <int M>
__device__ __forceinline__ void st_blk(double* base, size_t plane, const double (&x)[M][M]) {
#pragma unroll
    for (int j = 0; j < M; ++j)
#pragma unroll
        for (int i = 0; i < M; ++i) base[(size_t)(i + M * j) * plane] = x[i][j];
}

template <int M>
__device__ __forceinline__ void ld_vec(double (&x)[M], const double* base, size_t plane) {
#pragma unroll
    for (int i = 0; i < M; ++i) x[i] = base[(size_t)i * plane];
}

template <int M>
__device__ __forceinline__ void st_vec(double* base, size_t plane, const double (&x)[M]) {
#pragma unroll
    for (int i = 0; i < M; ++i) base[(size_t)i * plane] = x[i];
}

}  // namespace pbt
