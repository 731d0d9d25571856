// pbt_kernels.cuh -- the solver kernels, written once over an arithmetic
// `Num` (pbt_num.cuh: F64 = plain FP64, FF = float-float on the FP32 pipes)
// and a compile-time block size M.
//
// One thread owns one (system, segment) pair; consecutive threads own
// consecutive systems, so every block-element access of a warp is one
// contiguous 256-byte segment of the reference GPU layout
// X[sys + nsys*(row + nrow*(i + M*j))].  All m x m arithmetic is unrolled.
//
//   k_thomas        single-segment fast path: plain block Thomas on the whole
//                   line (the reduced-solve recurrence of btdma_many_gpu_v2,
//                   Fortran_Original/src/mod_btdma_gpu_v2.f90:241-350, applied
//                   to the original rows).  Same x as the two-stage method
//                   with one segment, at ~40% of its flops.
//   k_modi          stage 1 of the two-stage method, one segment:
//                   btdma_many_modi_gpu_v2 (mod_btdma_gpu_v2.f90:618-866).  The
//                   two reduced rows go straight into the reduced system's
//                   layout, which replaces the pack + MPI_ALLTOALLV + unpack
//                   of :1309-1342.
//   k_reduced       stage 2: block Thomas on the 2P-row reduced system (B = I),
//                   btdma_many_gpu_v2 (:241-350).
//   k_reduced_cyclic stage 2 of the cyclic solve: btdma_many_cycl
//                   (Fortran_Original/src/mod_btdma_cpu.f90:80-183).
//   k_update        stage 3: x_q = d'_q - A'_q x_first - C'_q x_last
//                   (btdma_many_update_gpu_v2, mod_btdma_gpu_v2.f90:868-919),
//                   reading the reduced solution in place (replaces the
//                   backward MPI_ALLTOALLV of :1344-1374).
//
// Storage rules: inputs are FP64 and converted on load (Num::in); the
// solution is converted on store (Num::out).  Intermediates -- the factors in
// the plan's workspace, d'/y parked in D, the reduced system -- are raw 8-byte
// Num values (Num::lds / Num::sts); factors written in place into the
// caller's A and C are converted to FP64 so those arrays stay valid doubles.
#pragma once

#include <math_constants.h>

#include <type_traits>

#include "pbt_util.cuh"
#include "pbt_internal.h"
#include "pbt_num.cuh"

namespace pbt {

// Loop unrolling policy (PBT_UNROLL precedes every m x m loop): fully
// unrolled by default, so the blocks live in registers.  A translation unit
// instantiating only M = 7..10 defines PBT_UNROLL as "unroll 1" first: those
// blocks do not fit in registers anyway, and full unrolling would only
// multiply compile time (minutes per variant), so their loops stay rolled and
// the blocks live in local memory.
#ifndef PBT_UNROLL
#define PBT_UNROLL _Pragma("unroll")
#endif

__device__ __forceinline__ void seg_rows(int n, int p, int s, int& first, int& last) {
    const int base = n / p, rem = n % p;
    first = s * base + (s < rem ? s : rem);
    last = first + base + (s < rem ? 1 : 0) - 1;
}

// ---------------------------------------------------------------------------
// Gaussian elimination with partial pivoting on [a | b] (M x M, M x NR);
// the solution a^{-1} b is left in b.  This is the block solve of the
// reference GPU path (gesv / gesv_mrhs2 / gesv_mrhs3,
// Fortran_Original/src/mod_btdma_gpu_v2.f90:921-1123, which does not pivot)
// with the partial pivoting of the reference CPU path's LAPACK dgesv
// (Fortran_Original/src/mod_btdma_cpu.f90:339,357,381,421).  Pivot = first row of maximal |a(i,k)|
// (LAPACK idamax rule; for FF the high part decides); multipliers are
// a(i,k) * (1/a(k,k)) as in dgetf2.  Entries are accumulators, normalised
// only when their row becomes the pivot row.  A zero pivot sets `bad`; the
// arithmetic goes on (Inf/NaN), like the reference.
// ---------------------------------------------------------------------------
template <class Num, int M, int NR>
__device__ __forceinline__ void gesv(typename Num::Acc (&a)[M][M], typename Num::Acc (&b)[M][NR], unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    T rinv[M];
PBT_UNROLL
    for (int k = 0; k < M; ++k) {
        if (k + 1 < M) {
            int p = k;
            auto best = Num::akey(a[k][k]);
PBT_UNROLL
            for (int i = k + 1; i < M; ++i) {
                const auto v = Num::akey(a[i][k]);
                const bool gt = v > best;
                best = gt ? v : best;
                p = gt ? i : p;
            }
            // The swaps cost ~10x the rest of a pivot step in instructions;
            // skip them when no thread of the warp needs one (the common case
            // for the diagonally dominant blocks of implicit PDE schemes).
            if (__any_sync(__activemask(), p != k))
PBT_UNROLL
            for (int i = k + 1; i < M; ++i) {
                const unsigned s = (p == i);
PBT_UNROLL
                for (int c = k; c < M; ++c) {
                    const Acc t = a[k][c];
                    a[k][c] = Num::asel(s, a[i][c], t);
                    a[i][c] = Num::asel(s, t, a[i][c]);
                }
PBT_UNROLL
                for (int c = 0; c < NR; ++c) {
                    const Acc t = b[k][c];
                    b[k][c] = Num::asel(s, b[i][c], t);
                    b[i][c] = Num::asel(s, t, b[i][c]);
                }
            }
        }
        const T piv = Num::fin(a[k][k]);
        bad |= Num::is_zero(piv);
        const T r = Num::rcp(piv);
        rinv[k] = r;
        T uk[M], bk[NR];
PBT_UNROLL
        for (int c = k + 1; c < M; ++c) {
            uk[c] = Num::fin(a[k][c]);
            a[k][c] = Num::acc(uk[c]);
        }
PBT_UNROLL
        for (int c = 0; c < NR; ++c) {
            bk[c] = Num::fin(b[k][c]);
            b[k][c] = Num::acc(bk[c]);
        }
PBT_UNROLL
        for (int i = k + 1; i < M; ++i) {
            const T l = Num::mul(Num::fin(a[i][k]), r);
PBT_UNROLL
            for (int c = k + 1; c < M; ++c) Num::msub(a[i][c], l, uk[c]);
PBT_UNROLL
            for (int c = 0; c < NR; ++c) Num::msub(b[i][c], l, bk[c]);
        }
    }
PBT_UNROLL
    for (int k = M - 1; k >= 0; --k) {
PBT_UNROLL
        for (int c = 0; c < NR; ++c) {
            const T x = Num::mul(Num::fin(b[k][c]), rinv[k]);
            b[k][c] = Num::acc(x);
PBT_UNROLL
            for (int i = 0; i < k; ++i) Num::msub(b[i][c], Num::fin(a[i][k]), x);
        }
    }
}

// ---------------------------------------------------------------------------
// The same elimination split in two.  lu_factor pivots and eliminates the
// matrix alone and records what a right-hand side needs; lu_solve replays
// that on one right-hand-side column.  Solving column by column holds the
// factors plus one column in registers instead of the factors plus every
// column, and each column sees exactly the operations of gesv<Num, M, NR>,
// so the results are identical.  The multipliers stay where their row was
// at their step (later swaps do not move them), which is what the in-order
// replay in lu_solve needs.
// ---------------------------------------------------------------------------
template <class Num, int M>
struct LU {
    static_assert(M <= 16, "LU::piv packs the M - 1 pivot rows in 4 bits each");
    // Pivot rows of blocks up to 8 x 8 fit 32 bits (the staged kernels store
    // them as one float); larger blocks take 64.
    using Piv = typename std::conditional<(M <= 8), unsigned, unsigned long long>::type;
    // f[k][c] (c > k): row k of U, normalised; f[i][k] (i > k): multiplier
    // l_ik of step k; f[k][k]: 1 / U_kk.
    typename Num::T f[M][M];
    Piv piv = 0;         // 4 bits per step k: the row swapped with row k
    unsigned swaps = 0;  // bit k: some thread of the warp swapped at step k
};

template <class Num, int M>
__device__ __forceinline__ void lu_factor(typename Num::Acc (&a)[M][M], LU<Num, M>& lu, unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
PBT_UNROLL
    for (int k = 0; k < M; ++k) {
        if (k + 1 < M) {
            int p = k;
            auto best = Num::akey(a[k][k]);
PBT_UNROLL
            for (int i = k + 1; i < M; ++i) {
                const auto v = Num::akey(a[i][k]);
                const bool gt = v > best;
                best = gt ? v : best;
                p = gt ? i : p;
            }
            if (__any_sync(__activemask(), p != k)) {
                lu.swaps |= 1u << k;
PBT_UNROLL
                for (int i = k + 1; i < M; ++i) {
                    const unsigned s = (p == i);
PBT_UNROLL
                    for (int c = k; c < M; ++c) {
                        const Acc t = a[k][c];
                        a[k][c] = Num::asel(s, a[i][c], t);
                        a[i][c] = Num::asel(s, t, a[i][c]);
                    }
                }
            }
            lu.piv |= static_cast<typename LU<Num, M>::Piv>(p) << (4 * k);
        }
        const T pv = Num::fin(a[k][k]);
        bad |= Num::is_zero(pv);
        const T r = Num::rcp(pv);
        lu.f[k][k] = r;
        T uk[M];
PBT_UNROLL
        for (int c = k + 1; c < M; ++c) {
            uk[c] = Num::fin(a[k][c]);
            lu.f[k][c] = uk[c];
        }
PBT_UNROLL
        for (int i = k + 1; i < M; ++i) {
            const T l = Num::mul(Num::fin(a[i][k]), r);
            lu.f[i][k] = l;
PBT_UNROLL
            for (int c = k + 1; c < M; ++c) Num::msub(a[i][c], l, uk[c]);
        }
    }
}

// x = a^{-1} b for one column b (consumed) with the factors of lu_factor.
template <class Num, int M>
__device__ __forceinline__ void lu_solve(const LU<Num, M>& lu, typename Num::Acc (&b)[M], typename Num::T (&x)[M]) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
PBT_UNROLL
    for (int k = 0; k < M; ++k) {
        if (k + 1 < M && ((lu.swaps >> k) & 1u)) {
            const unsigned p = static_cast<unsigned>((lu.piv >> (4 * k)) & 15u);
PBT_UNROLL
            for (int i = k + 1; i < M; ++i) {
                const unsigned s = (p == static_cast<unsigned>(i));
                const Acc t = b[k];
                b[k] = Num::asel(s, b[i], t);
                b[i] = Num::asel(s, t, b[i]);
            }
        }
        const T bk = Num::fin(b[k]);
        b[k] = Num::acc(bk);
PBT_UNROLL
        for (int i = k + 1; i < M; ++i) Num::msub(b[i], lu.f[i][k], bk);
    }
PBT_UNROLL
    for (int k = M - 1; k >= 0; --k) {
        const T xk = Num::mul(Num::fin(b[k]), lu.f[k][k]);
        x[k] = xk;
PBT_UNROLL
        for (int i = 0; i < k; ++i) Num::msub(b[i], lu.f[i][k], xk);
    }
}

// ---------------------------------------------------------------------------
// Loads and stores of one block / vector at `base` (= X + sys + nsys*row).
// ---------------------------------------------------------------------------
template <class Num, int M>
__device__ __forceinline__ void in_blk(typename Num::T (&x)[M][M], const double* base, size_t plane) {
PBT_UNROLL
    for (int j = 0; j < M; ++j)
PBT_UNROLL
        for (int i = 0; i < M; ++i) x[i][j] = Num::in(base + (size_t)(i + M * j) * plane);
}
template <class Num, int M>
__device__ __forceinline__ void in_blk_ro(typename Num::T (&x)[M][M], const double* base, size_t plane) {
PBT_UNROLL
    for (int j = 0; j < M; ++j)
PBT_UNROLL
        for (int i = 0; i < M; ++i) x[i][j] = Num::in_ro(base + (size_t)(i + M * j) * plane);
}
template <class Num, int M>
__device__ __forceinline__ void ld_raw_blk(typename Num::T (&x)[M][M], const double* base, size_t plane) {
PBT_UNROLL
    for (int j = 0; j < M; ++j)
PBT_UNROLL
        for (int i = 0; i < M; ++i) x[i][j] = Num::lds(base + (size_t)(i + M * j) * plane);
}
template <class Num, int M>
__device__ __forceinline__ void st_raw_blk(double* base, size_t plane, const typename Num::T (&x)[M][M]) {
PBT_UNROLL
    for (int j = 0; j < M; ++j)
PBT_UNROLL
        for (int i = 0; i < M; ++i) Num::sts(base + (size_t)(i + M * j) * plane, x[i][j]);
}
template <class Num, int M>
__device__ __forceinline__ void ld_raw_vec(typename Num::T (&x)[M], const double* base, size_t plane) {
PBT_UNROLL
    for (int i = 0; i < M; ++i) x[i] = Num::lds(base + (size_t)i * plane);
}
template <class Num, int M>
__device__ __forceinline__ void st_raw_vec(double* base, size_t plane, const typename Num::T (&x)[M]) {
PBT_UNROLL
    for (int i = 0; i < M; ++i) Num::sts(base + (size_t)i * plane, x[i]);
}
// Solution values: converted to FP64 on store, their largest magnitude
// (Num::mag, an ordered integer with Inf/NaN above every finite value)
// collected in `amax` for range_bits.
template <class Num, int M>
__device__ __forceinline__ void out_vec(double* base, size_t plane, const typename Num::T (&x)[M], unsigned& amax) {
PBT_UNROLL
    for (int i = 0; i < M; ++i) {
        Num::out(base + (size_t)i * plane, x[i]);
        amax = max(amax, Num::mag(x[i]));
    }
}

// Factor storage: raw in the plan's workspace, FP64 when written in place.
template <class Num, int M>
__device__ __forceinline__ void st_fac_blk(double* base, size_t plane, const typename Num::T (&x)[M][M], bool raw) {
    if (raw || !Num::kConv) {
        st_raw_blk<Num, M>(base, plane, x);
    } else {
PBT_UNROLL
        for (int j = 0; j < M; ++j)
PBT_UNROLL
            for (int i = 0; i < M; ++i) Num::out(base + (size_t)(i + M * j) * plane, x[i][j]);
    }
}
// One factor value.  In place, factors are FP64 values of the library's own
// intermediates, so they convert without the input window (Num::in_rhs): A'
// decays along a segment, C' = R^{-1} C can be far smaller than C, and
// neither is out of the solve's range when it falls below 2^-96.
template <class Num>
__device__ __forceinline__ typename Num::T ld_fac(const double* p, bool raw) {
    return (raw || !Num::kConv) ? Num::lds(p) : Num::in_rhs(p);
}
template <class Num>
__device__ __forceinline__ void st_fac(double* p, typename Num::T v, bool raw) {
    if (raw || !Num::kConv)
        Num::sts(p, v);
    else
        Num::out(p, v);
}
template <class Num, int M>
__device__ __forceinline__ void ld_fac_blk(typename Num::T (&x)[M][M], const double* base, size_t plane, bool raw) {
    if (raw || !Num::kConv) {
        ld_raw_blk<Num, M>(x, base, plane);
    } else {
PBT_UNROLL
        for (int j = 0; j < M; ++j)
PBT_UNROLL
            for (int i = 0; i < M; ++i) x[i][j] = Num::in_rhs(base + (size_t)(i + M * j) * plane);
    }
}

template <class Num, int M>
__device__ __forceinline__ void to_acc(typename Num::Acc (&d)[M][M], const typename Num::T (&s)[M][M]) {
PBT_UNROLL
    for (int i = 0; i < M; ++i)
PBT_UNROLL
        for (int j = 0; j < M; ++j) d[i][j] = Num::acc(s[i][j]);
}

// ---------------------------------------------------------------------------
// Single-segment block Thomas.  Forward: R_q = B_q - A_q C'_{q-1},
// [C'_q | y_q] = R_q^{-1} [C_q | d_q - A_q y_{q-1}]; C' goes to cw, y to D.
// Backward: x_q = y_q - C'_q x_{q+1}.
// ---------------------------------------------------------------------------
// Launch shape of k_thomas: at most 128 registers per thread, i.e. 16 warps
// per SM, so the 2048 warps of a 65536-system batch run in one wave; 64-thread
// CTAs where the rows are not in step (FP64, FP32), in_step_tpb's CTAs (up
// to 256 threads) where they are (float-float).  The kernel is bound by memory latency at m = 5 (one thread
// carries a whole block row), so resident warps matter more than the few
// spills the cap causes: on GB300 the float-float m = 5 solve runs in 8.3 ms
// at 128 registers, 9.8 ms at 168 (a second, latency-bound wave) and 9.7 ms at
// 96 (spills).
#ifndef PBT_THOMAS_THREADS
#define PBT_THOMAS_THREADS 64
#endif
#ifndef PBT_THOMAS_MAXNREG
#define PBT_THOMAS_MAXNREG 128
#endif
// Compiler fence between the block rows of one row's loads (keeps only one
// row of A and B live; 0 lets the compiler hoist all of a row's loads).
#ifndef PBT_ROW_FENCE
#define PBT_ROW_FENCE 1
#endif
constexpr int kThomasThreads = PBT_THOMAS_THREADS;

// Geometry of one solve as a body sees it: pointers already offset to the
// thread's system (and segment), `plane` = element-plane stride, `rs` = row
// stride (the number of systems interleaved in the layout).
template <class Num, int M, bool InStep = false>
__device__ __forceinline__ void thomas_body(const double* A, const double* B, const double* C, double* D,
                                            double* CW, size_t plane0, size_t rs, int N, bool raw, unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    T cp[M][M], y[M];
    unsigned amax = 0;
    for (int q = 0; q < N; ++q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        const bool last = (q == N - 1);
        Acc r[M][M], x[M][M + 1];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            T ar[M];
            if (q > 0) {
PBT_UNROLL
                for (int k = 0; k < M; ++k) ar[k] = Num::in(A + o + (size_t)(i + M * k) * plane);
            }
            Acc t = Num::acc(Num::in_rhs(D + o + (size_t)i * plane));
            if (q > 0) {
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::msub(t, ar[k], y[k]);
            }
            x[i][M] = t;
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                Acc s = Num::acc(Num::in_ro(B + o + (size_t)(i + M * j) * plane));
                if (q > 0) {
PBT_UNROLL
                    for (int k = 0; k < M; ++k) Num::msub(s, ar[k], cp[k][j]);
                }
                r[i][j] = s;
            }
            if (PBT_ROW_FENCE) mem_fence_compiler();
        }
        if (!last) {
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) x[i][j] = Num::acc(Num::in(C + o + (size_t)(i + M * j) * plane));
            gesv<Num, M, M + 1>(r, x, bad);
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
PBT_UNROLL
                for (int j = 0; j < M; ++j) cp[i][j] = Num::fin(x[i][j]);
                y[i] = Num::fin(x[i][M]);
            }
            st_fac_blk<Num, M>(CW + o, plane, cp, raw);
            st_raw_vec<Num, M>(D + o, plane, y);
        } else {
            Acc xv[M][1];
PBT_UNROLL
            for (int i = 0; i < M; ++i) xv[i][0] = x[i][M];
            gesv<Num, M, 1>(r, xv, bad);
PBT_UNROLL
            for (int i = 0; i < M; ++i) y[i] = Num::fin(xv[i][0]);
            out_vec<Num, M>(D + o, plane, y, amax);
        }
    }
    for (int q = N - 2; q >= 0; --q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T c[M][M], t[M];
        ld_fac_blk<Num, M>(c, CW + o, plane, raw);
        ld_raw_vec<Num, M>(t, D + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], y[k]);
            t[i] = Num::fin(s);
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) y[i] = t[i];
        out_vec<Num, M>(D + o, plane, y, amax);
    }
    bad |= range_bits<Num>(amax, true);
}

// Which body the direct-load single-segment kernel runs per block size:
// thomas_body (fused gesv, every right-hand side in registers) for m <= 4,
// where that fits the register budget and is the fastest form (GB300,
// float-float m = 4, 131072 systems: 14.8 ms vs 17.0 ms split); thomas_body_lu
// for m = 5, 6 (float-float m = 5, 65536 systems: 7.1 ms vs 8.6 ms fused);
// thomas_body with local-memory blocks above.
#ifndef PBT_THOMAS_LU_MIN
#define PBT_THOMAS_LU_MIN 5
#endif
// Load scheduling of thomas_body_lu, chosen per block size by measurement
// (GB300, float-float, 65536 systems): prefetching the next C column one
// column ahead helps m = 5 (7.09 -> 6.91 ms, N = 256; FP64 neither gains nor
// has the registers for it); reading A and C
// through the read-only path, which lets the assembler move C loads past the
// factor stores, helps m = 6 (10.38 -> 9.27 ms, N = 128); together they lose
// (registers).
// Loops over block columns kept rolled (one copy of the column's code
// instead of m): the fully unrolled float-float row is ~100 KB of code, and
// with a dozen warps at different points of it the warps stall on
// instruction fetch.  Measured on GB300 (65536 systems, float-float): m = 5
// 6.89 -> 6.53 ms, m = 6 9.02 -> 6.00 ms with both the C-column and the
// A-column loops rolled; FP64 (smaller code, bound by its pipe) gains
// nothing and keeps them unrolled.  A rolled A loop reads y_{q-1}[k] from
// shared memory (cps slot M*M + k) instead of a register.
template <class Num>
__host__ __device__ constexpr bool lu_rolled() {
    return Num::kConv;
}
// Variants of the rolled float-float row, chosen by measurement (GB300,
// pencil batch m = 5): the d column solved inside the C-column loop as its
// first column, one copy of the column solve's code less (PBT_LU_MERGE_Y:
// 6.25 -> 5.93 ms); the C-column loop unrolled by 2 (6.79 ms) or the
// A-column loop by 2 or 5 (6.50 / 6.43 ms) lose.
#ifndef PBT_LU_MERGE_Y
#define PBT_LU_MERGE_Y 1
#endif
#ifndef PBT_LU_COL_UNROLL
#define PBT_LU_COL_UNROLL 1
#endif
#ifndef PBT_LU_K_UNROLL
#define PBT_LU_K_UNROLL 1
#endif
template <class Num, int M>
__host__ __device__ constexpr bool lu_prefetch_c() {
    return M == 5 && Num::kConv;
}
// Same for the columns of A at m = 5 (float-float, 65536 systems: 6.15 ->
// 6.14 ms; 16384 systems: 3.81 -> 3.15 ms); at m = 6 it costs registers
// (5.83 -> 6.23 ms).
template <class Num, int M>
__host__ __device__ constexpr bool lu_prefetch_a() {
    return M == 5 && Num::kConv;
}
template <int M>
__host__ __device__ constexpr bool lu_ldg() {
    return M == 6;
}
constexpr int kThomasLuMinBlock = PBT_THOMAS_LU_MIN;
constexpr int kThomasLuMaxBlock = 6;
// Whether the split-row-step kernels keep their CTA's warps in step row by
// row (a barrier per row; InStep of thomas_body_lu / modi_body_lu).  Measured
// on GB300 (m = 5): float-float issue is bound by instruction fetch, and
// warps that run the same rows together share the instruction cache -- the
// pencil batch (65536 x 256) 5.93 -> 5.46 ms in one segment, 18.7 -> 13.0 ms
// in 16; the FP64 solve is bound by its pipe and gains nothing (12.65 ms
// without, 14.09 ms with).
template <class Num>
__host__ __device__ constexpr bool rows_in_step() {
    return std::is_same<Num, FF>::value;
}
// Which kernels run in step, by measurement (float-float, GB300): the split
// row step (m = 5, 6) and the periodic solve up to m = 6 (m = 5 pencil batch
// of periodic lines 14.15 -> 12.09 ms); the fused forms up to m = 4, which
// gain 1-2 % (m = 4: 65536 x 256 4.10 -> 4.01 ms, 256 lines of 32768 rows
// in 128 segments 5.00 -> 4.94 ms).  From m = 7 on, where the fused forms keep
// their blocks in local memory, the barrier costs 6-10 % (m = 8, 16384 x 256:
// 57.5 -> 60.7 ms) and is left out, as in the adjoint (m = 4, 16384 lines
// of 512 rows: 6.27 -> 6.85 ms with it).
template <class Num, int M>
__host__ __device__ constexpr bool fused_in_step() {
    return rows_in_step<Num>() && M <= 4;
}
// The fused local stage also in FP32 (the refined solve's two-stage passes),
// up to m = 6: pencil batch in 16 segments, refined, 18.14 -> 17.95 ms.
template <class Num, int M>
__host__ __device__ constexpr bool modi_in_step() {
    return fused_in_step<Num, M>() || (std::is_same<Num, F32>::value && M <= 6);
}
template <class Num, int M>
__host__ __device__ constexpr bool cyclic_in_step() {
    return rows_in_step<Num>() && M <= 6;
}

// Registers a thread of kernel k takes (cudaFuncGetAttributes; 255 when the
// query fails).
template <class K>
int kernel_regs(K* k) {
    cudaFuncAttributes a{};
    if (cudaFuncGetAttributes(&a, k) != cudaSuccess) {
        cudaGetLastError();
        return 255;
    }
    return a.numRegs > 0 ? a.numRegs : 255;
}

// CTA size of the in-step kernels: up to 256 threads, as many as two CTAs an
// SM allow with `smem_thread` bytes of shared memory and `regs` registers a
// thread, reduced so
// that `units` threads make whole waves of CTAs over the SMs (65536 systems
// on 152 SMs: 224 threads, 293 CTAs, at most two an SM).  A CTA size fixed by
// the caller (threads_per_block) is kept.
inline int in_step_tpb(const SolveArgs& g, long long units, size_t smem_thread, int regs) {
    if (!g.tpb_auto) return g.tpb;
    int cap = 256;
    while (cap > 32 && (2 * ((size_t)cap * smem_thread + 1024) > 228u * 1024u || 2L * cap * regs > 65536L)) cap -= 32;
    const long long sms = g.sms > 0 ? g.sms : 1;
    const long long waves = (units + cap * sms - 1) / (cap * sms);
    long long tpb = (units + waves * sms - 1) / (waves * sms);
    tpb = (tpb + 31) / 32 * 32;
    return (int)(tpb < 32 ? 32 : (tpb > cap ? cap : tpb));
}

template <int M>
__host__ __device__ constexpr bool thomas_uses_lu() {
    return M >= kThomasLuMinBlock && M <= kThomasLuMaxBlock;
}
// Block Thomas with the row step split into factor and column solves
// (lu_factor / lu_solve), for the register-resident block sizes.  The
// previous row's C' lives in shared memory (`cps`: this thread's M*M raw
// values, element (k, j) at cps[(k*M + j) * cstride], then y_{q-1} at
// cps[(M*M + k) * cstride]) instead of registers:
// the row reads it one row k at a time, so the registers hold the row's
// accumulators, the factors and one column, not also C'_{q-1} and every
// right-hand side.  R_q = B_q - A_q C'_{q-1} starts from B, as in
// thomas_body (adding B last instead measured slower in this form, and costs
// m*m extra FP64 adds in the FP64 solve).  The operations and their order are
// exactly those of the TMA-staged kernel k_thomas_staged, so the two agree
// bit for bit.
//
// InStep: the CTA's threads meet at a barrier at the top of every row (forward
// and backward), so its warps run the same stretch of code together and share
// the instruction cache; a thread without a system (past the last one, in a
// partial CTA) takes the same barriers in thomas_idle_rows.
template <class Num, int M, bool MergeY = (PBT_LU_MERGE_Y != 0), bool InStep = false>
__device__ __forceinline__ void thomas_body_lu(const double* A, const double* B, const double* C, double* D,
                                               double* CW, double* cps, int cstride, size_t plane0, size_t rs,
                                               int N, bool raw, unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    // Element e = i + M*j of a row's block is at base + e*plane: every phase
    // walks its array in increasing e with one running pointer, and re-reads
    // the plane stride through opaque() so that no phase keeps a table of
    // 64-bit element addresses alive across the arithmetic.
    T y[M];
    unsigned amax = 0;
    for (int q = 0; q < N; ++q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const bool last = (q == N - 1);
        Acc r[M][M], xd[M];
        {
            const size_t plane = opaque(plane0);
            const double* pd = D + o;
PBT_UNROLL
            for (int i = 0; i < M; ++i, pd += plane) xd[i] = Num::acc(Num::in_rhs(pd));
        }
        {
            const size_t plane = opaque(plane0);
            const double* pb = B + o;
PBT_UNROLL
            for (int j = 0; j < M; ++j)
PBT_UNROLL
                for (int i = 0; i < M; ++i, pb += plane) r[i][j] = Num::acc(Num::in_ro(pb));
        }
        if (q > 0) {
            const size_t plane = opaque(plane0);
            const double* pa = A + o;
            // lu_prefetch_a: column k+1 of A is loaded (raw) before column k is
            // used, so one column is always in flight.
            double an[M];
            if constexpr (lu_prefetch_a<Num, M>()) {
PBT_UNROLL
                for (int i = 0; i < M; ++i, pa += plane) an[i] = __ldg(pa);
            }
            constexpr int kKUnroll = lu_rolled<Num>() ? PBT_LU_K_UNROLL : M;
#pragma unroll(kKUnroll)
            for (int k = 0; k < M; ++k) {
                T ck[M];
PBT_UNROLL
                for (int j = 0; j < M; ++j) ck[j] = Num::lds(cps + (k * M + j) * cstride);
                T yk;
                if constexpr (lu_rolled<Num>())
                    yk = Num::lds(cps + (M * M + k) * cstride);
                else
                    yk = y[k];
                double ac[M];
                if constexpr (lu_prefetch_a<Num, M>()) {
PBT_UNROLL
                    for (int i = 0; i < M; ++i) ac[i] = an[i];
                    if (k + 1 < M) {
PBT_UNROLL
                        for (int i = 0; i < M; ++i, pa += plane) an[i] = __ldg(pa);
                    }
                }
PBT_UNROLL
                for (int i = 0; i < M; ++i) {
                    T a;
                    if constexpr (lu_prefetch_a<Num, M>()) {
                        a = Num::in(&ac[i]);
                    } else {
                        a = lu_ldg<M>() ? Num::in_ro(pa) : Num::in(pa);
                        pa += plane;
                    }
PBT_UNROLL
                    for (int j = 0; j < M; ++j) Num::msub(r[i][j], a, ck[j]);
                    Num::msub(xd[i], a, yk);
                }
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
        }
        LU<Num, M> lu;
        lu_factor<Num, M>(r, lu, bad);
        // MergeY: y as column -1 of the rolled column loop (one copy of the
        // column solve's code for y and C).
        if constexpr (MergeY && lu_rolled<Num>()) {
            const size_t plane = opaque(plane0);
            const double* pc = C + o;
            double* pw = CW + o;
            auto ld_c = [&](const double* p) -> double { return (lu_ldg<M>() && raw) ? __ldg(p) : *p; };
            double nxt[M];
            if (lu_prefetch_c<Num, M>() && !last) {
PBT_UNROLL
                for (int i = 0; i < M; ++i, pc += plane) nxt[i] = ld_c(pc);
            }
            const int jend = last ? 0 : M;
#pragma unroll 1
            for (int j = -1; j < jend; ++j) {
                Acc cj[M];
                T xj[M];
                if (j < 0) {
PBT_UNROLL
                    for (int i = 0; i < M; ++i) cj[i] = xd[i];
                } else if constexpr (lu_prefetch_c<Num, M>()) {
                    double cur[M];
PBT_UNROLL
                    for (int i = 0; i < M; ++i) cur[i] = nxt[i];
                    if (j + 1 < M) {
PBT_UNROLL
                        for (int i = 0; i < M; ++i, pc += plane) nxt[i] = ld_c(pc);
                    }
PBT_UNROLL
                    for (int i = 0; i < M; ++i) cj[i] = Num::acc(Num::in(&cur[i]));
                } else {
PBT_UNROLL
                    for (int i = 0; i < M; ++i, pc += plane) {
                        const double v = ld_c(pc);
                        cj[i] = Num::acc(Num::in(&v));
                    }
                }
                lu_solve<Num, M>(lu, cj, xj);
                if (j < 0) {
PBT_UNROLL
                    for (int i = 0; i < M; ++i) {
                        y[i] = xj[i];
                        Num::sts(cps + (M * M + i) * cstride, xj[i]);
                    }
                } else {
PBT_UNROLL
                    for (int i = 0; i < M; ++i, pw += plane) {
                        if (raw || !Num::kConv)
                            Num::sts(pw, xj[i]);
                        else
                            Num::out(pw, xj[i]);
                        Num::sts(cps + (i * M + j) * cstride, xj[i]);
                    }
                }
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
            if (last) {
                out_vec<Num, M>(D + o, plane, y, amax);
                break;
            }
            st_raw_vec<Num, M>(D + o, plane, y);
            continue;
        }
        lu_solve<Num, M>(lu, xd, y);
        if constexpr (lu_rolled<Num>()) {
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::sts(cps + (M * M + k) * cstride, y[k]);
        }
        {
            const size_t plane = opaque(plane0);
            if (last) {
                out_vec<Num, M>(D + o, plane, y, amax);
                break;
            }
            st_raw_vec<Num, M>(D + o, plane, y);
        }
        const size_t plane = opaque(plane0);
        const double* pc = C + o;
        double* pw = CW + o;
        // C is read-only unless the factors go into it (in place): then its
        // loads may not pass the stores of earlier columns.  With
        // lu_prefetch_c the next column's raw values are loaded before the
        // current column is solved and stored, so one column is always in
        // flight whatever the aliasing (lu_prefetch_c, lu_ldg).
        auto ld_c = [&](const double* p) -> double { return (lu_ldg<M>() && raw) ? __ldg(p) : *p; };
        double nxt[M];
        if constexpr (lu_prefetch_c<Num, M>()) {
PBT_UNROLL
            for (int i = 0; i < M; ++i, pc += plane) nxt[i] = ld_c(pc);
        }
        constexpr int kColUnroll = lu_rolled<Num>() ? PBT_LU_COL_UNROLL : M;
#pragma unroll(kColUnroll)
        for (int j = 0; j < M; ++j) {
            Acc cj[M];
            T xj[M];
            if constexpr (lu_prefetch_c<Num, M>()) {
                double cur[M];
PBT_UNROLL
                for (int i = 0; i < M; ++i) cur[i] = nxt[i];
                if (j + 1 < M) {
PBT_UNROLL
                    for (int i = 0; i < M; ++i, pc += plane) nxt[i] = ld_c(pc);
                }
PBT_UNROLL
                for (int i = 0; i < M; ++i) cj[i] = Num::acc(Num::in(&cur[i]));
            } else {
PBT_UNROLL
                for (int i = 0; i < M; ++i, pc += plane) {
                    const double v = ld_c(pc);
                    cj[i] = Num::acc(Num::in(&v));
                }
            }
            lu_solve<Num, M>(lu, cj, xj);
PBT_UNROLL
            for (int i = 0; i < M; ++i, pw += plane) {
                if (raw || !Num::kConv)
                    Num::sts(pw, xj[i]);
                else
                    Num::out(pw, xj[i]);
                Num::sts(cps + (i * M + j) * cstride, xj[i]);
            }
            if (PBT_ROW_FENCE) mem_fence_compiler();
        }
    }
    for (int q = N - 2; q >= 0; --q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T c[M][M], t[M];
        ld_fac_blk<Num, M>(c, CW + o, plane, raw);
        ld_raw_vec<Num, M>(t, D + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], y[k]);
            t[i] = Num::fin(s);
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) y[i] = t[i];
        out_vec<Num, M>(D + o, plane, y, amax);
    }
    bad |= range_bits<Num>(amax, true);
}


template <class Num, int M>
__host__ __device__ constexpr bool thomas_in_step() {
    return thomas_uses_lu<M>() ? rows_in_step<Num>() : fused_in_step<Num, M>();
}
// The barriers of thomas_body_lu / thomas_body <..., InStep = true> for a
// thread without a system: the same loop headers, one barrier per forward and
// backward row.
static __device__ __noinline__ void thomas_idle_rows(int N) {
    for (int q = 0; q < N; ++q) cta_row_barrier();
    for (int q = N - 2; q >= 0; --q) cta_row_barrier();
}

template <class Num, int M>
__global__ void __maxnreg__(PBT_THOMAS_MAXNREG) k_thomas(const SolveArgs g) {
    constexpr bool kStep = thomas_in_step<Num, M>();
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) {
        if constexpr (kStep) thomas_idle_rows(g.nrow);
        return;
    }
    unsigned bad = 0;
    if constexpr (thomas_uses_lu<M>()) {
        extern __shared__ double thomas_cps[];
        thomas_body_lu<Num, M, (PBT_LU_MERGE_Y != 0), kStep>(
            g.a + sys, g.b + sys, g.c + sys, g.d + sys, g.cw + sys, thomas_cps + threadIdx.x, blockDim.x,
            (size_t)g.nsys * g.nrow, (size_t)g.nsys, g.nrow, g.factors_raw != 0, bad);
    } else {
        thomas_body<Num, M, kStep>(g.a + sys, g.b + sys, g.c + sys, g.d + sys, g.cw + sys, (size_t)g.nsys * g.nrow,
                            (size_t)g.nsys, g.nrow, g.factors_raw != 0, bad);
    }
    report_status(g.status, bad);
}

// The same solve for lines addressed by strides (pbt_solve_noncyclic_lines).
// Kept apart from k_thomas, whose code generation at m = 5 proved sensitive:
// folding the strides into it (chosen at run time or by a template parameter,
// with the strides carried in SolveArgs) made the reference-layout solve ~5 %
// slower.
template <class Num, int M>
__global__ void __maxnreg__(PBT_THOMAS_MAXNREG) k_thomas_lines(const SolveArgs g, const LineStrides ls) {
    constexpr bool kStep = thomas_in_step<Num, M>();
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) {
        if constexpr (kStep) thomas_idle_rows(g.nrow);
        return;
    }
    unsigned bad = 0;
    const size_t o = (size_t)(sys % ls.lin) * (size_t)ls.in + (size_t)(sys / ls.lin) * (size_t)ls.out;
    if constexpr (thomas_uses_lu<M>()) {
        extern __shared__ double thomas_cps[];
        thomas_body_lu<Num, M, (PBT_LU_MERGE_Y != 0), kStep>(g.a + o, g.b + o, g.c + o, g.d + o, g.cw + o, thomas_cps + threadIdx.x, blockDim.x,
                               (size_t)ls.elem, (size_t)ls.row, g.nrow, g.factors_raw != 0, bad);
    } else {
        thomas_body<Num, M, kStep>(g.a + o, g.b + o, g.c + o, g.d + o, g.cw + o, (size_t)ls.elem, (size_t)ls.row, g.nrow,
                            g.factors_raw != 0, bad);
    }
    report_status(g.status, bad);
}

// ---------------------------------------------------------------------------
// Periodic lines in one segment: btdma_many_cycl
// (Fortran_Original/src/mod_btdma_cpu.f90:80-183) applied to the whole line,
// the GPU counterpart of the two-stage cyclic solve with P = 1.  Row 0 is the
// anchor; rows 1..N-1 are eliminated with the fill-in column e, which carries
// the coupling to x_0 (e_1 = -A_1, e_{N-1} = -C_{N-1}, zero in between):
//   forward, q = 1..N-1:  R_q = B_q - A_q C'_{q-1} (R_1 = B_1),
//     [y_q | e'_q | C'_q] = R_q^{-1} [d_q - A_q y_{q-1} | e_q - A_q e'_{q-1} | C_q]
//   backward, q = N-2..1: y_q -= C'_q y_{q+1},  e'_q -= C'_q e'_{q+1}
//   row 0: (B_0 + A_0 e'_{N-1} + C_0 e'_1) x_0 = d_0 - A_0 y_{N-1} - C_0 y_1
//   rows 1..N-1: x_q = y_q + e'_q x_0.
// The row step is split as in thomas_body_lu: R_q is factored once and y, the
// m columns of e' and the m columns of C' are solved one column at a time.
// Per thread, shared memory holds C'_{q-1} (slots k*M + j), y_{q-1} (M*M + k)
// and e'_{q-1} (kE + k*M + j).  Before the factorisation, W = A_q e'_{q-1}
// replaces e'_{q-1} in its slots (the product the reference forms with
// dgemm), so that no m x m accumulator block beyond R is live at a time; the
// e-columns then overwrite W column by column.  e' goes to EW (raw values of
// the arithmetic, nsys * N * m * m), C' to CW as in k_thomas, y (then the
// back-substituted y) to D.  Needs N >= 3.
// ---------------------------------------------------------------------------
// Column k of a block (M raw FP64 values, `plane` apart, read through `pa`,
// which advances by one column per call) into `cur`: with Ahead, `nxt`
// already holds column k and column k + 1 is loaded into it.
template <int M, bool Ahead>
__device__ __forceinline__ void ld_col_ahead(double (&cur)[M], double (&nxt)[M], const double*& pa, size_t plane,
                                             int k) {
    if constexpr (Ahead) {
PBT_UNROLL
        for (int i = 0; i < M; ++i) cur[i] = nxt[i];
        if (k + 1 < M) {
PBT_UNROLL
            for (int i = 0; i < M; ++i, pa += plane) nxt[i] = __ldg(pa);
        }
    } else {
PBT_UNROLL
        for (int i = 0; i < M; ++i, pa += plane) cur[i] = __ldg(pa);
    }
}

template <class Num, int M>
__host__ __device__ constexpr int cyclic_slots() {
    return 2 * M * M + M;
}

template <class Num, int M, bool InStep = false>
__device__ __forceinline__ void thomas_cyclic_body(const double* A, const double* B, const double* C, double* D,
                                                   double* CW, double* EW, double* cps, int cstride, size_t plane0,
                                                   size_t rs, int N, bool raw, unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    constexpr int kY = M * M;      // y_{q-1}
    constexpr int kE = M * M + M;  // e'_{q-1}, then W, then e'_q
    // Column loops rolled for float-float (code size, as in thomas_body_lu)
    // and from m = 5 on in FP64 too: unrolled, the FP64 m = 5 body spills
    // ~0.6 KB a thread at the 128-register cap, rolled it spills nothing.
    constexpr bool kRolled = lu_rolled<Num>() || M >= 5;
    // A's columns one ahead up to m = 5 (at m = 6 the extra registers spill).
    constexpr bool kPrefetchA = M <= 5;
    auto slot = [&](int s) -> double* { return cps + s * cstride; };
    T y[M];
    for (int q = 1; q < N; ++q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const bool last = (q == N - 1);
        // W = A_q e'_{q-1} into the e slots; row 1: W = A_1 (its e is -A_1).
        if (q == 1) {
            const size_t plane = opaque(plane0);
            const double* pa = A + o;
PBT_UNROLL
            for (int j = 0; j < M; ++j)
PBT_UNROLL
                for (int i = 0; i < M; ++i, pa += plane) Num::sts(slot(kE + i * M + j), Num::in(pa));
        } else {
            const size_t plane = opaque(plane0);
            const double* pa = A + o;
            Acc w[M][M];
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) w[i][j] = Num::acc0();
            // kPrefetchA: column k + 1 of A is loaded (raw) before column k
            // is used.
            double an[M];
            if constexpr (kPrefetchA) {
PBT_UNROLL
                for (int i = 0; i < M; ++i, pa += plane) an[i] = __ldg(pa);
            }
#pragma unroll(kRolled ? 1 : M)
            for (int k = 0; k < M; ++k) {
                T ak[M], ek[M];
                double ac[M];
                ld_col_ahead<M, kPrefetchA>(ac, an, pa, plane, k);
PBT_UNROLL
                for (int i = 0; i < M; ++i) ak[i] = Num::in(&ac[i]);
PBT_UNROLL
                for (int j = 0; j < M; ++j) ek[j] = Num::lds(slot(kE + k * M + j));
PBT_UNROLL
                for (int i = 0; i < M; ++i)
PBT_UNROLL
                    for (int j = 0; j < M; ++j) Num::mac(w[i][j], ak[i], ek[j]);
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) Num::sts(slot(kE + i * M + j), Num::fin(w[i][j]));
        }
        Acc r[M][M], xd[M];
        {
            const size_t plane = opaque(plane0);
            const double* pd = D + o;
PBT_UNROLL
            for (int i = 0; i < M; ++i, pd += plane) xd[i] = Num::acc(Num::in_rhs(pd));
        }
        {
            const size_t plane = opaque(plane0);
            const double* pb = B + o;
PBT_UNROLL
            for (int j = 0; j < M; ++j)
PBT_UNROLL
                for (int i = 0; i < M; ++i, pb += plane) r[i][j] = Num::acc(Num::in_ro(pb));
        }
        if (q > 1) {
            const size_t plane = opaque(plane0);
            const double* pa = A + o;
            double an[M];
            if constexpr (kPrefetchA) {
PBT_UNROLL
                for (int i = 0; i < M; ++i, pa += plane) an[i] = __ldg(pa);
            }
#pragma unroll(kRolled ? 1 : M)
            for (int k = 0; k < M; ++k) {
                T ck[M];
PBT_UNROLL
                for (int j = 0; j < M; ++j) ck[j] = Num::lds(slot(k * M + j));
                T yk;
                if constexpr (kRolled)
                    yk = Num::lds(slot(kY + k));
                else
                    yk = y[k];
                double ac[M];
                ld_col_ahead<M, kPrefetchA>(ac, an, pa, plane, k);
PBT_UNROLL
                for (int i = 0; i < M; ++i) {
                    const T a = Num::in(&ac[i]);
PBT_UNROLL
                    for (int j = 0; j < M; ++j) Num::msub(r[i][j], a, ck[j]);
                    Num::msub(xd[i], a, yk);
                }
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
        }
        LU<Num, M> lu;
        lu_factor<Num, M>(r, lu, bad);
        lu_solve<Num, M>(lu, xd, y);
        if constexpr (kRolled) {
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::sts(slot(kY + k), y[k]);
        }
        st_raw_vec<Num, M>(D + o, opaque(plane0), y);
        // The 2m right-hand-side columns in one rolled loop (one copy of the
        // column solve's code): jj < m, column jj of e_q - W (e_q = -C_{N-1}
        // on the last row, else 0) into EW and the e slots; jj >= m, column
        // jj - m of C_q into CW and the C' slots (not on the last row).  y
        // keeps its own solve: inside the loop it measured slower here (the
        // pencil batch as periodic lines, float-float: 14.79 vs 14.07 ms).
        {
            const size_t plane = opaque(plane0);
            const int ncol = last ? M : 2 * M;
#pragma unroll 1
            for (int jj = 0; jj < ncol; ++jj) {
                const bool ecol = jj < M;
                const int j = ecol ? jj : jj - M;
                const double* pc = C + o + (size_t)(M * j) * plane;
                Acc v[M];
                T xj[M];
                if (ecol) {
PBT_UNROLL
                    for (int i = 0; i < M; ++i) {
                        const T w = Num::lds(slot(kE + i * M + j));
                        if (last) {
                            v[i] = Num::acc(Num::neg(Num::in(pc + (size_t)i * plane)));
                            Num::msub(v[i], w, Num::one());
                        } else {
                            v[i] = Num::acc(Num::neg(w));
                        }
                    }
                } else {
PBT_UNROLL
                    for (int i = 0; i < M; ++i) v[i] = Num::acc(Num::in(pc + (size_t)i * plane));
                }
                lu_solve<Num, M>(lu, v, xj);
                double* pw = (ecol ? EW : CW) + o + (size_t)(M * j) * plane;
                const int s0 = ecol ? kE + j : j;
PBT_UNROLL
                for (int i = 0; i < M; ++i) {
                    if (ecol || raw || !Num::kConv)
                        Num::sts(pw + (size_t)i * plane, xj[i]);
                    else
                        Num::out(pw + (size_t)i * plane, xj[i]);
                    Num::sts(slot(s0 + i * M), xj[i]);
                }
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
        }
        if (last) break;
    }
    // Row 0 needs e'_{N-1} and y_{N-1} as the forward sweep left them: they
    // move to the C' and y slots, which the backward sweep does not use.
PBT_UNROLL
    for (int s = 0; s < M * M; ++s) Num::sts(slot(s), Num::lds(slot(kE + s)));
PBT_UNROLL
    for (int k = 0; k < M; ++k) Num::sts(slot(kY + k), y[k]);
    for (int q = N - 2; q >= 1; --q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T c[M][M], t[M];
        ld_fac_blk<Num, M>(c, CW + o, plane, raw);
        ld_raw_vec<Num, M>(t, D + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], y[k]);
            t[i] = Num::fin(s);
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) y[i] = t[i];
        st_raw_vec<Num, M>(D + o, plane, y);
        double* pe = EW + o;
        // e'_q's columns one ahead (raw 8-byte values).
        double en[M], ec[M];
        const double* pn = pe;
        if constexpr (kPrefetchA) {
PBT_UNROLL
            for (int i = 0; i < M; ++i, pn += plane) en[i] = *pn;
        }
#pragma unroll(kRolled ? 1 : M)
        for (int j = 0; j < M; ++j) {
            T ej[M], nv[M];
PBT_UNROLL
            for (int k = 0; k < M; ++k) ej[k] = Num::lds(slot(kE + k * M + j));
            if constexpr (kPrefetchA) {
PBT_UNROLL
                for (int i = 0; i < M; ++i) ec[i] = en[i];
                if (j + 1 < M) {
PBT_UNROLL
                    for (int i = 0; i < M; ++i, pn += plane) en[i] = *pn;
                }
            } else {
PBT_UNROLL
                for (int i = 0; i < M; ++i, pn += plane) ec[i] = *pn;
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                Acc s = Num::acc(Num::from_raw(ec[i]));
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], ej[k]);
                nv[i] = Num::fin(s);
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i, pe += plane) {
                Num::sts(pe, nv[i]);
                Num::sts(slot(kE + i * M + j), nv[i]);
            }
        }
    }
    // Row 0; y = y_1 and the e slots hold e'_1 (both back-substituted).
    // R_0 and its right-hand side are accumulated by outer products, one
    // column of A_0 (then of C_0) at a time, so that only R_0 and one column
    // are live; each entry still sums its terms in the order B, A_0 e'_{N-1}
    // (k ascending), C_0 e'_1 (k ascending).
    unsigned amax = 0;
    T x0[M];
    {
        Acc r[M][M], t[M];
        {
            const size_t plane = opaque(plane0);
            const double* pd = D;
PBT_UNROLL
            for (int i = 0; i < M; ++i, pd += plane) t[i] = Num::acc(Num::in_rhs(pd));
            const double* pb = B;
PBT_UNROLL
            for (int j = 0; j < M; ++j)
PBT_UNROLL
                for (int i = 0; i < M; ++i, pb += plane) r[i][j] = Num::acc(Num::in_ro(pb));
        }
PBT_UNROLL
        for (int h = 0; h < 2; ++h) {
            // h = 0: A_0 with e'_{N-1}, y_{N-1} (C' and y slots); h = 1: C_0
            // with e'_1 (e slots) and y_1 (registers).
            const size_t plane = opaque(plane0);
            const double* pa = (h == 0 ? A : C);
            const int es = (h == 0 ? 0 : kE);
#pragma unroll(kRolled ? 1 : M)
            for (int k = 0; k < M; ++k) {
                T ak[M], ek[M];
PBT_UNROLL
                for (int i = 0; i < M; ++i, pa += plane) ak[i] = Num::in(pa);
PBT_UNROLL
                for (int j = 0; j < M; ++j) ek[j] = Num::lds(slot(es + k * M + j));
                const T yk = (h == 0) ? Num::lds(slot(kY + k)) : y[k];
PBT_UNROLL
                for (int i = 0; i < M; ++i) {
PBT_UNROLL
                    for (int j = 0; j < M; ++j) Num::mac(r[i][j], ak[i], ek[j]);
                    Num::msub(t[i], ak[i], yk);
                }
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
        }
        LU<Num, M> lu;
        lu_factor<Num, M>(r, lu, bad);
        lu_solve<Num, M>(lu, t, x0);
        out_vec<Num, M>(D, opaque(plane0), x0, amax);
    }
    for (int q = 1; q < N; ++q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T e[M][M], t[M];
        ld_raw_blk<Num, M>(e, EW + o, plane);
        ld_raw_vec<Num, M>(t, D + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::mac(s, e[i][k], x0[k]);
            t[i] = Num::fin(s);
        }
        out_vec<Num, M>(D + o, plane, t, amax);
    }
    bad |= range_bits<Num>(amax, true);
}

// The barriers of thomas_cyclic_body<..., InStep = true> for a thread
// without a system: the same loop headers (forward, backward, solution).
static __device__ __noinline__ void cyclic_idle_rows(int N) {
    for (int q = 1; q < N; ++q) cta_row_barrier();
    for (int q = N - 2; q >= 1; --q) cta_row_barrier();
    for (int q = 1; q < N; ++q) cta_row_barrier();
}

template <class Num, int M>
__global__ void __maxnreg__(PBT_THOMAS_MAXNREG) k_thomas_cyclic(const SolveArgs g) {
    constexpr bool kStep = cyclic_in_step<Num, M>();
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) {
        if constexpr (kStep) cyclic_idle_rows(g.nrow);
        return;
    }
    extern __shared__ double thomas_cps[];
    unsigned bad = 0;
    thomas_cyclic_body<Num, M, kStep>(g.a + sys, g.b + sys, g.c + sys, g.d + sys, g.cw + sys, g.re + sys,
                               thomas_cps + threadIdx.x, blockDim.x, (size_t)g.nsys * g.nrow, (size_t)g.nsys,
                               g.nrow, g.factors_raw != 0, bad);
    report_status(g.status, bad);
}

// ---------------------------------------------------------------------------
// Stage 1: modified elimination of one segment (rows f..l, n = l - f + 1).
// ---------------------------------------------------------------------------
// A..CW point at the segment's first row of this system; RA..RD at this
// system in the reduced layout (row stride rrs, plane stride rplane).
template <class Num, int M, bool InStep = false>
__device__ __forceinline__ void modi_body(const double* A, const double* B, const double* C, double* D, double* AW,
                                          double* CW, size_t plane0, size_t rs, int n, bool raw, double* RA,
                                          double* RC, double* RD, size_t rplane, size_t rrs, int seg, unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;

    T ap[M][M], cp[M][M], dp[M];
    // Rows 1 and 2 of the segment: [A'|C'|d'] = B^{-1}[A|C|d]; rows 3..n:
    // R = B - A C'_{q-1}; [A'|C'|d'] = R^{-1}[-A A'_{q-1} | C | d - A d'_{q-1}].
    for (int q = 0; q < n; ++q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        const bool first2 = (q < 2);
        Acc r[M][M], x[M][2 * M + 1];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            T ar[M];
PBT_UNROLL
            for (int k = 0; k < M; ++k) ar[k] = Num::in(A + o + (size_t)(i + M * k) * plane);
            Acc t = Num::acc(Num::in_rhs(D + o + (size_t)i * plane));
            if (!first2) {
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::msub(t, ar[k], dp[k]);
            }
            x[i][2 * M] = t;
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                Acc u = Num::acc(Num::in_ro(B + o + (size_t)(i + M * j) * plane));
                if (first2) {
                    x[i][j] = Num::acc(ar[j]);
                } else {
                    Acc s = Num::acc0();
PBT_UNROLL
                    for (int k = 0; k < M; ++k) {
                        Num::msub(s, ar[k], ap[k][j]);
                        Num::msub(u, ar[k], cp[k][j]);
                    }
                    x[i][j] = s;
                }
                r[i][j] = u;
            }
            mem_fence_compiler();
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i)
PBT_UNROLL
            for (int j = 0; j < M; ++j) x[i][M + j] = Num::acc(Num::in(C + o + (size_t)(i + M * j) * plane));
        gesv<Num, M, 2 * M + 1>(r, x, bad);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                ap[i][j] = Num::fin(x[i][j]);
                cp[i][j] = Num::fin(x[i][M + j]);
            }
            dp[i] = Num::fin(x[i][2 * M]);
        }
        st_fac_blk<Num, M>(AW + o, plane0, ap, raw);
        st_fac_blk<Num, M>(CW + o, plane0, cp, raw);
        st_raw_vec<Num, M>(D + o, plane0, dp);
    }
    // Reduced row 2*seg+1 = the segment's last row (A'_n, C'_n, d'_n).
    {
        const size_t ro = rrs * (size_t)(2 * seg + 1);
        st_raw_blk<Num, M>(RA + ro, rplane, ap);
        st_raw_blk<Num, M>(RC + ro, rplane, cp);
        st_raw_vec<Num, M>(RD + ro, rplane, dp);
    }
    // Backward sweep, rows n-2 .. 2 (1-based): carried row = q+1.
    {
        const int q1 = (n >= 4) ? n - 2 : 1;
        const size_t o1 = (size_t)q1 * rs;
        ld_fac_blk<Num, M>(ap, AW + o1, plane0, raw);
        ld_fac_blk<Num, M>(cp, CW + o1, plane0, raw);
        ld_raw_vec<Num, M>(dp, D + o1, plane0);
    }
    for (int q = n - 3; q >= 1; --q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T a[M][M], c[M][M], dq[M];
        ld_fac_blk<Num, M>(a, AW + o, plane, raw);
        ld_fac_blk<Num, M>(c, CW + o, plane, raw);
        ld_raw_vec<Num, M>(dq, D + o, plane);
        // Row by row: row i of the new A', C' needs only row i of C'_q.
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc t = Num::acc(dq[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(t, c[i][k], dp[k]);
            dq[i] = Num::fin(t);
            T nc[M];
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                Acc s = Num::acc(a[i][j]);
                Acc u = Num::acc0();
PBT_UNROLL
                for (int k = 0; k < M; ++k) {
                    Num::msub(s, c[i][k], ap[k][j]);
                    Num::msub(u, c[i][k], cp[k][j]);
                }
                a[i][j] = Num::fin(s);
                nc[j] = Num::fin(u);
            }
PBT_UNROLL
            for (int j = 0; j < M; ++j) c[i][j] = nc[j];
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                ap[i][j] = a[i][j];
                cp[i][j] = c[i][j];
            }
            dp[i] = dq[i];
        }
        st_fac_blk<Num, M>(AW + o, plane, ap, raw);
        st_fac_blk<Num, M>(CW + o, plane, cp, raw);
        st_raw_vec<Num, M>(D + o, plane, dp);
    }
    // Row 1: R = I - C'_1 A'_2; [A'_1|C'_1|d'_1] = R^{-1}[A'_1 | -C'_1 C'_2 | d'_1 - C'_1 d'_2].
    {
        const size_t plane = opaque(plane0);
        Acc r[M][M], x[M][2 * M + 1];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            T c0[M];
PBT_UNROLL
            for (int k = 0; k < M; ++k) c0[k] = ld_fac<Num>(CW + (size_t)(i + M * k) * plane, raw);
            Acc t = Num::acc(Num::lds(D + (size_t)i * plane));
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(t, c0[k], dp[k]);
            x[i][2 * M] = t;
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                Acc s = Num::acc(i == j ? Num::one() : Num::zero());
                Acc u = Num::acc0();
PBT_UNROLL
                for (int k = 0; k < M; ++k) {
                    Num::msub(s, c0[k], ap[k][j]);
                    Num::msub(u, c0[k], cp[k][j]);
                }
                r[i][j] = s;
                x[i][M + j] = u;
            }
            mem_fence_compiler();
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i)
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                x[i][j] = Num::acc(ld_fac<Num>(AW + (size_t)(i + M * j) * plane, raw));
            }
        gesv<Num, M, 2 * M + 1>(r, x, bad);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                ap[i][j] = Num::fin(x[i][j]);
                cp[i][j] = Num::fin(x[i][M + j]);
            }
            dp[i] = Num::fin(x[i][2 * M]);
        }
        st_fac_blk<Num, M>(AW, plane, ap, raw);
        st_fac_blk<Num, M>(CW, plane, cp, raw);
        st_raw_vec<Num, M>(D, plane, dp);
        const size_t ro = rrs * (size_t)(2 * seg);
        st_raw_blk<Num, M>(RA + ro, rplane, ap);
        st_raw_blk<Num, M>(RC + ro, rplane, cp);
        st_raw_vec<Num, M>(RD + ro, rplane, dp);
    }
}

#ifndef PBT_MODI_LU_MIN
#define PBT_MODI_LU_MIN 5
#endif
// The local stage with the row step split (lu_factor / lu_solve), for the
// register-resident block sizes where the fused 2m+1-column elimination of
// modi_body spills (m = 5: ~1.5 KB a thread at 255 registers, 8 warps an SM).
// Same algebra and storage as modi_body, organised like thomas_cyclic_body:
// per thread, shared memory holds C'_{q-1} (slots k*M + j), d'_{q-1} (M*M + k)
// and A'_{q-1} (kE + k*M + j); W = A_q A'_{q-1} (the reference's dgemm)
// replaces A'_{q-1} in its slots before R_q is formed, so at most one m x m
// accumulator block is live; R_q is factored once and d', the m columns of A'
// and the m columns of C' are solved one column at a time (one rolled loop).
// The backward sweep and the first row's step work column by column the same
// way, with the carried row's A' and C' in the slots.  64-thread CTAs at 128
// registers: 16 warps an SM where the shared memory allows.
// Not for FP32 (the refined solve's corrections): its single-float values fit
// the fused form's 255 registers with few spills, and the split form measured
// slower there (pencil batch, P = 16, two FP32 solves per refined solve:
// 23.4 ms against 18.2 ms).
template <class Num, int M>
__host__ __device__ constexpr bool modi_uses_lu() {
    return M >= PBT_MODI_LU_MIN && M <= 6 && !std::is_same<Num, F32>::value;
}

template <class Num, int M, bool InStep = false>
__device__ __forceinline__ void modi_body_lu(const double* A, const double* B, const double* C, double* D,
                                             double* AW, double* CW, double* cps, int cstride, size_t plane0,
                                             size_t rs, int n, bool raw, double* RA, double* RC, double* RD,
                                             size_t rplane, size_t rrs, int seg, unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    constexpr int kY = M * M;      // d'_{q-1}
    constexpr int kE = M * M + M;  // A'_{q-1}, then W, then A'_q
    constexpr bool kPrefetchA = M <= 5;
    auto slot = [&](int s) -> double* { return cps + s * cstride; };
    T y[M];  // d' of the row just solved (the carried row in the backward sweep)

    // Forward.  Rows 0, 1: [A'|C'|d'] = B^{-1}[A|C|d]; rows 2..n-1:
    // R = B - A C'_{q-1}; [A'|C'|d'] = R^{-1}[-A A'_{q-1} | C | d - A d'_{q-1}].
    for (int q = 0; q < n; ++q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const bool first2 = (q < 2);
        if (!first2) {
            const size_t plane = opaque(plane0);
            const double* pa = A + o;
            Acc w[M][M];
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) w[i][j] = Num::acc0();
            double an[M];
            if constexpr (kPrefetchA) {
PBT_UNROLL
                for (int i = 0; i < M; ++i, pa += plane) an[i] = __ldg(pa);
            }
#pragma unroll 1
            for (int k = 0; k < M; ++k) {
                T ak[M], ek[M];
                double ac[M];
                ld_col_ahead<M, kPrefetchA>(ac, an, pa, plane, k);
PBT_UNROLL
                for (int i = 0; i < M; ++i) ak[i] = Num::in(&ac[i]);
PBT_UNROLL
                for (int j = 0; j < M; ++j) ek[j] = Num::lds(slot(kE + k * M + j));
PBT_UNROLL
                for (int i = 0; i < M; ++i)
PBT_UNROLL
                    for (int j = 0; j < M; ++j) Num::mac(w[i][j], ak[i], ek[j]);
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) Num::sts(slot(kE + i * M + j), Num::fin(w[i][j]));
        }
        Acc r[M][M], xd[M];
        {
            const size_t plane = opaque(plane0);
            const double* pd = D + o;
PBT_UNROLL
            for (int i = 0; i < M; ++i, pd += plane) xd[i] = Num::acc(Num::in_rhs(pd));
            const double* pb = B + o;
PBT_UNROLL
            for (int j = 0; j < M; ++j)
PBT_UNROLL
                for (int i = 0; i < M; ++i, pb += plane) r[i][j] = Num::acc(Num::in_ro(pb));
        }
        if (!first2) {
            const size_t plane = opaque(plane0);
            const double* pa = A + o;
            double an[M];
            if constexpr (kPrefetchA) {
PBT_UNROLL
                for (int i = 0; i < M; ++i, pa += plane) an[i] = __ldg(pa);
            }
#pragma unroll 1
            for (int k = 0; k < M; ++k) {
                T ck[M];
PBT_UNROLL
                for (int j = 0; j < M; ++j) ck[j] = Num::lds(slot(k * M + j));
                const T yk = Num::lds(slot(kY + k));
                double ac[M];
                ld_col_ahead<M, kPrefetchA>(ac, an, pa, plane, k);
PBT_UNROLL
                for (int i = 0; i < M; ++i) {
                    const T a = Num::in(&ac[i]);
PBT_UNROLL
                    for (int j = 0; j < M; ++j) Num::msub(r[i][j], a, ck[j]);
                    Num::msub(xd[i], a, yk);
                }
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
        }
        LU<Num, M> lu;
        lu_factor<Num, M>(r, lu, bad);
        lu_solve<Num, M>(lu, xd, y);
PBT_UNROLL
        for (int k = 0; k < M; ++k) Num::sts(slot(kY + k), y[k]);
        st_raw_vec<Num, M>(D + o, opaque(plane0), y);
        // jj < m: column jj of A' (right-hand side A on rows 0, 1, else -W);
        // jj >= m: column jj - m of C'.
        {
            const size_t plane = opaque(plane0);
#pragma unroll 1
            for (int jj = 0; jj < 2 * M; ++jj) {
                const bool acol = jj < M;
                const int j = acol ? jj : jj - M;
                const size_t co = o + (size_t)(M * j) * plane;
                Acc v[M];
                T xj[M];
                if (acol && !first2) {
PBT_UNROLL
                    for (int i = 0; i < M; ++i) v[i] = Num::acc(Num::neg(Num::lds(slot(kE + i * M + j))));
                } else {
                    const double* ps = (acol ? A : C) + co;
PBT_UNROLL
                    for (int i = 0; i < M; ++i) v[i] = Num::acc(Num::in(ps + (size_t)i * plane));
                }
                lu_solve<Num, M>(lu, v, xj);
                double* pw = (acol ? AW : CW) + co;
                const int s0 = acol ? kE + j : j;
PBT_UNROLL
                for (int i = 0; i < M; ++i) {
                    st_fac<Num>(pw + (size_t)i * plane, xj[i], raw);
                    Num::sts(slot(s0 + i * M), xj[i]);
                }
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
        }
    }
    // Reduced row 2*seg+1 = the segment's last row (A'_n, C'_n, d'_n).
    {
        const size_t ro = rrs * (size_t)(2 * seg + 1);
PBT_UNROLL
        for (int j = 0; j < M; ++j)
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                Num::sts(RA + ro + (size_t)(i + M * j) * rplane, Num::lds(slot(kE + i * M + j)));
                Num::sts(RC + ro + (size_t)(i + M * j) * rplane, Num::lds(slot(i * M + j)));
            }
        st_raw_vec<Num, M>(RD + ro, rplane, y);
    }
    // Backward, rows n-3 .. 1 (0-based), carried row q+1 starting at n-2:
    // A'_q -= C'_q A'_{q+1};  C'_q = -C'_q C'_{q+1};  d'_q -= C'_q d'_{q+1}.
    if (n >= 3) {
        const int q1 = (n >= 4) ? n - 2 : 1;
        const size_t o1 = (size_t)q1 * rs;
        const size_t plane = opaque(plane0);
PBT_UNROLL
        for (int j = 0; j < M; ++j)
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                const size_t e = (size_t)(i + M * j) * plane;
                Num::sts(slot(kE + i * M + j), ld_fac<Num>(AW + o1 + e, raw));
                Num::sts(slot(i * M + j), ld_fac<Num>(CW + o1 + e, raw));
            }
        ld_raw_vec<Num, M>(y, D + o1, plane);
    }
    for (int q = n - 3; q >= 1; --q) {
        if constexpr (InStep) cta_row_barrier();
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T c[M][M], t[M];
        ld_fac_blk<Num, M>(c, CW + o, plane, raw);
        ld_raw_vec<Num, M>(t, D + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], y[k]);
            t[i] = Num::fin(s);
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) y[i] = t[i];
        st_raw_vec<Num, M>(D + o, plane, y);
#pragma unroll 1
        for (int jj = 0; jj < 2 * M; ++jj) {
            const bool acol = jj < M;
            const int j = acol ? jj : jj - M;
            const int s0 = acol ? kE + j : j;
            double* pw = (acol ? AW : CW) + o + (size_t)(M * j) * plane;
            T cj[M], nv[M];
PBT_UNROLL
            for (int k = 0; k < M; ++k) cj[k] = Num::lds(slot(s0 + k * M));
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                Acc s = acol ? Num::acc(ld_fac<Num>(pw + (size_t)i * plane, raw)) : Num::acc0();
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], cj[k]);
                nv[i] = Num::fin(s);
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                st_fac<Num>(pw + (size_t)i * plane, nv[i], raw);
                Num::sts(slot(s0 + i * M), nv[i]);
            }
            if (PBT_ROW_FENCE) mem_fence_compiler();
        }
    }
    // Row 0: R = I - C'_0 A'_1;
    // [A'_0 | C'_0 | d'_0] = R^{-1} [A'_0 | -C'_0 C'_1 | d'_0 - C'_0 d'_1],
    // with row 1's values (A'_1, C'_1 in the slots, d'_1 in y, which moves to
    // its slots for the rolled loop below).  W2 = C'_0 C'_1 replaces C'_1 in
    // its slots first.
    {
        const size_t plane = opaque(plane0);
PBT_UNROLL
        for (int k = 0; k < M; ++k) Num::sts(slot(kY + k), y[k]);
        {
            Acc w[M][M];
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) w[i][j] = Num::acc0();
#pragma unroll 1
            for (int k = 0; k < M; ++k) {
                T ck[M], ek[M];
PBT_UNROLL
                for (int i = 0; i < M; ++i) ck[i] = ld_fac<Num>(CW + (size_t)(i + M * k) * plane, raw);
PBT_UNROLL
                for (int j = 0; j < M; ++j) ek[j] = Num::lds(slot(k * M + j));
PBT_UNROLL
                for (int i = 0; i < M; ++i)
PBT_UNROLL
                    for (int j = 0; j < M; ++j) Num::mac(w[i][j], ck[i], ek[j]);
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) Num::sts(slot(i * M + j), Num::fin(w[i][j]));
        }
        Acc r[M][M], xd[M];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            xd[i] = Num::acc(Num::lds(D + (size_t)i * plane));
PBT_UNROLL
            for (int j = 0; j < M; ++j) r[i][j] = Num::acc(i == j ? Num::one() : Num::zero());
        }
#pragma unroll 1
        for (int k = 0; k < M; ++k) {
            T ck[M], ek[M];
PBT_UNROLL
            for (int i = 0; i < M; ++i) ck[i] = ld_fac<Num>(CW + (size_t)(i + M * k) * plane, raw);
PBT_UNROLL
            for (int j = 0; j < M; ++j) ek[j] = Num::lds(slot(kE + k * M + j));
            const T yk = Num::lds(slot(kY + k));
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
PBT_UNROLL
                for (int j = 0; j < M; ++j) Num::msub(r[i][j], ck[i], ek[j]);
                Num::msub(xd[i], ck[i], yk);
            }
            if (PBT_ROW_FENCE) mem_fence_compiler();
        }
        LU<Num, M> lu;
        lu_factor<Num, M>(r, lu, bad);
        lu_solve<Num, M>(lu, xd, y);
        st_raw_vec<Num, M>(D, plane, y);
        const size_t ro = rrs * (size_t)(2 * seg);
        st_raw_vec<Num, M>(RD + ro, rplane, y);
#pragma unroll 1
        for (int jj = 0; jj < 2 * M; ++jj) {
            const bool acol = jj < M;
            const int j = acol ? jj : jj - M;
            double* pw = (acol ? AW : CW) + (size_t)(M * j) * plane;
            Acc v[M];
            T xj[M];
PBT_UNROLL
            for (int i = 0; i < M; ++i)
                v[i] = acol ? Num::acc(ld_fac<Num>(pw + (size_t)i * plane, raw))
                            : Num::acc(Num::neg(Num::lds(slot(j + i * M))));
            lu_solve<Num, M>(lu, v, xj);
            double* pr = (acol ? RA : RC) + ro + (size_t)(M * j) * rplane;
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                st_fac<Num>(pw + (size_t)i * plane, xj[i], raw);
                Num::sts(pr + (size_t)i * rplane, xj[i]);
            }
            if (PBT_ROW_FENCE) mem_fence_compiler();
        }
    }
}

// The barriers of modi_body_lu<..., InStep = true> for a thread without a
// system: the same loop headers, one barrier per forward and backward row.
static __device__ __noinline__ void modi_idle_rows(int n) {
    for (int q = 0; q < n; ++q) cta_row_barrier();
    for (int q = n - 3; q >= 1; --q) cta_row_barrier();
}

template <class Num, int M>
__global__ void __maxnreg__(PBT_THOMAS_MAXNREG) k_modi_lu(const SolveArgs g) {
    constexpr bool kStep = rows_in_step<Num>();
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    const int seg = blockIdx.y;
    int f, l;
    seg_rows(g.nrow, g.nseg, seg, f, l);
    if (sys >= g.nsys) {
        if constexpr (kStep) modi_idle_rows(l - f + 1);
        return;
    }
    extern __shared__ double thomas_cps[];
    const size_t rs = (size_t)g.nsys;
    const size_t fo = (size_t)f * rs + sys;
    unsigned bad = 0;
    modi_body_lu<Num, M, kStep>(g.a + fo, g.b + fo, g.c + fo, g.d + fo, g.aw + fo, g.cw + fo,
                                thomas_cps + threadIdx.x, blockDim.x, rs * g.nrow, rs, l - f + 1,
                                g.factors_raw != 0, g.ra + sys, g.rc + sys, g.rd + sys, rs * 2 * g.nseg, rs, seg,
                                bad);
    report_status(g.status, bad);
}

template <class Num, int M>
__global__ void __launch_bounds__(256) k_modi(const SolveArgs g) {
    constexpr bool kStep = modi_in_step<Num, M>();
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    const int seg = blockIdx.y;
    int f, l;
    seg_rows(g.nrow, g.nseg, seg, f, l);
    if (sys >= g.nsys) {
        if constexpr (kStep) modi_idle_rows(l - f + 1);
        return;
    }
    const size_t rs = (size_t)g.nsys;
    const size_t fo = (size_t)f * rs + sys;
    unsigned bad = 0;
    modi_body<Num, M, kStep>(g.a + fo, g.b + fo, g.c + fo, g.d + fo, g.aw + fo, g.cw + fo, rs * g.nrow, rs, l - f + 1,
                      g.factors_raw != 0, g.ra + sys, g.rc + sys, g.rd + sys, rs * 2 * g.nseg, rs, seg, bad);
    report_status(g.status, bad);
}

// ---------------------------------------------------------------------------
// Stage 2: block Thomas on the R = 2P reduced rows (B = I).  Row 0's A and
// row R-1's C are never read.  C' overwrites rc, the solution overwrites rd.
// ---------------------------------------------------------------------------
template <class Num, int M>
__device__ __forceinline__ void reduced_body(const double* RA, double* RC, double* RD, size_t plane0, size_t rs,
                                             int R, unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;

    T cp[M][M], y[M];
    // Row 0: B = I, so [C'|y] = [C|d] exactly.
    ld_raw_blk<Num, M>(cp, RC, plane0);
    ld_raw_vec<Num, M>(y, RD, plane0);
    for (int q = 1; q < R; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        const bool last = (q == R - 1);
        Acc r[M][M], x[M][M + 1];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            T ar[M];
PBT_UNROLL
            for (int k = 0; k < M; ++k) ar[k] = Num::lds(RA + o + (size_t)(i + M * k) * plane);
            Acc t = Num::acc(Num::lds(RD + o + (size_t)i * plane));
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(t, ar[k], y[k]);
            x[i][M] = t;
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                Acc s = Num::acc(i == j ? Num::one() : Num::zero());
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::msub(s, ar[k], cp[k][j]);
                r[i][j] = s;
            }
            mem_fence_compiler();
        }
        if (!last) {
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) x[i][j] = Num::acc(Num::lds(RC + o + (size_t)(i + M * j) * plane));
            gesv<Num, M, M + 1>(r, x, bad);
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
PBT_UNROLL
                for (int j = 0; j < M; ++j) cp[i][j] = Num::fin(x[i][j]);
                y[i] = Num::fin(x[i][M]);
            }
            st_raw_blk<Num, M>(RC + o, plane, cp);
        } else {
            Acc xv[M][1];
PBT_UNROLL
            for (int i = 0; i < M; ++i) xv[i][0] = x[i][M];
            gesv<Num, M, 1>(r, xv, bad);
PBT_UNROLL
            for (int i = 0; i < M; ++i) y[i] = Num::fin(xv[i][0]);
        }
        st_raw_vec<Num, M>(RD + o, plane, y);
    }
    // The reduced solution (the segments' end rows) stands for the system's
    // solution in the range check: a whole line below the float-float limit,
    // or a non-finite value, shows here.
    unsigned amax = 0;
PBT_UNROLL
    for (int i = 0; i < M; ++i) amax = max(amax, Num::mag(y[i]));
    for (int q = R - 2; q >= 0; --q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T c[M][M], t[M];
        ld_raw_blk<Num, M>(c, RC + o, plane);
        ld_raw_vec<Num, M>(t, RD + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], y[k]);
            t[i] = Num::fin(s);
            amax = max(amax, Num::mag(t[i]));
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) y[i] = t[i];
        st_raw_vec<Num, M>(RD + o, plane, y);
    }
    bad |= range_bits<Num>(amax, true);
}

// The reduced solve with the row step split (lu_factor / lu_solve), for the
// batch's local-stage launch at m = 5, 6, where the fused reduced_body would
// spill heavily at that launch's 128 registers.  Same recurrence and stores as
// reduced_body (B = I; C' overwrites rc, the solution rd, both raw); C'_{q-1}
// and y_{q-1} live in this thread's shared-memory slots (k*M + j and
// M*M + k), as in thomas_body_lu.
template <class Num, int M>
__device__ __forceinline__ void reduced_body_lu(const double* RA, double* RC, double* RD, double* cps, int cstride,
                                                size_t plane0, size_t rs, int R, unsigned& bad) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    constexpr int kY = M * M;
    auto slot = [&](int s) -> double* { return cps + s * cstride; };
    T y[M];
    {
        // Row 0: B = I, so [C'|y] = [C|d] exactly.
        const size_t plane = opaque(plane0);
PBT_UNROLL
        for (int j = 0; j < M; ++j)
PBT_UNROLL
            for (int i = 0; i < M; ++i) Num::sts(slot(i * M + j), Num::lds(RC + (size_t)(i + M * j) * plane));
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            y[i] = Num::lds(RD + (size_t)i * plane);
            Num::sts(slot(kY + i), y[i]);
        }
    }
    for (int q = 1; q < R; ++q) {
        const size_t o = (size_t)q * rs;
        const bool last = (q == R - 1);
        Acc r[M][M], xd[M];
        {
            const size_t plane = opaque(plane0);
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                xd[i] = Num::acc(Num::lds(RD + o + (size_t)i * plane));
PBT_UNROLL
                for (int j = 0; j < M; ++j) r[i][j] = Num::acc(i == j ? Num::one() : Num::zero());
            }
            const double* pa = RA + o;
#pragma unroll 1
            for (int k = 0; k < M; ++k) {
                T ck[M], ak[M];
PBT_UNROLL
                for (int j = 0; j < M; ++j) ck[j] = Num::lds(slot(k * M + j));
                const T yk = Num::lds(slot(kY + k));
PBT_UNROLL
                for (int i = 0; i < M; ++i, pa += plane) ak[i] = Num::lds(pa);
PBT_UNROLL
                for (int i = 0; i < M; ++i) {
PBT_UNROLL
                    for (int j = 0; j < M; ++j) Num::msub(r[i][j], ak[i], ck[j]);
                    Num::msub(xd[i], ak[i], yk);
                }
                if (PBT_ROW_FENCE) mem_fence_compiler();
            }
        }
        LU<Num, M> lu;
        lu_factor<Num, M>(r, lu, bad);
        lu_solve<Num, M>(lu, xd, y);
        const size_t plane = opaque(plane0);
        st_raw_vec<Num, M>(RD + o, plane, y);
        if (last) break;
PBT_UNROLL
        for (int k = 0; k < M; ++k) Num::sts(slot(kY + k), y[k]);
#pragma unroll 1
        for (int j = 0; j < M; ++j) {
            double* pc = RC + o + (size_t)(M * j) * plane;
            Acc cj[M];
            T xj[M];
PBT_UNROLL
            for (int i = 0; i < M; ++i) cj[i] = Num::acc(Num::lds(pc + (size_t)i * plane));
            lu_solve<Num, M>(lu, cj, xj);
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                Num::sts(pc + (size_t)i * plane, xj[i]);
                Num::sts(slot(i * M + j), xj[i]);
            }
            if (PBT_ROW_FENCE) mem_fence_compiler();
        }
    }
    // Backward, as reduced_body, with its range check of the line.
    unsigned amax = 0;
PBT_UNROLL
    for (int i = 0; i < M; ++i) amax = max(amax, Num::mag(y[i]));
    for (int q = R - 2; q >= 0; --q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T c[M][M], t[M];
        ld_raw_blk<Num, M>(c, RC + o, plane);
        ld_raw_vec<Num, M>(t, RD + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], y[k]);
            t[i] = Num::fin(s);
            amax = max(amax, Num::mag(t[i]));
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) y[i] = t[i];
        st_raw_vec<Num, M>(RD + o, plane, y);
    }
    bad |= range_bits<Num>(amax, true);
}

template <class Num, int M>
__global__ void __launch_bounds__(128) k_reduced(const SolveArgs g) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    unsigned bad = 0;
    const size_t rs = (size_t)g.nsys;
    reduced_body<Num, M>(g.ra + sys, g.rc + sys, g.rd + sys, rs * 2 * g.nseg, rs, 2 * g.nseg, bad);
    report_status(g.status, bad);
}

// ---------------------------------------------------------------------------
// Stage 2, cyclic: periodic block Thomas on the R = 2P reduced rows (B = I)
// with the fill-in column E, following btdma_many_cycl
// (Fortran_Original/src/mod_btdma_cpu.f90:80-183).  Needs R >= 4.
// ---------------------------------------------------------------------------
template <class Num, int M>
__global__ void __launch_bounds__(128) k_reduced_cyclic(const SolveArgs g) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    const int R = 2 * g.nseg;
    const size_t plane0 = (size_t)g.nsys * R;
    const size_t rs = (size_t)g.nsys;
    const double* RA = g.ra + sys;
    double* RC = g.rc + sys;
    double* RD = g.rd + sys;
    double* RE = g.re + sys;
    unsigned bad = 0;

    // Row 1: B = I, so [d'|e'|c'] = [d | -A_1 | C_1] exactly.
    T cp[M][M], ep[M][M], dp[M];
    {
        T a1[M][M];
        ld_raw_blk<Num, M>(a1, RA + rs, plane0);
        ld_raw_blk<Num, M>(cp, RC + rs, plane0);
        ld_raw_vec<Num, M>(dp, RD + rs, plane0);
PBT_UNROLL
        for (int i = 0; i < M; ++i)
PBT_UNROLL
            for (int j = 0; j < M; ++j) ep[i][j] = Num::neg(a1[i][j]);
        st_raw_blk<Num, M>(RE + rs, plane0, ep);
    }
    // Rows 2..R-1: R_q = I - A_q C'_{q-1};
    // [d'|e'|c'] = R_q^{-1} [d - A_q d'_{q-1} | e_q - A_q e'_{q-1} | C_q],
    // with e_q = 0 except e_{R-1} = -C_{R-1}.
    for (int q = 2; q < R; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        const bool last = (q == R - 1);
        Acc r[M][M], x[M][2 * M + 1];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            T ar[M];
PBT_UNROLL
            for (int k = 0; k < M; ++k) ar[k] = Num::lds(RA + o + (size_t)(i + M * k) * plane);
            Acc t = Num::acc(Num::lds(RD + o + (size_t)i * plane));
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(t, ar[k], dp[k]);
            x[i][0] = t;
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                const T cij = Num::lds(RC + o + (size_t)(i + M * j) * plane);
                Acc s = Num::acc(i == j ? Num::one() : Num::zero());
                Acc u = Num::acc(last ? Num::neg(cij) : Num::zero());
PBT_UNROLL
                for (int k = 0; k < M; ++k) {
                    Num::msub(s, ar[k], cp[k][j]);
                    Num::msub(u, ar[k], ep[k][j]);
                }
                r[i][j] = s;
                x[i][1 + j] = u;
                x[i][1 + M + j] = Num::acc(cij);
            }
            mem_fence_compiler();
        }
        gesv<Num, M, 2 * M + 1>(r, x, bad);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            dp[i] = Num::fin(x[i][0]);
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                ep[i][j] = Num::fin(x[i][1 + j]);
                cp[i][j] = Num::fin(x[i][1 + M + j]);
            }
        }
        st_raw_vec<Num, M>(RD + o, plane, dp);
        st_raw_blk<Num, M>(RE + o, plane, ep);
        st_raw_blk<Num, M>(RC + o, plane, cp);
    }
    T elast[M][M], dlast[M];
PBT_UNROLL
    for (int i = 0; i < M; ++i) {
        dlast[i] = dp[i];
PBT_UNROLL
        for (int j = 0; j < M; ++j) elast[i][j] = ep[i][j];
    }
    // Backward, rows R-2..1: d'_q -= C'_q d'_{q+1}; e'_q -= C'_q e'_{q+1}.
    for (int q = R - 2; q >= 1; --q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T c[M][M], e[M][M], t[M];
        ld_raw_blk<Num, M>(c, RC + o, plane);
        ld_raw_blk<Num, M>(e, RE + o, plane);
        ld_raw_vec<Num, M>(t, RD + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], dp[k]);
            t[i] = Num::fin(s);
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                Acc u = Num::acc(e[i][j]);
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::msub(u, c[i][k], ep[k][j]);
                e[i][j] = Num::fin(u);
            }
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            dp[i] = t[i];
PBT_UNROLL
            for (int j = 0; j < M; ++j) ep[i][j] = e[i][j];
        }
        st_raw_vec<Num, M>(RD + o, plane, dp);
        st_raw_blk<Num, M>(RE + o, plane, ep);
    }
    // Row 0: (I + A_0 e'_{R-1} + C_0 e'_1) x_0 = d_0 - A_0 d'_{R-1} - C_0 d'_1.
    T x0[M];
    {
        T a0[M][M], c0[M][M];
        ld_raw_blk<Num, M>(a0, RA, plane0);
        ld_raw_blk<Num, M>(c0, RC, plane0);
        Acc r[M][M], x[M][1];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc t = Num::acc(Num::lds(RD + (size_t)i * plane0));
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(t, a0[i][k], dlast[k]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(t, c0[i][k], dp[k]);
            x[i][0] = t;
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                Acc s = Num::acc(i == j ? Num::one() : Num::zero());
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::mac(s, a0[i][k], elast[k][j]);
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::mac(s, c0[i][k], ep[k][j]);
                r[i][j] = s;
            }
        }
        gesv<Num, M, 1>(r, x, bad);
PBT_UNROLL
        for (int i = 0; i < M; ++i) x0[i] = Num::fin(x[i][0]);
        st_raw_vec<Num, M>(RD, plane0, x0);
    }
    // Rows 1..R-1: x_q = d'_q + e'_q x_0; the range check as in reduced_body.
    unsigned amax = 0;
PBT_UNROLL
    for (int i = 0; i < M; ++i) amax = max(amax, Num::mag(x0[i]));
    for (int q = 1; q < R; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T e[M][M], t[M];
        ld_raw_blk<Num, M>(e, RE + o, plane);
        ld_raw_vec<Num, M>(t, RD + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::mac(s, e[i][k], x0[k]);
            t[i] = Num::fin(s);
            amax = max(amax, Num::mag(t[i]));
        }
        st_raw_vec<Num, M>(RD + o, plane, t);
    }
    bad |= range_bits<Num>(amax, true);
    report_status(g.status, bad);
}

// ---------------------------------------------------------------------------
// Stage 3: interior update of one segment from the reduced solution.
// ---------------------------------------------------------------------------
template <class Num, int M>
__device__ __forceinline__ void update_body(const double* AW, const double* CW, double* D, size_t plane0, size_t rs,
                                            int n, bool raw, const double* RD, size_t rplane, size_t rrs, int seg,
                                            unsigned& amax) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    T x0[M], xn[M];
    ld_raw_vec<Num, M>(x0, RD + rrs * (size_t)(2 * seg), rplane);
    ld_raw_vec<Num, M>(xn, RD + rrs * (size_t)(2 * seg + 1), rplane);
    out_vec<Num, M>(D, plane0, x0, amax);
    out_vec<Num, M>(D + (size_t)(n - 1) * rs, plane0, xn, amax);
    for (int q = 1; q < n - 1; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T a[M][M], c[M][M], t[M];
        ld_fac_blk<Num, M>(a, AW + o, plane, raw);
        ld_fac_blk<Num, M>(c, CW + o, plane, raw);
        ld_raw_vec<Num, M>(t, D + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, a[i][k], x0[k]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], xn[k]);
            t[i] = Num::fin(s);
        }
        out_vec<Num, M>(D + o, plane, t, amax);
    }
}

template <class Num, int M>
__global__ void __launch_bounds__(128) k_update(const SolveArgs g) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    const int seg = blockIdx.y;
    int f, l;
    seg_rows(g.nrow, g.nseg, seg, f, l);
    const size_t rs = (size_t)g.nsys;
    const size_t fo = (size_t)f * rs + sys;
    unsigned amax = 0;
    update_body<Num, M>(g.aw + fo, g.cw + fo, g.d + fo, rs * g.nrow, rs, l - f + 1, g.factors_raw != 0, g.rd + sys,
                        rs * 2 * g.nseg, rs, seg, amax);
    // One segment of a line: Inf/NaN only (the reduced solve checked the
    // line's magnitude).
    report_status(g.status, range_bits<Num>(amax, false));
}

// ---------------------------------------------------------------------------
// Adjoint.  For x = M^{-1} d and a loss L(x) with g = dL/dx, the gradients are
// lambda = M^{-T} g = dL/dd and dL/dM = -lambda x^T on M's block pattern:
//   dA_q = -lambda_q x_{q-1}^T,  dB_q = -lambda_q x_q^T,  dC_q = -lambda_q x_{q+1}^T
// (dA_0 = dC_{N-1} = 0: those blocks never enter the non-cyclic solve).
// M^T is block tridiagonal with the lower and upper blocks swapped and every
// block transposed:  At_q = C_{q-1}^T,  Bt_q = B_q^T,  Ct_q = A_{q+1}^T.
//
// k_adjoint: single-segment block Thomas on M^T, reading A, B, C with
// transposed indexing (no transposed copy), with the gradient assembly fused
// into its backward sweep: when lambda_q is known, dB_q, dC_q and dA_{q+1} are
// written.  The forward factors are recomputed (the forward solve's workspace
// is reused for the adjoint's own C').  g holds dL/dx on entry and lambda on
// return; da/db/dc may be null.
// ---------------------------------------------------------------------------
// The gradient blocks that row q of the adjoint's backward sweep completes:
//   dB_q = -lambda_q x_q^T,  dC_q = -lambda_q x_{q+1}^T (0 at the last row),
//   dA_{q+1} = -lambda_{q+1} x_q^T, and dA_0 = 0 at q = 0,
// from lambda_q (lq) and lambda_{q+1} (ln, when `next`) as the FP64 values the
// sweep stores, and x_q, x_{q+1} read from X (this thread's system).  Nothing
// is carried across rows but the sweep's own y: the first form of this sweep
// kept lambda_q, lambda_{q+1}, x_q and x_{q+1} in six m-long per-thread arrays,
// copied and reset together between rows, and its FP64 rolled-loop
// instantiation (m >= 7) returned a wrong lambda from the last row on -- right
// when fully unrolled, in float-float, or without those arrays, and unchanged
// by ptxas -O0 -- so that construct is avoided.
template <class Num, int M>
__device__ __forceinline__ void adjoint_gradients(const AdjointArgs& adj, const typename Num::T (&lq)[M],
                                                  const typename Num::T (&ln)[M], bool next, const double* X,
                                                  int sys, size_t o, size_t plane, size_t rs, int q) {
PBT_UNROLL
    for (int i = 0; i < M; ++i) {
        const double li = Num::f64(lq[i]);
        const double lni = next ? Num::f64(ln[i]) : 0.0;
PBT_UNROLL
        for (int j = 0; j < M; ++j) {
            const size_t e = sys + o + (size_t)(i + M * j) * plane;
            const double xj = __ldg(X + o + (size_t)j * plane);
            const double xnj = next ? __ldg(X + o + rs + (size_t)j * plane) : 0.0;
            if (adj.db) adj.db[e] = -li * xj;
            if (adj.dc) adj.dc[e] = -li * xnj;
            if (adj.da) {
                if (next) adj.da[e + rs] = -lni * xj;
                if (q == 0) adj.da[e] = 0.0;
            }
        }
    }
}

template <class Num, int M>
__global__ void __maxnreg__(PBT_THOMAS_MAXNREG) k_adjoint(const SolveArgs g, const AdjointArgs adj) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    const int N = g.nrow;
    const size_t plane0 = (size_t)g.nsys * N;
    const size_t rs = (size_t)g.nsys;
    const double* A = g.a + sys;
    const double* B = g.b + sys;
    const double* C = g.c + sys;
    double* G = adj.g + sys;
    double* CW = g.cw + sys;
    unsigned bad = 0, amax = 0;

    // Forward over the transposed rows.
    T cp[M][M], y[M];
    for (int q = 0; q < N; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        const bool last = (q == N - 1);
        Acc r[M][M], x[M][M + 1];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            // row i of At_q = C_{q-1}^T: element (i, k) = C_{q-1}(k, i)
            T ar[M];
            if (q > 0) {
PBT_UNROLL
                for (int k = 0; k < M; ++k) ar[k] = Num::in(C + o - rs + (size_t)(k + M * i) * plane);
            }
            Acc t = Num::acc(Num::in_rhs(G + o + (size_t)i * plane));
            if (q > 0) {
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::msub(t, ar[k], y[k]);
            }
            x[i][M] = t;
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                Acc s = Num::acc(Num::in_ro(B + o + (size_t)(j + M * i) * plane));  // Bt_q(i, j) = B_q(j, i)
                if (q > 0) {
PBT_UNROLL
                    for (int k = 0; k < M; ++k) Num::msub(s, ar[k], cp[k][j]);
                }
                r[i][j] = s;
            }
            if (PBT_ROW_FENCE) mem_fence_compiler();
        }
        if (!last) {
            // Ct_q = A_{q+1}^T: element (i, j) = A_{q+1}(j, i)
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int j = 0; j < M; ++j) x[i][j] = Num::acc(Num::in(A + o + rs + (size_t)(j + M * i) * plane));
            gesv<Num, M, M + 1>(r, x, bad);
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
PBT_UNROLL
                for (int j = 0; j < M; ++j) cp[i][j] = Num::fin(x[i][j]);
                y[i] = Num::fin(x[i][M]);
            }
            st_raw_blk<Num, M>(CW + o, plane, cp);
            st_raw_vec<Num, M>(G + o, plane, y);
        } else {
            Acc xv[M][1];
PBT_UNROLL
            for (int i = 0; i < M; ++i) xv[i][0] = x[i][M];
            gesv<Num, M, 1>(r, xv, bad);
PBT_UNROLL
            for (int i = 0; i < M; ++i) y[i] = Num::fin(xv[i][0]);
        }
    }
    // Backward: lambda_q = y_q - Ct'_q lambda_{q+1}; y holds lambda_{q+1} on
    // entry to row q and lambda_q after it.  The gradient blocks of row q
    // take lambda_q from t and lambda_{q+1} from y before y is overwritten.
    const double* X = adj.x + sys;
    out_vec<Num, M>(G + (size_t)(N - 1) * rs, plane0, y, amax);
    adjoint_gradients<Num, M>(adj, y, y, false, X, sys, (size_t)(N - 1) * rs, plane0, rs, N - 1);
    for (int q = N - 2; q >= 0; --q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        T c[M][M], t[M];
        ld_raw_blk<Num, M>(c, CW + o, plane);
        ld_raw_vec<Num, M>(t, G + o, plane);
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            Acc s = Num::acc(t[i]);
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], y[k]);
            t[i] = Num::fin(s);
        }
        out_vec<Num, M>(G + o, plane, t, amax);
        adjoint_gradients<Num, M>(adj, t, y, true, X, sys, o, plane, rs, q);
PBT_UNROLL
        for (int i = 0; i < M; ++i) y[i] = t[i];
    }
    bad |= range_bits<Num>(amax, true);
    report_status(g.status, bad);
}

// Segmented adjoint, step 1: materialise M^T's blocks (At, Bt, Ct) in the
// reference layout; step 3 (after the ordinary two-stage solve of M^T lambda
// = g): the gradient blocks from lambda and x.  One thread per (system, row).
template <int M>
__global__ void k_transpose_blocks(const SolveArgs g, double* __restrict__ At, double* __restrict__ Bt,
                                   double* __restrict__ Ct) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t plane = (size_t)g.nsys * g.nrow;
    if (idx >= plane) return;
    const int q = (int)(idx / (size_t)g.nsys);
    const size_t rs = (size_t)g.nsys;
PBT_UNROLL
    for (int j = 0; j < M; ++j)
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            const size_t e = idx + (size_t)(i + M * j) * plane, et = (size_t)(j + M * i) * plane;
            Bt[e] = __ldg(g.b + idx + et);
            At[e] = (q > 0) ? __ldg(g.c + idx - rs + et) : 0.0;
            Ct[e] = (q + 1 < g.nrow) ? __ldg(g.a + idx + rs + et) : 0.0;
        }
}

template <int M>
__global__ void k_gradients(const SolveArgs g, const AdjointArgs adj) {
    const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t plane = (size_t)g.nsys * g.nrow;
    if (idx >= plane) return;
    const int q = (int)(idx / (size_t)g.nsys);
    const size_t rs = (size_t)g.nsys;
    double lam[M], xm[M], x0[M], xp[M];
PBT_UNROLL
    for (int i = 0; i < M; ++i) {
        lam[i] = adj.g[idx + (size_t)i * plane];
        x0[i] = __ldg(adj.x + idx + (size_t)i * plane);
        xm[i] = (q > 0) ? __ldg(adj.x + idx - rs + (size_t)i * plane) : 0.0;
        xp[i] = (q + 1 < g.nrow) ? __ldg(adj.x + idx + rs + (size_t)i * plane) : 0.0;
    }
PBT_UNROLL
    for (int j = 0; j < M; ++j)
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            const size_t e = idx + (size_t)(i + M * j) * plane;
            if (adj.da) adj.da[e] = -lam[i] * xm[j];
            if (adj.db) adj.db[e] = -lam[i] * x0[j];
            if (adj.dc) adj.dc[e] = -lam[i] * xp[j];
        }
}

// ---------------------------------------------------------------------------
// Iterative refinement (precision PBT_PREC_FP32_REFINE), FP64 parts.
//   k_residual64: E = d - M X for every system, in FP64 (the one FP64 pass of
//                 the refined solve): r_q = d_q - A_q x_{q-1} - B_q x_q - C_q x_{q+1}
//                 (A_0 and C_{N-1} not read, as in the non-cyclic solve).
//   k_accumulate: X += E, and the largest max|E| / max|X| over the systems
//                 into *stat (as ordered float bits) for the convergence test.
// Both run one thread per (system, block row i): a CTA is M warps over the
// same 32 systems (warp i = row i), so the FP64 pipe and the memory system
// see M times the threads of one per system; the M warps read the same x
// values, which the first of them brings into L1.
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(32 * M, 4) k_residual64(const SolveArgs g, const double* __restrict__ X,
                                                       double* __restrict__ E) {
    const int i = threadIdx.y;
    const int sys = blockIdx.x * 32 + threadIdx.x;
    if (sys >= g.nsys) return;
    const int N = g.nrow;
    const size_t plane0 = (size_t)g.nsys * N;
    const size_t rs = (size_t)g.nsys;
    double xm[M], x0[M], xp[M];
PBT_UNROLL
    for (int k = 0; k < M; ++k) {
        xm[k] = 0.0;
        x0[k] = X[sys + (size_t)k * plane0];
    }
    for (int q = 0; q < N; ++q) {
        const size_t o = (size_t)q * rs + sys;
        const size_t plane = opaque(plane0);
        const bool has_next = (q + 1 < N);
PBT_UNROLL
        for (int k = 0; k < M; ++k) xp[k] = has_next ? X[o + rs + (size_t)k * plane] : 0.0;
        double t = __ldg(g.d + o + (size_t)i * plane);
PBT_UNROLL
        for (int k = 0; k < M; ++k) t = fma(-__ldg(g.b + o + (size_t)(i + M * k) * plane), x0[k], t);
        if (q > 0) {
PBT_UNROLL
            for (int k = 0; k < M; ++k) t = fma(-__ldg(g.a + o + (size_t)(i + M * k) * plane), xm[k], t);
        }
        if (has_next) {
PBT_UNROLL
            for (int k = 0; k < M; ++k) t = fma(-__ldg(g.c + o + (size_t)(i + M * k) * plane), xp[k], t);
        }
        E[o + (size_t)i * plane] = t;
PBT_UNROLL
        for (int k = 0; k < M; ++k) {
            xm[k] = x0[k];
            x0[k] = xp[k];
        }
    }
}

// The refinement's per-system statistic: max|e| and max|x| over a system's
// correction e and updated solution x; a non-finite x makes max|e| +Inf
// (fmax would skip a NaN).
__device__ __forceinline__ void refine_stat(double& emax, double& xmax, double e, double x) {
    emax = fmax(emax, fabs(e));
    xmax = fmax(xmax, fabs(x));
    if ((__double2hiint(x) & 0x7ff00000) == 0x7ff00000) emax = CUDART_INF;
}
// One system's convergence statistic max|e| / max|x| (+Inf when undefined or
// not finite) into *stat, and its range check into the plan's status word: a
// solution that is not finite, or that lies wholly below 2^-100 (where the
// FP32 corrections underflow and stop refining it), is a range failure.
__device__ __forceinline__ void refine_report(double emax, double xmax, unsigned* stat, unsigned long long* status) {
    float ratio = (xmax > 0.0) ? (float)(emax / xmax) : (emax > 0.0 ? INFINITY : 0.f);
    if (!(ratio == ratio)) ratio = INFINITY;
    atomicMax(stat, __float_as_uint(ratio));
    if (!(ratio < INFINITY) || (xmax > 0.0 && xmax < 0x1p-100)) atomicOr(status, kRangeMark);
}

template <int M>
__global__ void __launch_bounds__(32 * M) k_accumulate(const SolveArgs g, double* __restrict__ X,
                                                       const double* __restrict__ E, unsigned* stat) {
    __shared__ double red[2][M][32];
    const int i = threadIdx.y, lane = threadIdx.x;
    const int sys = blockIdx.x * 32 + lane;
    double emax = 0.0, xmax = 0.0;
    if (sys < g.nsys) {
        const size_t plane = (size_t)g.nsys * g.nrow;
        const size_t rs = (size_t)g.nsys;
        for (int q = 0; q < g.nrow; ++q) {
            const size_t o = (size_t)q * rs + sys + (size_t)i * plane;
            const double e = E[o];
            const double x = X[o] + e;
            X[o] = x;
            refine_stat(emax, xmax, e, x);
        }
    }
    red[0][i][lane] = emax;
    red[1][i][lane] = xmax;
    __syncthreads();
    if (i == 0) {
PBT_UNROLL
        for (int k = 1; k < M; ++k) {
            emax = fmax(emax, red[0][k][lane]);
            xmax = fmax(xmax, red[1][k][lane]);
        }
        if (sys < g.nsys) refine_report(emax, xmax, stat, g.status);
    }
}

// k_refine_step: one whole correction of the refined solve in one pass over
// A, B, C, when the first FP32 pass kept its factors (the staged kernel,
// m <= 6).  Forward, row by row: the FP64 residual r_q = d_q - A_q x_{q-1} -
// B_q x_q - C_q x_{q+1} (the k_residual64 operations in the same order), then
// t = r_q - A_q y_{q-1} and y_q = R_q^{-1} t in FP32 with the stored LU of R_q
// (the operations of the FP32 solve, so e is the FP32 solve of r bit for bit;
// the factors come from ra.lu, tiled by warp as the staged pass wrote them);
// backward: e_q = y_q - C'_q e_{q+1} with the FP32 pass's C' (floats, as the
// staged FP32 kernel keeps them), and x_q += e_q with the convergence
// statistic of k_accumulate.  It reads A, B, C once per
// correction where the separate residual, FP32 solve and accumulate read them
// twice and move x and r three more times.  One thread per system, plain
// loads: the refined solve uses k_refine_staged (the same operations with the
// forward inputs staged through a TMA ring) and falls back to this kernel
// when the tensor maps cannot be encoded.
template <int M>
__global__ void __launch_bounds__(64) k_refine_step(const SolveArgs g, const RefineArgs ra) {
    if constexpr (M > kStagedMaxBlock) {
        return;  // the factors are kept by the staged kernel only (m <= 6)
    } else {
        const int sys = blockIdx.x * blockDim.x + threadIdx.x;
        if (sys >= g.nsys) return;
        const int N = g.nrow;
        const size_t plane0 = (size_t)g.nsys * N;
        const size_t rs = (size_t)g.nsys;
        const size_t ngroups = ((size_t)g.nsys + 31) / 32;
        float* Y = ra.y + sys;
        double* X = ra.x + sys;
        double xm[M], x0[M], xp[M];
        float yp[M];
PBT_UNROLL
        for (int k = 0; k < M; ++k) {
            xm[k] = 0.0;
            x0[k] = X[(size_t)k * plane0];
            yp[k] = 0.f;
        }
        for (int q = 0; q < N; ++q) {
            const size_t o = (size_t)q * rs;
            const size_t plane = opaque(plane0);
            const bool has_next = (q + 1 < N);
PBT_UNROLL
            for (int k = 0; k < M; ++k) xp[k] = has_next ? X[o + rs + (size_t)k * plane] : 0.0;
            double r[M];
            F32::Acc ta[M];
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                double t = __ldg(g.d + sys + o + (size_t)i * plane);
PBT_UNROLL
                for (int k = 0; k < M; ++k) t = fma(-__ldg(g.b + sys + o + (size_t)(i + M * k) * plane), x0[k], t);
                r[i] = t;
            }
            float an[M][M];
            if (q > 0) {
PBT_UNROLL
                for (int i = 0; i < M; ++i)
PBT_UNROLL
                    for (int k = 0; k < M; ++k) {
                        const double a = __ldg(g.a + sys + o + (size_t)(i + M * k) * plane);
                        r[i] = fma(-a, xm[k], r[i]);
                        an[i][k] = FF::split(a).h;
                    }
            }
            if (has_next) {
PBT_UNROLL
                for (int i = 0; i < M; ++i)
PBT_UNROLL
                    for (int k = 0; k < M; ++k)
                        r[i] = fma(-__ldg(g.c + sys + o + (size_t)(i + M * k) * plane), xp[k], r[i]);
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i) ta[i] = F32::acc(FF::split_wide(r[i]).h);
            if (q > 0) {
PBT_UNROLL
                for (int k = 0; k < M; ++k)
PBT_UNROLL
                    for (int i = 0; i < M; ++i) F32::msub(ta[i], an[i][k], yp[k]);
            }
            LU<F32, M> lu;
            {
                const float* lf = ra.lu + ((size_t)q * ngroups + (sys >> 5)) * (size_t)(32 * (M * M + 1)) + (sys & 31);
PBT_UNROLL
                for (int j = 0; j < M; ++j)
PBT_UNROLL
                    for (int i = 0; i < M; ++i) lu.f[i][j] = __ldcs(lf + 32 * (i + M * j));
                lu.piv = __float_as_uint(__ldcs(lf + 32 * M * M));
            }
            lu.swaps = 0;
PBT_UNROLL
            for (int k = 0; k + 1 < M; ++k)
                if (__any_sync(__activemask(), ((lu.piv >> (4 * k)) & 15u) != (unsigned)k)) lu.swaps |= 1u << k;
            lu_solve<F32, M>(lu, ta, yp);
PBT_UNROLL
            for (int i = 0; i < M; ++i) Y[o + (size_t)i * plane] = yp[i];
PBT_UNROLL
            for (int k = 0; k < M; ++k) {
                xm[k] = x0[k];
                x0[k] = xp[k];
            }
        }
        double emax = 0.0, xmax = 0.0;
        float e[M];
        for (int q = N - 1; q >= 0; --q) {
            const size_t o = (size_t)q * rs;
            const size_t plane = opaque(plane0);
            F32::Acc v[M];
PBT_UNROLL
            for (int i = 0; i < M; ++i) v[i] = F32::acc(Y[o + (size_t)i * plane]);
            if (q < N - 1) {
PBT_UNROLL
                for (int i = 0; i < M; ++i)
PBT_UNROLL
                    for (int k = 0; k < M; ++k)
                        F32::msub(v[i], __ldg(reinterpret_cast<const float*>(g.cw) + sys + o + (size_t)(i + M * k) * plane),
                                  e[k]);
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                e[i] = F32::fin(v[i]);
                double* px = X + o + (size_t)i * plane;
                const double ed = FF::widen(e[i]);
                const double x = *px + ed;
                *px = x;
                refine_stat(emax, xmax, ed, x);
            }
        }
        refine_report(emax, xmax, ra.stat, g.status);
    }
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
inline unsigned grid_x(int nsys, int tpb) { return (unsigned)((nsys + tpb - 1) / tpb); }

template <class Num, int M>
cudaError_t launch_thomas(const SolveArgs& g) {
    constexpr bool kStep = thomas_in_step<Num, M>();
    constexpr size_t kSmemThread = thomas_uses_lu<M>() ? (M * M + M) * sizeof(double) : 0;
    static const int regs = kernel_regs(k_thomas<Num, M>);
    const int tpb =
        kStep ? in_step_tpb(g, g.nsys, kSmemThread, regs) : (g.tpb < kThomasThreads ? g.tpb : kThomasThreads);
    const size_t smem = (size_t)tpb * kSmemThread;
    if (smem > 48u * 1024u) {
        const cudaError_t e =
            cudaFuncSetAttribute(k_thomas<Num, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    k_thomas<Num, M><<<grid_x(g.nsys, tpb), tpb, smem, g.stream>>>(g);
    return cudaGetLastError();
}
template <class Num, int M>
cudaError_t launch_thomas_lines(const SolveArgs& g, const LineStrides& ls) {
    if constexpr (std::is_same<Num, F32>::value) {
        return cudaErrorInvalidValue;  // FP64 and float-float plans only
    } else {
        constexpr size_t kSmemThread = thomas_uses_lu<M>() ? (M * M + M) * sizeof(double) : 0;
        static const int regs = kernel_regs(k_thomas_lines<Num, M>);
        const int tpb = thomas_in_step<Num, M>() ? in_step_tpb(g, g.nsys, kSmemThread, regs)
                                                 : (g.tpb < kThomasThreads ? g.tpb : kThomasThreads);
        const size_t smem = (size_t)tpb * kSmemThread;
        if (smem > 48u * 1024u) {
            const cudaError_t e =
                cudaFuncSetAttribute(k_thomas_lines<Num, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        k_thomas_lines<Num, M><<<grid_x(g.nsys, tpb), tpb, smem, g.stream>>>(g, ls);
        return cudaGetLastError();
    }
}
// Block sizes above 6 run 32-thread CTAs (their slots take 0.9-1.7 KB a
// thread); above 48 KB a CTA the kernel opts in to the larger carve-out.
template <class Num, int M>
cudaError_t launch_thomas_cyclic(const SolveArgs& g) {
    if constexpr (std::is_same<Num, F32>::value) {
        return cudaErrorInvalidValue;  // FP64 and float-float plans only
    } else {
        int tpb = g.tpb < kThomasThreads ? g.tpb : kThomasThreads;
        if (M > 6) tpb = 32;
        if (cyclic_in_step<Num, M>()) {
            static const int regs = kernel_regs(k_thomas_cyclic<Num, M>);
            tpb = in_step_tpb(g, g.nsys, cyclic_slots<Num, M>() * sizeof(double), regs);
        }
        const size_t smem = (size_t)tpb * cyclic_slots<Num, M>() * sizeof(double);
        if (smem > 48u * 1024u) {
            const cudaError_t e = cudaFuncSetAttribute(k_thomas_cyclic<Num, M>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        k_thomas_cyclic<Num, M><<<grid_x(g.nsys, tpb), tpb, smem, g.stream>>>(g);
        return cudaGetLastError();
    }
}
template <class Num, int M>
cudaError_t launch_modi(const SolveArgs& g) {
    if constexpr (modi_uses_lu<Num, M>()) {
        constexpr size_t kSmemThread = cyclic_slots<Num, M>() * sizeof(double);
        static const int regs = kernel_regs(k_modi_lu<Num, M>);
        const int tpb = rows_in_step<Num>() ? in_step_tpb(g, (long long)g.nsys * g.nseg, kSmemThread, regs)
                                            : (g.tpb < kThomasThreads ? g.tpb : kThomasThreads);
        const size_t smem = (size_t)tpb * kSmemThread;
        if (smem > 48u * 1024u) {
            const cudaError_t e =
                cudaFuncSetAttribute(k_modi_lu<Num, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        dim3 grid(grid_x(g.nsys, tpb), (unsigned)g.nseg);
        k_modi_lu<Num, M><<<grid, tpb, smem, g.stream>>>(g);
    } else {
        static const int regs = kernel_regs(k_modi<Num, M>);
        const int tpb = modi_in_step<Num, M>() ? in_step_tpb(g, (long long)g.nsys * g.nseg, 0, regs) : g.tpb;
        dim3 grid(grid_x(g.nsys, tpb), (unsigned)g.nseg);
        k_modi<Num, M><<<grid, tpb, 0, g.stream>>>(g);
    }
    return cudaGetLastError();
}
template <class Num, int M>
cudaError_t launch_reduced(const SolveArgs& g) {
    k_reduced<Num, M><<<grid_x(g.nsys, g.tpb), g.tpb, 0, g.stream>>>(g);
    return cudaGetLastError();
}
template <class Num, int M>
cudaError_t launch_reduced_cyclic(const SolveArgs& g) {
    k_reduced_cyclic<Num, M><<<grid_x(g.nsys, g.tpb), g.tpb, 0, g.stream>>>(g);
    return cudaGetLastError();
}
template <class Num, int M>
cudaError_t launch_adjoint(const SolveArgs& g, const AdjointArgs& adj) {
    const int tpb = g.tpb < kThomasThreads ? g.tpb : kThomasThreads;
    k_adjoint<Num, M><<<grid_x(g.nsys, tpb), tpb, 0, g.stream>>>(g, adj);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_transpose_blocks(const SolveArgs& g, double* At, double* Bt, double* Ct) {
    const size_t n = (size_t)g.nsys * g.nrow;
    k_transpose_blocks<M><<<(unsigned)((n + 255) / 256), 256, 0, g.stream>>>(g, At, Bt, Ct);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_gradients(const SolveArgs& g, const AdjointArgs& adj) {
    const size_t n = (size_t)g.nsys * g.nrow;
    k_gradients<M><<<(unsigned)((n + 255) / 256), 256, 0, g.stream>>>(g, adj);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_residual(const SolveArgs& g, const double* X, double* E) {
    k_residual64<M><<<grid_x(g.nsys, 32), dim3(32, M), 0, g.stream>>>(g, X, E);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_refine_step(const SolveArgs& g, const RefineArgs& ra) {
    if (M > kStagedMaxBlock) return cudaErrorInvalidValue;
    k_refine_step<M><<<grid_x(g.nsys, 64), 64, 0, g.stream>>>(g, ra);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_accumulate(const SolveArgs& g, double* X, const double* E, unsigned* stat) {
    k_accumulate<M><<<grid_x(g.nsys, 32), dim3(32, M), 0, g.stream>>>(g, X, E, stat);
    return cudaGetLastError();
}
template <class Num, int M>
cudaError_t launch_update(const SolveArgs& g) {
    dim3 grid(grid_x(g.nsys, g.tpb), (unsigned)g.nseg);
    k_update<Num, M><<<grid, g.tpb, 0, g.stream>>>(g);
    return cudaGetLastError();
}

}  // namespace pbt
