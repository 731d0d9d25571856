// pbt_staged.cuh -- the single-segment block Thomas solve with its inputs
// staged through shared memory by the Tensor Memory Accelerator.
//
// Why: one thread carries one system's whole block row, and a 65536-system
// batch has only 2048 warps -- 13.5 per SM -- so the direct-load kernel
// (k_thomas) waits on global loads it cannot issue early enough (a row's
// inputs are 3m^2 + m doubles, more than its register budget).  Here the
// loads are asynchronous bulk tensor copies (cp.async.bulk.tensor) into a
// ring of shared-memory slots, issued one ring ahead of use, and the
// arithmetic reads shared memory.
//
// Shape: one warp per CTA, one system per lane, 32 consecutive systems per
// CTA.  A ring item is one block COLUMN of one array for the CTA's 32 systems:
// elements (0..m-1, j) of row q, which in the reference layout
// X[sys + nsys*(row + nrow*(i + m*j))] is the 3-D box {32 systems, 1 row,
// m planes} at (s0, q, j*m) of the tensor {nsys, nrow, planes}.  In shared
// memory the box lands as slot[i][lane], so lane l reads its column from
// slot + l + 32*i without bank conflicts.
//
// Item order, forward sweep (row q): d_q, B_q columns 0..m-1, A_q columns,
// C_q columns -- the order the row consumes them: R = B - A C'_{q-1}
// and rhs = d - A y_{q-1} are accumulated column by column of A (C'_{q-1}
// read from shared memory one row at a time), R is factorised (lu_factor), and
// y_q and the columns of C'_q are solved one at a time (lu_solve), each
// C'_q column going to the factor workspace and to shared memory for the
// next row.  A_0 and C_{nrow-1} are fetched and ignored, so every row has the
// same 1 + 3m items.  Backward sweep (row q = nrow-2 .. 0): C'_q columns
// 0..m-1 from the factor workspace, then y_q.  The arithmetic, and so every
// result bit, is that of the direct-load kernel k_thomas.
//
// Ring protocol: R slots, one mbarrier each.  Item n uses slot n % R and
// completes phase (n / R) & 1 of its barrier.  Lane 0 issues item n + R into
// the slot of item n as soon as every lane has read item n (__syncwarp), so
// each copy has R items of arithmetic to land in.  Between the sweeps every
// lane fences its generic-proxy global stores (C'_q, y_q) against the
// async-proxy reads of the backward sweep.  Every wait is bounded (2 s on
// the global timer); a wait that runs out adds kStallMark to the status word,
// stops issuing, waits (bounded) for the copies already in flight and ends
// the CTA.
#pragma once

#include <cuda.h>

#include "pbt_kernels.cuh"

namespace pbt {

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s per wait

static __device__ __noinline__ bool mbar_wait_slow(unsigned bar, unsigned parity, unsigned long long limit_ns) {
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
    return mbar_try_wait(bar, parity) || mbar_wait_slow(bar, parity, kWaitLimitNs);
}
// 3-D tile load of `map` at (x, y, z) into shared memory, completing on `bar`.
// x (the system index) is a multiple of 32, so x * 8 bytes is 16-byte aligned.
__device__ __forceinline__ void tma_load_3d(unsigned dst, const CUtensorMap* map, int x, int y, int z, unsigned bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async_shared() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// Block-column loops kept rolled (see lu_rolled) only where that measured
// faster in this kernel: float-float at m = 4 (GB300, 16384 systems: 4.48
// vs 4.67 ms; 131072: 14.7 vs 15.9 ms).  At m = 3, 5, 6, and for the
// smaller FP32 code at m = 4 (11.6 vs 10.4 ms), the runtime item bookkeeping
// of a rolled loop costs more than the smaller code saves.
template <class Num, int M>
__host__ __device__ constexpr bool staged_rolled() {
    return lu_rolled<Num>() && sizeof(typename Num::T) == 8 && M == 4;
}
// Shared memory of one CTA: the ring (R items of M*32 doubles), C'_{q-1}
// (M*M*32 raw values) and, with rolled loops, y_{q-1} (M*32).  Sized so that
// 14 one-warp CTAs fit in an SM (14 * (15.06 KB + 1 KB reserved) <= 228 KB):
// 14 * 152 = 2128 resident warps cover a 65536-system batch (2048 warps) in
// one wave, with a 6-item ring at m = 5.
constexpr int kStagedSmemBudget = 15424;
template <class Num, int M>
__host__ __device__ constexpr int staged_fixed_slots() {
    return M * M + (staged_rolled<Num, M>() ? M : 0);
}
template <class Num, int M>
__host__ __device__ constexpr int staged_ring() {
    return (kStagedSmemBudget - staged_fixed_slots<Num, M>() * 256) / (M * 256 + 8) < 4 ? 4
           : (kStagedSmemBudget - staged_fixed_slots<Num, M>() * 256) / (M * 256 + 8) > 3 * (1 + 3 * M)
               ? 3 * (1 + 3 * M)
               : (kStagedSmemBudget - staged_fixed_slots<Num, M>() * 256) / (M * 256 + 8);
}
template <class Num, int M>
__host__ __device__ constexpr int staged_smem_bytes() {
    return (staged_ring<Num, M>() * M + staged_fixed_slots<Num, M>()) * 32 * 8;
}

// Forward item k of a row: which array and which plane offset.  Items: d_q,
// the B columns, the A columns, then the C columns.
template <class Num, int M>
__device__ __forceinline__ const CUtensorMap* fwd_item(const ThomasMaps& mp, int k, int& z) {
    if (k == 0) {
        z = 0;
        return &mp.d;
    }
    if (k <= M) {
        z = (k - 1) * M;
        return &mp.b;
    }
    if (k <= 2 * M) {
        z = (k - 1 - M) * M;
        return &mp.a;
    }
    z = (k - 1 - 2 * M) * M;
    return &mp.c;
}
// Backward item k of a row: C'_q column k (k < M) or y_q (k == M).
template <int M>
__device__ __forceinline__ const CUtensorMap* bwd_item(const ThomasMaps& mp, int k, int& z) {
    if (k < M) {
        z = k * M;
        return &mp.w;
    }
    z = 0;
    return &mp.d;
}

template <class Num>
__device__ __forceinline__ typename Num::T fac_in(const double* p, bool raw) {
    return (raw || !Num::kConv) ? Num::lds(p) : Num::in(p);
}

// Resident one-warp CTAs per SM the register budget is sized for (16: at most
// 128 registers a thread; shared memory allows 15).
#ifndef PBT_STAGED_MIN_CTAS
#define PBT_STAGED_MIN_CTAS 16
#endif

// FP32 (the refined solve's first pass) keeps its factors where the plan
// provides g.aw.
template <class Num, int M>
constexpr bool kKeepLU = std::is_same<Num, F32>::value && !staged_rolled<Num, M>();

template <class Num, int M>
__global__ void __launch_bounds__(32, PBT_STAGED_MIN_CTAS) k_thomas_staged(const __grid_constant__ ThomasMaps maps, const SolveArgs g) {
    using T = typename Num::T;
    using Acc = typename Num::Acc;
    constexpr int R = staged_ring<Num, M>();
    constexpr int K = 1 + 3 * M;  // forward items per row
    constexpr int K2 = M + 1;     // backward items per row
    constexpr unsigned kSlotBytes = M * 32 * 8;
    extern __shared__ __align__(128) double ring[];
    __shared__ __align__(8) unsigned long long bars[R];

    const int lane = threadIdx.x;
    const int s0 = blockIdx.x * 32;
    const bool active = s0 + lane < g.nsys;
    const int N = g.nrow;
    const size_t plane0 = (size_t)g.nsys * N;
    const bool raw = g.factors_raw != 0;
    const unsigned ring_s = smem_u32(ring), bar_s = smem_u32(bars);
    double* const D = g.d + s0 + lane;
    double* const CW = g.cw + s0 + lane;

    if (lane == 0) {
        for (int j = 0; j < R; ++j) mbar_init(bar_s + 8u * j, 1);
        fence_mbar_init();
    }
    __syncwarp();

    // Consumer position: the next item's slot and barrier phase, and how many
    // items of the whole sequence (forward, then backward) were consumed.
    int slot = 0;
    unsigned phase = 0;
    int n_cons = 0;
    bool ok = true;

    // FP32 keeps C' as floats (its map is FLOAT32): those items are half a slot.
    constexpr bool kFloatCW = std::is_same<Num, F32>::value;
    auto issue = [&](int s, const CUtensorMap* map, int row, int z) {
        const unsigned bytes = (kFloatCW && map == &maps.w) ? kSlotBytes / 2 : kSlotBytes;
        mbar_expect_tx(bar_s + 8u * s, bytes);
        tma_load_3d(ring_s + kSlotBytes * s, map, s0, row, z, bar_s + 8u * s);
    };
    auto take = [&]() -> const double* {
        if (ok) ok = __all_sync(0xffffffffu, mbar_wait(bar_s + 8u * slot, phase));
        return ring + slot * (M * 32) + lane;
    };
    // Release the current item and refill its slot with the item R later
    // (map == nullptr: the sequence of this sweep has ended).
    auto give = [&](const CUtensorMap* map, int row, int z) {
        if (!ok) return;
        __syncwarp();
        if (lane == 0 && map != nullptr) {
            fence_proxy_async_shared();
            issue(slot, map, row, z);
        }
        ++n_cons;
        if (++slot == R) {
            slot = 0;
            phase ^= 1u;
        }
    };
    // Item R positions after item k of forward row q.
    auto fwd_next = [&](int q, int k, int& row, int& z) -> const CUtensorMap* {
        const int kk = k + R;
        row = q + kk / K;
        return row < N ? fwd_item<Num, M>(maps, kk % K, z) : nullptr;
    };
    auto bwd_next = [&](int b, int k, int& row, int& z) -> const CUtensorMap* {
        const int kk = k + R;
        const int bb = b + kk / K2;
        row = N - 2 - bb;
        return bb < N - 1 ? bwd_item<M>(maps, kk % K2, z) : nullptr;
    };

    if (lane == 0) {
        for (int j = 0; j < R && j < N * K; ++j) {
            int z;
            const CUtensorMap* mp = fwd_item<Num, M>(maps, j % K, z);
            issue(j, mp, j / K, z);
        }
    }

    unsigned bad = 0, amax = 0;
    T y[M];
    // This lane's C'_{q-1}: (k, j) at cps[32 * (k*M + j)]; y_{q-1}[k] at cps[32 * (M*M + k)].
    double* const cps = ring + R * M * 32 + lane;
    for (int q = 0; q < N; ++q) {
        const size_t o = (size_t)q * g.nsys;
        const bool last = (q == N - 1);
        Acc r[M][M], xd[M];
        int nrow_, nz;
        {
            const double* p = take();
PBT_UNROLL
            for (int i = 0; i < M; ++i) xd[i] = Num::acc(Num::in_rhs(p + 32 * i));
            if constexpr (kKeepLU<Num, M>) {
                // The refined solve's first pass keeps the right-hand side
                // (in g.ra) as it streams by: D is solved in place.
                if (g.ra != nullptr && active && ok) {
PBT_UNROLL
                    for (int i = 0; i < M; ++i) g.ra[(size_t)(s0 + lane) + o + plane0 * (size_t)i] = p[32 * i];
                }
            }
            const CUtensorMap* nm = fwd_next(q, 0, nrow_, nz);
            give(nm, nrow_, nz);
        }
        // Items 1..2M: the A and B columns in the order fwd_item gives.
        auto a_cols = [&](int k0) {
#pragma unroll(staged_rolled<Num, M>() ? 1 : M)
            for (int k = 0; k < M; ++k) {
                const double* p = take();
                if (q > 0) {
                    T ck[M];
PBT_UNROLL
                    for (int j = 0; j < M; ++j) ck[j] = Num::lds(cps + 32 * (k * M + j));
                    T yk;
                    if constexpr (staged_rolled<Num, M>())
                        yk = Num::lds(cps + 32 * (M * M + k));
                    else
                        yk = y[k];
PBT_UNROLL
                    for (int i = 0; i < M; ++i) {
                        const T a = Num::in(p + 32 * i);
PBT_UNROLL
                        for (int j = 0; j < M; ++j) Num::msub(r[i][j], a, ck[j]);
                        Num::msub(xd[i], a, yk);
                    }
                }
                const CUtensorMap* nm = fwd_next(q, k0 + k, nrow_, nz);
                give(nm, nrow_, nz);
            }
        };
        auto b_cols = [&](int k0) {
PBT_UNROLL
            for (int j = 0; j < M; ++j) {
                const double* p = take();
PBT_UNROLL
                for (int i = 0; i < M; ++i) r[i][j] = Num::acc(Num::in(p + 32 * i));
                const CUtensorMap* nm = fwd_next(q, k0 + j, nrow_, nz);
                give(nm, nrow_, nz);
            }
        };
        b_cols(1);
        a_cols(1 + M);
        LU<Num, M> lu;
        lu_factor<Num, M>(r, lu, bad);
        if constexpr (kKeepLU<Num, M>) {
            // The refined solve's first pass keeps the FP32 factors of R_q for
            // its corrections (k_refine_step), as floats in aw, tiled by warp:
            // for row q and this CTA's 32 systems, (M*M + 1) runs of 32 floats
            // (factor (i, j) in run i + M*j, the pivot code in run M*M), so a
            // warp writes 4*32*(M*M + 1) contiguous bytes a row, streaming
            // (evict-first: they are read once, a whole sweep later).
            if (g.aw != nullptr && active && ok) {
                float* lf = reinterpret_cast<float*>(g.aw) +
                            ((size_t)q * gridDim.x + blockIdx.x) * (size_t)(32 * (M * M + 1)) + lane;
PBT_UNROLL
                for (int j = 0; j < M; ++j)
PBT_UNROLL
                    for (int i = 0; i < M; ++i) __stcs(lf + 32 * (i + M * j), lu.f[i][j]);
                __stcs(lf + 32 * M * M, __uint_as_float(lu.piv));
            }
        }
        lu_solve<Num, M>(lu, xd, y);
        if constexpr (staged_rolled<Num, M>()) {
PBT_UNROLL
            for (int k = 0; k < M; ++k) Num::sts(cps + 32 * (M * M + k), y[k]);
        }
        {
            const size_t plane = opaque(plane0);
            if (!last) {
                if (active && ok) st_raw_vec<Num, M>(D + o, plane, y);
            } else {
                if (active && ok) out_vec<Num, M>(D + o, plane, y, amax);
            }
        }
        const size_t plane = opaque(plane0);
        double* pw = CW + o;
#pragma unroll(staged_rolled<Num, M>() ? 1 : M)
        for (int j = 0; j < M; ++j) {
            const double* p = take();
            if (!last) {
                Acc cj[M];
                T xj[M];
PBT_UNROLL
                for (int i = 0; i < M; ++i) cj[i] = Num::acc(Num::in(p + 32 * i));
                lu_solve<Num, M>(lu, cj, xj);
PBT_UNROLL
                for (int i = 0; i < M; ++i, pw += plane) {
                    if (active && ok) {
                        if constexpr (kFloatCW) {
                            reinterpret_cast<float*>(g.cw)[(size_t)(s0 + lane) + o + plane0 * (size_t)(i + M * j)] =
                                xj[i];
                        } else if (raw || !Num::kConv) {
                            Num::sts(pw, xj[i]);
                        } else {
                            Num::out(pw, xj[i]);
                        }
                    }
                    Num::sts(cps + 32 * (i * M + j), xj[i]);
                }
            }
            const CUtensorMap* nm = fwd_next(q, 1 + 2 * M + j, nrow_, nz);
            give(nm, nrow_, nz);
        }
        if (!ok) break;
    }

    int n_end = N * K;  // end of the sweep in progress (items)
    if (ok) {
        // The backward sweep reads, through the async proxy, what this warp's
        // lanes just stored through the generic proxy.
        fence_proxy_async_global();
        __syncwarp();
        n_end = N * K + (N - 1) * K2;
        if (lane == 0) {
            for (int j = 0; j < R && j < (N - 1) * K2; ++j) {
                int z;
                const CUtensorMap* mp = bwd_item<M>(maps, j % K2, z);
                const int s = (slot + j) % R;
                issue(s, mp, N - 2 - j / K2, z);
            }
        }
        for (int b = 0; b < N - 1; ++b) {
            const int q = N - 2 - b;
            const size_t o = (size_t)q * g.nsys;
            T c[M][M], t[M];
            int nrow_, nz;
PBT_UNROLL
            for (int k = 0; k < M; ++k) {
                const double* p = take();
                if constexpr (kFloatCW) {
                    const float* pf = reinterpret_cast<const float*>(p - lane) + lane;
PBT_UNROLL
                    for (int i = 0; i < M; ++i) c[i][k] = pf[32 * i];
                } else {
PBT_UNROLL
                    for (int i = 0; i < M; ++i) c[i][k] = fac_in<Num>(p + 32 * i, raw);
                }
                const CUtensorMap* nm = bwd_next(b, k, nrow_, nz);
                give(nm, nrow_, nz);
            }
            {
                const double* p = take();
PBT_UNROLL
                for (int i = 0; i < M; ++i) t[i] = Num::lds(p + 32 * i);
                const CUtensorMap* nm = bwd_next(b, M, nrow_, nz);
                give(nm, nrow_, nz);
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                Acc s = Num::acc(t[i]);
PBT_UNROLL
                for (int k = 0; k < M; ++k) Num::msub(s, c[i][k], y[k]);
                t[i] = Num::fin(s);
            }
PBT_UNROLL
            for (int i = 0; i < M; ++i) y[i] = t[i];
            if (active && ok) out_vec<Num, M>(D + o, plane0, y, amax);
            if (!ok) break;
        }
    }

    if (!ok) {
        // A wait ran out: report it, then wait (boundedly) for the copies
        // still in flight -- items n_cons .. n_cons+R-1 of the current sweep --
        // so none lands in shared memory after the CTA has ended.
        if (lane == 0) {
            atomicAdd(g.status, kStallMark);
            int s = slot;
            unsigned ph = phase;
            for (int j = 0; j < R && n_cons + j < n_end; ++j) {
                if (!mbar_try_wait(bar_s + 8u * s, ph)) mbar_wait_slow(bar_s + 8u * s, ph, kWaitLimitNs / 4);
                if (++s == R) {
                    s = 0;
                    ph ^= 1u;
                }
            }
        }
        __syncwarp();
        return;
    }
    if (active) report_status(g.status, bad | range_bits<Num>(amax, true));
}

// ---------------------------------------------------------------------------
// k_refine_staged: one correction of the refined solve (the work of
// k_refine_step, the same operations in the same order, so the same bits)
// with the forward sweep's FP64 inputs -- d (here the kept right-hand side),
// the B, A and C columns, 1 + 3m items a row in that order -- staged through
// a TMA ring as in k_thomas_staged.  Nothing else lives in shared memory, so
// the ring is longer.  The factors, x and the backward sweep's C' and y use
// plain loads (a fifth of the traffic).
template <int M>
__host__ __device__ constexpr int refine_ring() {
    return kStagedSmemBudget / (M * 256 + 8) > 3 * (1 + 3 * M) ? 3 * (1 + 3 * M) : kStagedSmemBudget / (M * 256 + 8);
}

template <int M>
__global__ void __launch_bounds__(32, PBT_STAGED_MIN_CTAS)
    k_refine_staged(const __grid_constant__ ThomasMaps maps, const SolveArgs g, const RefineArgs ra) {
    constexpr int R = refine_ring<M>();
    constexpr int K = 1 + 3 * M;  // items a row
    constexpr unsigned kSlotBytes = M * 32 * 8;
    extern __shared__ __align__(128) double ring[];
    __shared__ __align__(8) unsigned long long bars[R];

    const int lane = threadIdx.x;
    const int s0 = blockIdx.x * 32;
    const int sys = s0 + lane;
    const bool active = sys < g.nsys;
    const int N = g.nrow;
    const size_t plane0 = (size_t)g.nsys * N;
    const size_t rs = (size_t)g.nsys;
    const size_t ngroups = ((size_t)g.nsys + 31) / 32;
    const unsigned ring_s = smem_u32(ring), bar_s = smem_u32(bars);
    const float* const C32 = reinterpret_cast<const float*>(g.cw);

    if (lane == 0) {
        for (int j = 0; j < R; ++j) mbar_init(bar_s + 8u * j, 1);
        fence_mbar_init();
    }
    __syncwarp();

    int slot = 0;
    unsigned phase = 0;
    int n_cons = 0;
    bool ok = true;
    const int n_end = N * K;
    auto issue = [&](int s, const CUtensorMap* map, int row, int z) {
        mbar_expect_tx(bar_s + 8u * s, kSlotBytes);
        tma_load_3d(ring_s + kSlotBytes * s, map, s0, row, z, bar_s + 8u * s);
    };
    auto take = [&]() -> const double* {
        if (ok) ok = __all_sync(0xffffffffu, mbar_wait(bar_s + 8u * slot, phase));
        return ring + slot * (M * 32) + lane;
    };
    // Release the current item (item n_cons) and refill its slot with item
    // n_cons + R, if the sweep has one.
    auto give = [&]() {
        if (!ok) return;
        __syncwarp();
        const int nn = n_cons + R;
        if (lane == 0 && nn < n_end) {
            int z;
            const CUtensorMap* mp = fwd_item<F64, M>(maps, nn % K, z);
            fence_proxy_async_shared();
            issue(slot, mp, nn / K, z);
        }
        ++n_cons;
        if (++slot == R) {
            slot = 0;
            phase ^= 1u;
        }
    };
    if (lane == 0) {
        for (int j = 0; j < R && j < n_end; ++j) {
            int z;
            const CUtensorMap* mp = fwd_item<F64, M>(maps, j % K, z);
            issue(j, mp, j / K, z);
        }
    }

    double xm[M], x0[M], xp[M];
    float y[M];
PBT_UNROLL
    for (int k = 0; k < M; ++k) {
        xm[k] = 0.0;
        x0[k] = active ? ra.x[sys + (size_t)k * plane0] : 0.0;
        y[k] = 0.f;
    }
    for (int q = 0; q < N; ++q) {
        const size_t o = (size_t)q * rs + sys;
        const size_t plane = opaque(plane0);
        const bool has_next = (q + 1 < N);
PBT_UNROLL
        for (int k = 0; k < M; ++k) xp[k] = (has_next && active) ? ra.x[o + rs + (size_t)k * plane] : 0.0;
        double r[M];
        float an[M][M];
        {
            const double* p = take();
PBT_UNROLL
            for (int i = 0; i < M; ++i) r[i] = p[32 * i];
            give();
        }
PBT_UNROLL
        for (int k = 0; k < M; ++k) {
            const double* p = take();
PBT_UNROLL
            for (int i = 0; i < M; ++i) r[i] = fma(-p[32 * i], x0[k], r[i]);
            give();
        }
PBT_UNROLL
        for (int k = 0; k < M; ++k) {
            const double* p = take();
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                const double a = p[32 * i];
                if (q > 0) r[i] = fma(-a, xm[k], r[i]);
                an[i][k] = FF::split(a).h;
            }
            give();
        }
PBT_UNROLL
        for (int k = 0; k < M; ++k) {
            const double* p = take();
            if (has_next) {
PBT_UNROLL
                for (int i = 0; i < M; ++i) r[i] = fma(-p[32 * i], xp[k], r[i]);
            }
            give();
        }
        if (!ok) break;
        F32::Acc ta[M];
PBT_UNROLL
        for (int i = 0; i < M; ++i) ta[i] = F32::acc(FF::split_wide(r[i]).h);
        if (q > 0) {
PBT_UNROLL
            for (int k = 0; k < M; ++k)
PBT_UNROLL
                for (int i = 0; i < M; ++i) F32::msub(ta[i], an[i][k], y[k]);
        }
        LU<F32, M> lu;
        if (active) {
            const float* lf = ra.lu + ((size_t)q * ngroups + blockIdx.x) * (size_t)(32 * (M * M + 1)) + lane;
PBT_UNROLL
            for (int j = 0; j < M; ++j)
PBT_UNROLL
                for (int i = 0; i < M; ++i) lu.f[i][j] = __ldcs(lf + 32 * (i + M * j));
            lu.piv = __float_as_uint(__ldcs(lf + 32 * M * M));
        } else {
PBT_UNROLL
            for (int j = 0; j < M; ++j)
PBT_UNROLL
                for (int i = 0; i < M; ++i) lu.f[i][j] = (i == j) ? 1.f : 0.f;
            lu.piv = 0;
PBT_UNROLL
            for (int k = 0; k + 1 < M; ++k) lu.piv |= (unsigned)k << (4 * k);
        }
        lu.swaps = 0;
PBT_UNROLL
        for (int k = 0; k + 1 < M; ++k)
            if (__any_sync(0xffffffffu, ((lu.piv >> (4 * k)) & 15u) != (unsigned)k)) lu.swaps |= 1u << k;
        lu_solve<F32, M>(lu, ta, y);
        if (active) {
PBT_UNROLL
            for (int i = 0; i < M; ++i) ra.y[o + (size_t)i * plane] = y[i];
        }
PBT_UNROLL
        for (int k = 0; k < M; ++k) {
            xm[k] = x0[k];
            x0[k] = xp[k];
        }
    }

    if (!ok) {
        // A wait ran out: report it, then wait (boundedly) for the copies
        // still in flight so none lands in shared memory after the CTA ends.
        if (lane == 0) {
            atomicAdd(g.status, kStallMark);
            int s = slot;
            unsigned ph = phase;
            for (int j = 0; j < R && n_cons + j < n_end; ++j) {
                if (!mbar_try_wait(bar_s + 8u * s, ph)) mbar_wait_slow(bar_s + 8u * s, ph, kWaitLimitNs / 4);
                if (++s == R) {
                    s = 0;
                    ph ^= 1u;
                }
            }
        }
        __syncwarp();
        return;
    }
    if (!active) return;
    double emax = 0.0, xmax = 0.0;
    float e[M];
    // Backward, on plain loads: row q's C' and y are loaded while row q+1
    // finishes (the forward sweep's registers are free by now).
    float cn[M][M], yn[M];
PBT_UNROLL
    for (int i = 0; i < M; ++i)
PBT_UNROLL
        for (int k = 0; k < M; ++k) cn[i][k] = 0.f;
    {
        const size_t o = (size_t)(N - 1) * rs + sys;
PBT_UNROLL
        for (int i = 0; i < M; ++i) yn[i] = ra.y[o + (size_t)i * plane0];
    }
    for (int q = N - 1; q >= 0; --q) {
        const size_t o = (size_t)q * rs + sys;
        const size_t plane = opaque(plane0);
        float cq[M][M], yq[M];
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            yq[i] = yn[i];
PBT_UNROLL
            for (int k = 0; k < M; ++k) cq[i][k] = cn[i][k];
        }
        if (q > 0) {
            const size_t op = o - rs;
PBT_UNROLL
            for (int i = 0; i < M; ++i) {
                yn[i] = ra.y[op + (size_t)i * plane];
PBT_UNROLL
                for (int k = 0; k < M; ++k) cn[i][k] = __ldg(C32 + op + (size_t)(i + M * k) * plane);
            }
        }
        F32::Acc v[M];
PBT_UNROLL
        for (int i = 0; i < M; ++i) v[i] = F32::acc(yq[i]);
        if (q < N - 1) {
PBT_UNROLL
            for (int i = 0; i < M; ++i)
PBT_UNROLL
                for (int k = 0; k < M; ++k) F32::msub(v[i], cq[i][k], e[k]);
        }
PBT_UNROLL
        for (int i = 0; i < M; ++i) {
            e[i] = F32::fin(v[i]);
            double* px = ra.x + o + (size_t)i * plane;
            const double ed = FF::widen(e[i]);
            const double x = *px + ed;
            *px = x;
            refine_stat(emax, xmax, ed, x);
        }
    }
    refine_report(emax, xmax, ra.stat, g.status);
}

template <int M>
cudaError_t launch_refine_staged(const SolveArgs& g, const ThomasMaps& maps, const RefineArgs& ra) {
    if (M > kStagedMaxBlock) return cudaErrorNotSupported;
    constexpr int smem = refine_ring<M>() * M * 32 * 8;
    static bool configured = false;  // per instantiation; idempotent, so a race is harmless
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_refine_staged<M>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    const unsigned grid = (unsigned)((g.nsys + 31) / 32);
    k_refine_staged<M><<<grid, 32, smem, g.stream>>>(maps, g, ra);
    return cudaGetLastError();
}

template <class Num, int M>
cudaError_t launch_thomas_staged(const SolveArgs& g, const ThomasMaps& maps) {
    if (M > kStagedMaxBlock) return cudaErrorNotSupported;
    constexpr int smem = staged_smem_bytes<Num, M>();
    static bool configured = false;  // per instantiation; idempotent, so a race is harmless
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(k_thomas_staged<Num, M>,
                                             cudaFuncAttributePreferredSharedMemoryCarveout,
                                             cudaSharedmemCarveoutMaxShared);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    const unsigned grid = (unsigned)((g.nsys + 31) / 32);
    k_thomas_staged<Num, M><<<grid, 32, smem, g.stream>>>(maps, g);
    return cudaGetLastError();
}

}  // namespace pbt
