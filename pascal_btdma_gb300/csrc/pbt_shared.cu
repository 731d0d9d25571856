// pbt_shared.cu -- include/pbt_shared.h: lines that share one matrix, solved
// in place in a strided field.
//
// The block Thomas recurrence of a shared matrix does not depend on the right
// hand side, so it is factorised once, on the host, in FP64:
//   R_0 = B_0,  R_q = B_q - A_q C'_{q-1},  C'_q = R_q^{-1} C_q,
// each R_q by Gaussian elimination with partial pivoting (first row of
// maximal |a|, the LAPACK idamax rule of the reference CPU path's dgesv,
// Fortran_Original/src/mod_btdma_cpu.f90:339-421), kept as the row swapped in
// at each step, the multipliers, the U rows and 1/U_kk.  A line's solve is
// then  y_q = R_q^{-1}(d_q - A_q y_{q-1}),  x_q = y_q - C'_q x_{q+1}:
// about 3*m^2 multiply-adds a row, every line reading the same factors (a
// broadcast from L1/L2) and only its own right-hand side and solution.  At
// m = 2 that is 12 FMAs a row against 64 bytes of traffic, over the FP64
// pipe's balance point on GB300 (626 G FMA/s against 6.7 TB/s), so the
// solve also runs in float-float arithmetic on the FP32 pipes (PBT_PREC_FF:
// factors stored as (h, l) float pairs, right-hand sides split on load, y
// kept as raw pairs in x between the sweeps, x joined back to FP64).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/pbt_shared.h"
#include "pbt_internal.h"
#include "pbt_num.cuh"

struct pbt_shared {
    int m = 0, nrow = 0, precision = PBT_PREC_FP64;
    double* fac = nullptr;        // per row q: A_q, the factors of R_q, C'_q (3*m*m 8-byte slots, element (i,j) at
                                  // i + m*j): FP64 values, or float-float pairs (h, l) for PBT_PREC_FF
    long long* piv = nullptr;     // per row q: 4 bits per elimination step, the row swapped in
    unsigned long long* status = nullptr;  // range failures of float-float solves (pbt_internal.h layout)
    unsigned magic = 0x50425453u;  // "PBTS"
};

namespace {

constexpr unsigned kSharedMagic = 0x50425453u;
constexpr int kSharedWarps = 4;
constexpr int kSharedThreads = 32 * kSharedWarps;

// A warp owns 32 consecutive lines and walks them in chunks of K block rows
// (K*M <= 16 doubles, 128 bytes of a line).  A chunk is staged in shared
// memory, [line][K*M] with an odd row stride S (no bank conflicts), by
// coalesced loads whatever the layout:
//   contiguous lines (elem_stride 1, row_stride M: the sweep along the fast
//     axis): each half-warp reads one line's chunk, 128 contiguous bytes;
//   otherwise: lane = line, one load per element of the chunk, 32 lines
//     side by side (256 contiguous bytes when stride_inner is 1).
// Each lane then runs its own line's recurrence on the tile and the tile is
// written back the same way.  The forward sweep leaves y in x; the last chunk
// turns around in shared memory, and the backward sweep reloads the other
// chunks last to first.  Latency is hidden by warps, not by prefetching in a
// warp: registers are capped so that as many blocks fit on an SM as the
// arithmetic allows without spills (shared_min_blocks).
template <int M>
struct SharedTile {
    static constexpr int K = 16 / M > 0 ? 16 / M : 1;
    static constexpr int KM = K * M;
    static constexpr int S = KM | 1;
};

// Blocks an SM must hold (the register cap), as many as fit without spills.
template <class Num, int M>
__host__ __device__ constexpr int shared_min_blocks() {
    return Num::kConv ? (M <= 2 ? 8 : M <= 4 ? 6 : 4) : (M <= 4 ? 5 : 4);
}

// Chunk moves.  fetch() issues a chunk's loads into registers (v: up to 16
// doubles a lane), deposit() puts them in the tile, store() writes the tile
// out; a lane's loads all go out before anything waits on them.
template <int M>
__device__ __forceinline__ void fetch(const double* src, double* v, long long base, bool live, int nlive, int q0, int kk,
                                      const pbt_lines& L, bool contiguous) {
    constexpr int K = SharedTile<M>::K;
    static_assert(SharedTile<M>::KM <= 16, "a chunk is at most 16 doubles of a line");
    const int lane = threadIdx.x & 31;
    if (contiguous) {
        const int len = kk * M, half = lane >> 4, e = lane & 15;
#pragma unroll
        for (int it = 0; it < 16; ++it) {
            const int j = 2 * it + half;
            const long long bj = __shfl_sync(0xffffffffu, base, j) + (long long)q0 * M + e;
            v[it] = (j < nlive && e < len) ? src[bj] : 0.0;
        }
    } else if (live) {
#pragma unroll
        for (int u = 0; u < K; ++u) {
            if (u < kk) {
                const long long r = base + (long long)(q0 + u) * L.row_stride;
#pragma unroll
                for (int i = 0; i < M; ++i) v[u * M + i] = src[r + i * L.elem_stride];
            }
        }
    }
}

template <int M>
__device__ __forceinline__ void deposit(const double* v, double* tile, bool live, int nlive, int kk, bool contiguous) {
    constexpr int K = SharedTile<M>::K, S = SharedTile<M>::S;
    const int lane = threadIdx.x & 31;
    if (contiguous) {
        const int len = kk * M, half = lane >> 4, e = lane & 15;
#pragma unroll
        for (int it = 0; it < 16; ++it) {
            const int j = 2 * it + half;
            if (j < nlive && e < len) tile[j * S + e] = v[it];
        }
    } else if (live) {
        double* my = tile + lane * S;
#pragma unroll
        for (int u = 0; u < K; ++u)
            if (u < kk)
#pragma unroll
                for (int i = 0; i < M; ++i) my[u * M + i] = v[u * M + i];
    }
    __syncwarp();
}

template <int M>
__device__ __forceinline__ void store(double* dst, const double* tile, long long base, bool live, int nlive, int q0,
                                      int kk, const pbt_lines& L, bool contiguous) {
    constexpr int K = SharedTile<M>::K, S = SharedTile<M>::S;
    const int lane = threadIdx.x & 31;
    __syncwarp();
    if (contiguous) {
        const int len = kk * M, half = lane >> 4, e = lane & 15;
#pragma unroll
        for (int it = 0; it < 16; ++it) {
            const int j = 2 * it + half;
            const long long bj = __shfl_sync(0xffffffffu, base, j) + (long long)q0 * M + e;
            if (j < nlive && e < len) dst[bj] = tile[j * S + e];
        }
    } else if (live) {
        const double* my = tile + lane * S;
#pragma unroll
        for (int u = 0; u < K; ++u) {
            if (u < kk) {
                const long long r = base + (long long)(q0 + u) * L.row_stride;
#pragma unroll
                for (int i = 0; i < M; ++i) dst[r + i * L.elem_stride] = my[u * M + i];
            }
        }
    }
    __syncwarp();
}

// One stored factor (an 8-byte slot of the factor array) in arithmetic Num.
template <class Num>
__device__ __forceinline__ typename Num::T ldf(const double* p);
template <>
__device__ __forceinline__ double ldf<pbt::F64>(const double* p) {
    return __ldg(p);
}
template <>
__device__ __forceinline__ pbt::ff ldf<pbt::FF>(const double* p) {
    const float2 f = __ldg(reinterpret_cast<const float2*>(p));
    return {f.x, f.y};
}

// y = R_q^{-1} (t - A_q y_prev) with the stored factors of R_q (t in, y out).
template <class Num, int M>
__device__ __forceinline__ void forward_row(const double* __restrict__ fac, const long long* __restrict__ pivs, int q,
                                            typename Num::T* t, typename Num::T* y) {
    using T = typename Num::T;
    const double* Aq = fac + (size_t)q * 3 * M * M;
    const double* F = Aq + M * M;
    const long long pq = __ldg(pivs + q);
    if (q > 0) {
#pragma unroll
        for (int i = 0; i < M; ++i) {
            typename Num::Acc a = Num::acc(t[i]);
#pragma unroll
            for (int k = 0; k < M; ++k) Num::msub(a, ldf<Num>(Aq + i + M * k), y[k]);
            t[i] = Num::fin(a);
        }
    }
    // Replay the elimination of R_q on t, then back-substitute.
#pragma unroll
    for (int k = 0; k < M; ++k) {
        if (k + 1 < M) {
            const int p = (int)((pq >> (4 * k)) & 15);
#pragma unroll
            for (int i = k + 1; i < M; ++i) {
                const unsigned sw = (p == i);
                const T a = t[k], b = t[i];
                t[k] = Num::sel(sw, b, a);
                t[i] = Num::sel(sw, a, b);
            }
        }
#pragma unroll
        for (int i = k + 1; i < M; ++i) {
            typename Num::Acc a = Num::acc(t[i]);
            Num::msub(a, ldf<Num>(F + i + M * k), t[k]);
            t[i] = Num::fin(a);
        }
    }
#pragma unroll
    for (int k = M - 1; k >= 0; --k) {
        const T xk = Num::mul(t[k], ldf<Num>(F + k + M * k));
        y[k] = xk;
#pragma unroll
        for (int i = 0; i < k; ++i) {
            typename Num::Acc a = Num::acc(t[i]);
            Num::msub(a, ldf<Num>(F + i + M * k), xk);
            t[i] = Num::fin(a);
        }
    }
}

// x_q = y_q - C'_q x_{q+1}: t holds y_q in, x is x_{q+1} in and x_q out.
template <class Num, int M>
__device__ __forceinline__ void backward_row(const double* __restrict__ fac, int q, const typename Num::T* t,
                                             typename Num::T* x) {
    const double* Cq = fac + (size_t)q * 3 * M * M + 2 * M * M;
    typename Num::T v[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
        typename Num::Acc a = Num::acc(t[i]);
#pragma unroll
        for (int k = 0; k < M; ++k) Num::msub(a, ldf<Num>(Cq + i + M * k), x[k]);
        v[i] = Num::fin(a);
    }
#pragma unroll
    for (int i = 0; i < M; ++i) x[i] = v[i];
}

// The tile holds FP64 right-hand sides on the way in, raw y values (Num's
// 8-byte workspace form) between the sweeps and FP64 solutions on the way out.
template <class Num, int M>
__global__ void __launch_bounds__(kSharedThreads, (shared_min_blocks<Num, M>())) k_shared(const double* __restrict__ fac,
                                                           const long long* __restrict__ pivs,
                                                           const double* rhs, double* x, int nrow, pbt_lines L,
                                                           int contiguous, unsigned long long* status) {
    using T = typename Num::T;
    constexpr int K = SharedTile<M>::K, S = SharedTile<M>::S;
    __shared__ double tiles[kSharedWarps][32 * S];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long nsys = (long long)L.nsys_inner * L.nsys_outer;
    const long long s0 = ((long long)blockIdx.x * kSharedWarps + w) * 32;
    if (s0 >= nsys) return;  // the whole warp
    double* tile = tiles[w];
    double* my = tile + lane * S;
    const long long s = s0 + lane;
    const bool live = s < nsys;
    const int nlive = (int)(nsys - s0 < 32 ? nsys - s0 : 32);
    long long base = 0;
    if (live) base = (s % L.nsys_inner) * L.stride_inner + (s / L.nsys_inner) * L.stride_outer;
    const bool cont = contiguous != 0;
    const int nchunk = (nrow + K - 1) / K;
    // Steps 0..nchunk-1: forward chunks first to last; then the backward
    // sweep over chunks nchunk-2 down to 0 (the last chunk turns around in
    // the tile).
    const int nsteps = 2 * nchunk - 1;
    T y[M];
#pragma unroll
    for (int i = 0; i < M; ++i) y[i] = Num::zero();
    unsigned amax = 0;  // largest |x| written, for the range check
    for (int st = 0; st < nsteps; ++st) {
        const bool fwd = st < nchunk;
        const int q0 = (fwd ? st : 2 * nchunk - 2 - st) * K, kk = min(K, nrow - q0);
        {
            double v[16];
            fetch<M>(fwd ? rhs : x, v, base, live, nlive, q0, kk, L, cont);
            deposit<M>(v, tile, live, nlive, kk, cont);
        }
        if (live && fwd) {
            const bool last = st == nchunk - 1;
#pragma unroll
            for (int u = 0; u < K; ++u) {
                if (u < kk) {
                    T t[M];
#pragma unroll
                    for (int i = 0; i < M; ++i) t[i] = Num::in_rhs(my + u * M + i);
                    forward_row<Num, M>(fac, pivs, q0 + u, t, y);
                    if (last && u == kk - 1) {  // y of the last row is its solution
#pragma unroll
                        for (int i = 0; i < M; ++i) {
                            Num::out(my + u * M + i, y[i]);
                            amax = max(amax, Num::mag(y[i]));
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < M; ++i) Num::sts(my + u * M + i, y[i]);
                    }
                }
            }
            if (last) {  // turn around in the tile
#pragma unroll
                for (int u = K - 2; u >= 0; --u) {
                    if (u + 1 < kk) {
                        T t[M];
#pragma unroll
                        for (int i = 0; i < M; ++i) t[i] = Num::lds(my + u * M + i);
                        backward_row<Num, M>(fac, q0 + u, t, y);
#pragma unroll
                        for (int i = 0; i < M; ++i) {
                            Num::out(my + u * M + i, y[i]);
                            amax = max(amax, Num::mag(y[i]));
                        }
                    }
                }
            }
        } else if (live) {
#pragma unroll
            for (int u = K - 1; u >= 0; --u) {
                T t[M];
#pragma unroll
                for (int i = 0; i < M; ++i) t[i] = Num::lds(my + u * M + i);
                backward_row<Num, M>(fac, q0 + u, t, y);
#pragma unroll
                for (int i = 0; i < M; ++i) {
                    Num::out(my + u * M + i, y[i]);
                    amax = max(amax, Num::mag(y[i]));
                }
            }
        }
        store<M>(x, tile, base, live, nlive, q0, kk, L, cont);
    }
    if (live) pbt::report_status(status, pbt::range_bits<Num>(amax, true));
}

template <int M>
cudaError_t launch_shared(const pbt_shared* sh, const double* rhs, double* x, const pbt_lines& L, cudaStream_t st) {
    const long long nsys = (long long)L.nsys_inner * L.nsys_outer;
    const long long warps = (nsys + 31) / 32;
    const long long grid = (warps + kSharedWarps - 1) / kSharedWarps;
    if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
    const int contiguous = (L.elem_stride == 1 && L.row_stride == M) ? 1 : 0;
    if (sh->precision == PBT_PREC_FF)
        k_shared<pbt::FF, M><<<(unsigned)grid, kSharedThreads, 0, st>>>(sh->fac, sh->piv, rhs, x, sh->nrow, L,
                                                                        contiguous, sh->status);
    else
        k_shared<pbt::F64, M><<<(unsigned)grid, kSharedThreads, 0, st>>>(sh->fac, sh->piv, rhs, x, sh->nrow, L,
                                                                         contiguous, sh->status);
    return cudaGetLastError();
}

// Elimination with partial pivoting of a (m x m, column-major) in place, as
// the kernels' lu_factor does: the multiplier of row i at step k stays where
// row i was at step k, U rows are kept normalised, the diagonal holds
// 1/U_kk; swaps[k] = the row swapped with row k.  False on a zero pivot.
bool host_factor(int m, double* a, int* swaps) {
    for (int k = 0; k < m; ++k) {
        int p = k;
        double best = std::fabs(a[k + m * k]);
        for (int i = k + 1; i < m; ++i) {
            const double v = std::fabs(a[i + m * k]);
            if (v > best) {
                best = v;
                p = i;
            }
        }
        swaps[k] = p;
        if (p != k)
            for (int c = k; c < m; ++c) {
                const double t = a[k + m * c];
                a[k + m * c] = a[p + m * c];
                a[p + m * c] = t;
            }
        if (a[k + m * k] == 0.0) return false;
        const double r = 1.0 / a[k + m * k];
        a[k + m * k] = r;
        for (int i = k + 1; i < m; ++i) {
            const double l = a[i + m * k] * r;
            a[i + m * k] = l;
            for (int c = k + 1; c < m; ++c) a[i + m * c] = std::fma(-l, a[k + m * c], a[i + m * c]);
        }
    }
    return true;
}

// Solve with the factors of host_factor: b (length m) in, solution out.
void host_solve(int m, const double* f, const int* swaps, double* b) {
    for (int k = 0; k < m; ++k) {
        const int p = swaps[k];
        if (p != k) {
            const double t = b[k];
            b[k] = b[p];
            b[p] = t;
        }
        for (int i = k + 1; i < m; ++i) b[i] = std::fma(-f[i + m * k], b[k], b[i]);
    }
    for (int k = m - 1; k >= 0; --k) {
        b[k] *= f[k + m * k];
        for (int i = 0; i < k; ++i) b[i] = std::fma(-f[i + m * k], b[k], b[i]);
    }
}

}  // namespace

extern "C" {

int pbt_shared_create(pbt_shared** out, int m, int nrow, const double* a, const double* b, const double* c,
                      int precision) {
    if (!out) return pbt::set_last_error(PBT_EINVAL, "shared_create: null argument");
    *out = nullptr;
    if (precision != PBT_PREC_FP64 && precision != PBT_PREC_FF)
        return pbt::set_last_error(PBT_EUNSUPPORTED, "shared_create: precision must be PBT_PREC_FP64 or PBT_PREC_FF");
    if (m < 1 || m > PBT_MAX_BLOCK || nrow < 2 || !a || !b || !c) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "shared_create: need 1 <= m <= %d, nrow >= 2 and three arrays (m=%d, nrow=%d)",
                      PBT_MAX_BLOCK, m, nrow);
        return pbt::set_last_error(PBT_EINVAL, buf);
    }
    const size_t mm = (size_t)m * m;
    std::vector<double> fac((size_t)nrow * 3 * mm);
    std::vector<long long> piv(nrow, 0);
    std::vector<double> cprev(mm, 0.0), R(mm), col(m);
    std::vector<int> sw(m);
    auto elem = [&](const double* x, int q, int i, int j) { return x[q + (size_t)nrow * (i + m * j)]; };
    for (int q = 0; q < nrow; ++q) {
        double* Aq = fac.data() + (size_t)q * 3 * mm;
        double* F = Aq + mm;
        double* Cq = F + mm;
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) Aq[i + m * j] = q > 0 ? elem(a, q, i, j) : 0.0;
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) {
                double v = elem(b, q, i, j);
                if (q > 0)
                    for (int k = 0; k < m; ++k) v = std::fma(-Aq[i + m * k], cprev[k + m * j], v);
                R[i + m * j] = v;
            }
        if (!host_factor(m, R.data(), sw.data())) {
            char buf[120];
            std::snprintf(buf, sizeof buf, "shared_create: zero pivot in block row %d", q);
            return pbt::set_last_error(PBT_ESINGULAR, buf);
        }
        std::memcpy(F, R.data(), mm * sizeof(double));
        long long pk = 0;
        for (int k = 0; k + 1 < m; ++k) pk |= (long long)sw[k] << (4 * k);
        piv[q] = pk;
        if (q + 1 < nrow) {
            for (int j = 0; j < m; ++j) {
                for (int i = 0; i < m; ++i) col[i] = elem(c, q, i, j);
                host_solve(m, F, sw.data(), col.data());
                for (int i = 0; i < m; ++i) Cq[i + m * j] = col[i];
            }
            std::memcpy(cprev.data(), Cq, mm * sizeof(double));
        }
    }
    if (precision == PBT_PREC_FF) {
        // (h, l) = (v rounded to float, the rest rounded to float): |l| <= ulp(h)/2.
        for (double& v : fac) {
            if (!(std::fabs(v) < 0x1p127))
                return pbt::set_last_error(PBT_ERANGE, "shared_create: a factor is outside the float-float range");
            const float h = (float)v, l = (float)(v - (double)h);
            float pair[2] = {h, l};
            std::memcpy(&v, pair, sizeof v);
        }
    }
    pbt_shared* s = new (std::nothrow) pbt_shared();
    if (!s) return pbt::set_last_error(PBT_ENOMEM, "shared_create: host allocation failed");
    s->m = m;
    s->nrow = nrow;
    s->precision = precision;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&s->fac), fac.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&s->piv), piv.size() * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&s->status), sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(s->status, 0, sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaMemcpy(s->fac, fac.data(), fac.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(s->piv, piv.data(), piv.size() * sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(s->fac);
        cudaFree(s->piv);
        cudaFree(s->status);
        delete s;
        return pbt::set_last_error(e == cudaErrorMemoryAllocation ? PBT_ENOMEM : PBT_ECUDA,
                                   (std::string("shared_create: ") + cudaGetErrorString(e)).c_str());
    }
    *out = s;
    return PBT_OK;
}

int pbt_shared_solve(const pbt_shared* s, const double* rhs, double* x, const pbt_lines* L, void* stream) {
    if (!s || s->magic != kSharedMagic) return pbt::set_last_error(PBT_ESTATE, "shared_solve: null or destroyed handle");
    if (!rhs || !x || !L) return pbt::set_last_error(PBT_EINVAL, "shared_solve: null argument");
    if (L->nsys_inner < 0 || L->nsys_outer < 0)
        return pbt::set_last_error(PBT_EINVAL, "shared_solve: negative line counts");
    if ((long long)L->nsys_inner * L->nsys_outer == 0) return PBT_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e;
    switch (s->m) {
        case 1: e = launch_shared<1>(s, rhs, x, *L, st); break;
        case 2: e = launch_shared<2>(s, rhs, x, *L, st); break;
        case 3: e = launch_shared<3>(s, rhs, x, *L, st); break;
        case 4: e = launch_shared<4>(s, rhs, x, *L, st); break;
        case 5: e = launch_shared<5>(s, rhs, x, *L, st); break;
        case 6: e = launch_shared<6>(s, rhs, x, *L, st); break;
        case 7: e = launch_shared<7>(s, rhs, x, *L, st); break;
        case 8: e = launch_shared<8>(s, rhs, x, *L, st); break;
        case 9: e = launch_shared<9>(s, rhs, x, *L, st); break;
        default: e = launch_shared<10>(s, rhs, x, *L, st); break;
    }
    if (e != cudaSuccess)
        return pbt::set_last_error(PBT_ECUDA, (std::string("shared_solve: ") + cudaGetErrorString(e)).c_str());
    return PBT_OK;
}

int pbt_shared_shape(const pbt_shared* s, int* m, int* nrow) {
    if (!s || s->magic != kSharedMagic) return pbt::set_last_error(PBT_ESTATE, "shared_shape: null or destroyed handle");
    if (m) *m = s->m;
    if (nrow) *nrow = s->nrow;
    return PBT_OK;
}

int pbt_shared_status(const pbt_shared* s, void* stream) {
    if (!s || s->magic != kSharedMagic) return pbt::set_last_error(PBT_ESTATE, "shared_status: null or destroyed handle");
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    unsigned long long w = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&w, s->status, sizeof w, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(s->status, 0, sizeof w);
    if (e != cudaSuccess)
        return pbt::set_last_error(PBT_ECUDA, (std::string("shared_status: ") + cudaGetErrorString(e)).c_str());
    if (w & pbt::kRangeMark)
        return pbt::set_last_error(PBT_ERANGE, "shared_status: a float-float solve left the arithmetic's range (a "
                                               "right-hand side outside 2^-96 <= |x| < 2^96, an overflow, or a line "
                                               "whose solution lies below 2^-100); those lines are not valid");
    return PBT_OK;
}

int pbt_shared_destroy(pbt_shared* s) {
    if (!s) return PBT_OK;
    if (s->magic != kSharedMagic) return pbt::set_last_error(PBT_ESTATE, "shared_destroy: destroyed handle");
    cudaFree(s->fac);
    cudaFree(s->piv);
    cudaFree(s->status);
    s->magic = 0;
    delete s;
    return PBT_OK;
}

}  // extern "C"
