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
// broadcast from L1/L2) and only its own right-hand side and solution.
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

struct pbt_shared {
    int m = 0, nrow = 0;
    double* fac = nullptr;        // per row q: A_q, the factors of R_q, C'_q (3*m*m doubles, element (i,j) at i + m*j)
    long long* piv = nullptr;     // per row q: 4 bits per elimination step, the row swapped in
    unsigned magic = 0x50425453u;  // "PBTS"
};

namespace {

constexpr unsigned kSharedMagic = 0x50425453u;
constexpr int kSharedThreads = 128;

template <int M>
__global__ void __launch_bounds__(kSharedThreads) k_shared(const double* __restrict__ fac,
                                                           const long long* __restrict__ pivs,
                                                           const double* rhs, double* x, int nrow, pbt_lines L) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nsys = (long long)L.nsys_inner * L.nsys_outer;
    if (s >= nsys) return;
    const long long s_in = s % L.nsys_inner, s_out = s / L.nsys_inner;
    const long long base = s_in * L.stride_inner + s_out * L.stride_outer;
    const double* r = rhs + base;
    double* o = x + base;
    double y[M];
    for (int q = 0; q < nrow; ++q) {
        const double* Aq = fac + (size_t)q * 3 * M * M;
        const double* F = Aq + M * M;
        const long long pq = __ldg(pivs + q);
        double t[M];
#pragma unroll
        for (int i = 0; i < M; ++i) t[i] = r[q * L.row_stride + i * L.elem_stride];
        if (q > 0) {
#pragma unroll
            for (int i = 0; i < M; ++i)
#pragma unroll
                for (int k = 0; k < M; ++k) t[i] = fma(-__ldg(Aq + i + M * k), y[k], t[i]);
        }
        // Replay the elimination of R_q on t, then back-substitute.
#pragma unroll
        for (int k = 0; k < M; ++k) {
            if (k + 1 < M) {
                const int p = (int)((pq >> (4 * k)) & 15);
#pragma unroll
                for (int i = k + 1; i < M; ++i) {
                    const bool sw = (p == i);
                    const double a = t[k], b = t[i];
                    t[k] = sw ? b : a;
                    t[i] = sw ? a : b;
                }
            }
#pragma unroll
            for (int i = k + 1; i < M; ++i) t[i] = fma(-__ldg(F + i + M * k), t[k], t[i]);
        }
#pragma unroll
        for (int k = M - 1; k >= 0; --k) {
            const double xk = t[k] * __ldg(F + k + M * k);
            y[k] = xk;
#pragma unroll
            for (int i = 0; i < k; ++i) t[i] = fma(-__ldg(F + i + M * k), xk, t[i]);
        }
#pragma unroll
        for (int i = 0; i < M; ++i) o[q * L.row_stride + i * L.elem_stride] = y[i];
    }
    for (int q = nrow - 2; q >= 0; --q) {
        const double* Cq = fac + (size_t)q * 3 * M * M + 2 * M * M;
        double t[M];
#pragma unroll
        for (int i = 0; i < M; ++i) t[i] = o[q * L.row_stride + i * L.elem_stride];
#pragma unroll
        for (int i = 0; i < M; ++i)
#pragma unroll
            for (int k = 0; k < M; ++k) t[i] = fma(-__ldg(Cq + i + M * k), y[k], t[i]);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            y[i] = t[i];
            o[q * L.row_stride + i * L.elem_stride] = t[i];
        }
    }
}

template <int M>
cudaError_t launch_shared(const pbt_shared* sh, const double* rhs, double* x, const pbt_lines& L, cudaStream_t st) {
    const long long nsys = (long long)L.nsys_inner * L.nsys_outer;
    const long long grid = (nsys + kSharedThreads - 1) / kSharedThreads;
    k_shared<M><<<(unsigned)grid, kSharedThreads, 0, st>>>(sh->fac, sh->piv, rhs, x, sh->nrow, L);
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

int pbt_shared_create(pbt_shared** out, int m, int nrow, const double* a, const double* b, const double* c) {
    if (!out) return pbt::set_last_error(PBT_EINVAL, "shared_create: null argument");
    *out = nullptr;
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
    pbt_shared* s = new (std::nothrow) pbt_shared();
    if (!s) return pbt::set_last_error(PBT_ENOMEM, "shared_create: host allocation failed");
    s->m = m;
    s->nrow = nrow;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&s->fac), fac.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&s->piv), piv.size() * sizeof(long long));
    if (e == cudaSuccess)
        e = cudaMemcpy(s->fac, fac.data(), fac.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(s->piv, piv.data(), piv.size() * sizeof(long long), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaGetLastError();
        cudaFree(s->fac);
        cudaFree(s->piv);
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

int pbt_shared_destroy(pbt_shared* s) {
    if (!s) return PBT_OK;
    if (s->magic != kSharedMagic) return pbt::set_last_error(PBT_ESTATE, "shared_destroy: destroyed handle");
    cudaFree(s->fac);
    cudaFree(s->piv);
    s->magic = 0;
    delete s;
    return PBT_OK;
}

}  // extern "C"
