// pbt_fp64.cuh -- plain FP64 kernels of the batched block-tridiagonal solve.
//
// One thread owns one (system, segment) pair; consecutive threads own
// consecutive systems, so every block-element access of a warp is one
// contiguous 256-byte segment of the reference GPU layout.  The whole m x m
// arithmetic is unrolled for the compile-time block size M.
//
//   k_thomas64   single-segment fast path: plain block Thomas on the whole
//                line (the reduced-solve recurrence of btdma_many_gpu_v2,
//                Fortran_Original/src/mod_btdma_gpu_v2.f90:241-350, applied
//                to the original rows).  Mathematically the same x as the
//                two-stage method with one segment, at ~40% of its flops.
//   k_modi64     stage 1 of the two-stage method, one segment:
//                btdma_many_modi_gpu_v2 (mod_btdma_gpu_v2.f90:618-866).  The
//                two reduced rows are written straight into the reduced
//                system's layout, which replaces the pack + MPI_ALLTOALLV +
//                unpack of :1309-1342.
//   k_reduced64  stage 2: block Thomas on the 2P-row reduced system with
//                B = I (btdma_many_gpu_v2, :241-350).
//   k_reduced_cyclic64  stage 2 of the cyclic solve (btdma_many_cycl,
//                Fortran_Original/src/mod_btdma_cpu.f90:80-183).
//   k_update64   stage 3: x_q = d'_q - A'_q x_first - C'_q x_last
//                (btdma_many_update_gpu_v2, mod_btdma_gpu_v2.f90:868-919);
//                the reduced solution is read in place, which replaces the
//                backward MPI_ALLTOALLV of :1344-1374.
#pragma once

#include "pbt_block64.cuh"
#include "pbt_internal.h"

namespace pbt {

__device__ __forceinline__ void seg_rows(int n, int p, int s, int& first, int& last) {
    const int base = n / p, rem = n % p;
    first = s * base + (s < rem ? s : rem);
    last = first + base + (s < rem ? 1 : 0) - 1;
}

// ---------------------------------------------------------------------------
// Single-segment block Thomas.  Forward: R_q = B_q - A_q C'_{q-1},
// [C'_q | y_q] = R_q^{-1} [C_q | d_q - A_q y_{q-1}]; C' goes to cw, y to D.
// Backward: x_q = y_q - C'_q x_{q+1}.
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(128) k_thomas64(const SolveArgs g) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    const int N = g.nrow;
    const size_t plane0 = (size_t)g.nsys * N;
    const size_t plane = plane0;
    const size_t rs = (size_t)g.nsys;
    const double* A = g.a + sys;
    const double* B = g.b + sys;
    const double* C = g.c + sys;
    double* D = g.d + sys;
    double* CW = g.cw + sys;
    bool bad = false;

    double cp[M][M], y[M];
    {
        double r[M][M], x[M][M + 1];
        ld_blk<M>(r, B, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) x[i][j] = C[(size_t)(i + M * j) * plane];
            x[i][M] = D[(size_t)i * plane];
        }
        gesv_pp<M, M + 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) cp[i][j] = x[i][j];
            y[i] = x[i][M];
        }
        st_blk<M>(CW, plane, cp);
        st_vec<M>(D, plane, y);
    }
    for (int q = 1; q < N - 1; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double a[M][M], r[M][M], x[M][M + 1];
        ld_blk_rw<M>(a, A + o, plane);
        ld_blk<M>(r, B + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double t = D[o + (size_t)i * plane];
#pragma unroll
            for (int l = 0; l < M; ++l) t = fma(-a[i][l], y[l], t);
            x[i][M] = t;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double s = r[i][j];
#pragma unroll
                for (int l = 0; l < M; ++l) s = fma(-a[i][l], cp[l][j], s);
                r[i][j] = s;
            }
        }
        mem_fence_compiler();
#pragma unroll
        for (int i = 0; i < M; ++i)
#pragma unroll
            for (int j = 0; j < M; ++j) x[i][j] = C[o + (size_t)(i + M * j) * plane];
        gesv_pp<M, M + 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) cp[i][j] = x[i][j];
            y[i] = x[i][M];
        }
        st_blk<M>(CW + o, plane, cp);
        st_vec<M>(D + o, plane, y);
    }
    {
        const size_t o = (size_t)(N - 1) * rs;
        double a[M][M], r[M][M], x[M][1];
        ld_blk_rw<M>(a, A + o, plane);
        ld_blk<M>(r, B + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double t = D[o + (size_t)i * plane];
#pragma unroll
            for (int l = 0; l < M; ++l) t = fma(-a[i][l], y[l], t);
            x[i][0] = t;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double s = r[i][j];
#pragma unroll
                for (int l = 0; l < M; ++l) s = fma(-a[i][l], cp[l][j], s);
                r[i][j] = s;
            }
        }
        gesv_pp<M, 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) y[i] = x[i][0];
        st_vec<M>(D + o, plane, y);
    }
    for (int q = N - 2; q >= 0; --q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double c[M][M], t[M];
        ld_blk_rw<M>(c, CW + o, plane);
        ld_vec<M>(t, D + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double s = t[i];
#pragma unroll
            for (int l = 0; l < M; ++l) s = fma(-c[i][l], y[l], s);
            t[i] = s;
        }
#pragma unroll
        for (int i = 0; i < M; ++i) y[i] = t[i];
        st_vec<M>(D + o, plane, y);
    }
    if (bad) atomicAdd(g.status, 1ull);
}

// ---------------------------------------------------------------------------
// Stage 1: modified elimination of one segment (rows f..l, n = l - f + 1).
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(128) k_modi64(const SolveArgs g) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    const int seg = blockIdx.y;
    int f, l;
    seg_rows(g.nrow, g.nseg, seg, f, l);
    const int n = l - f + 1;
    const size_t plane0 = (size_t)g.nsys * g.nrow;
    const size_t plane = plane0;
    const size_t rs = (size_t)g.nsys;
    const size_t fo = (size_t)f * rs + sys;
    const double* A = g.a + fo;
    const double* B = g.b + fo;
    const double* C = g.c + fo;
    double* D = g.d + fo;
    double* AW = g.aw + fo;
    double* CW = g.cw + fo;
    const int R = 2 * g.nseg;
    const size_t rplane = (size_t)g.nsys * R;
    bool bad = false;

    double ap[M][M], cp[M][M], dp[M];
    // Rows 1 and 2 of the segment: [A'|C'|d'] = B^{-1}[A|C|d].
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double r[M][M], x[M][2 * M + 1];
        ld_blk<M>(r, B + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) {
                x[i][j] = A[o + (size_t)(i + M * j) * plane];
                x[i][M + j] = C[o + (size_t)(i + M * j) * plane];
            }
            x[i][2 * M] = D[o + (size_t)i * plane];
        }
        gesv_pp<M, 2 * M + 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) {
                ap[i][j] = x[i][j];
                cp[i][j] = x[i][M + j];
            }
            dp[i] = x[i][2 * M];
        }
        st_blk<M>(AW + o, plane, ap);
        st_blk<M>(CW + o, plane, cp);
        st_vec<M>(D + o, plane, dp);
    }
    // Rows 3..n: R = B - A C'_{q-1};
    // [A'|C'|d'] = R^{-1}[-A A'_{q-1} | C | d - A d'_{q-1}].
    for (int q = 2; q < n; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double r[M][M], x[M][2 * M + 1];
        // One block row at a time: A_q and B_q are read row by row so that
        // only one row of each is live next to the carried A', C', d'.
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double ar[M];
#pragma unroll
            for (int k = 0; k < M; ++k) ar[k] = A[o + (size_t)(i + M * k) * plane];
            double t = D[o + (size_t)i * plane];
#pragma unroll
            for (int k = 0; k < M; ++k) t = fma(-ar[k], dp[k], t);
            x[i][2 * M] = t;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double s = 0.0, u = __ldg(B + o + (size_t)(i + M * j) * plane);
#pragma unroll
                for (int k = 0; k < M; ++k) {
                    s = fma(ar[k], ap[k][j], s);
                    u = fma(-ar[k], cp[k][j], u);
                }
                x[i][j] = -s;
                r[i][j] = u;
            }
            mem_fence_compiler();
        }
        mem_fence_compiler();
#pragma unroll
        for (int i = 0; i < M; ++i)
#pragma unroll
            for (int j = 0; j < M; ++j) x[i][M + j] = C[o + (size_t)(i + M * j) * plane];
        gesv_pp<M, 2 * M + 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) {
                ap[i][j] = x[i][j];
                cp[i][j] = x[i][M + j];
            }
            dp[i] = x[i][2 * M];
        }
        st_blk<M>(AW + o, plane, ap);
        st_blk<M>(CW + o, plane, cp);
        st_vec<M>(D + o, plane, dp);
    }
    // Reduced row 2*seg+1 = the segment's last row (A'_n, C'_n, d'_n).
    {
        const size_t ro = (size_t)sys + rs * (size_t)(2 * seg + 1);
        st_blk<M>(g.ra + ro, rplane, ap);
        st_blk<M>(g.rc + ro, rplane, cp);
        st_vec<M>(g.rd + ro, rplane, dp);
    }
    // Backward sweep, rows n-2 .. 2 (1-based): carried row = q+1.
    if (n >= 4) {
        const size_t o1 = (size_t)(n - 2) * rs;
        ld_blk_rw<M>(ap, AW + o1, plane);
        ld_blk_rw<M>(cp, CW + o1, plane);
        ld_vec<M>(dp, D + o1, plane);
        for (int q = n - 3; q >= 1; --q) {
            const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
            double a[M][M], c[M][M], dq[M];
            ld_blk_rw<M>(a, AW + o, plane);
            ld_blk_rw<M>(c, CW + o, plane);
            ld_vec<M>(dq, D + o, plane);
            // In place, row by row: row i of the new A' and C' needs only row
            // i of C'_q, so C'_q's row is overwritten once both are formed.
#pragma unroll
            for (int i = 0; i < M; ++i) {
                double t = dq[i];
#pragma unroll
                for (int k = 0; k < M; ++k) t = fma(-c[i][k], dp[k], t);
                dq[i] = t;
                double nc[M];
#pragma unroll
                for (int j = 0; j < M; ++j) {
                    double s = a[i][j], u = 0.0;
#pragma unroll
                    for (int k = 0; k < M; ++k) {
                        s = fma(-c[i][k], ap[k][j], s);
                        u = fma(c[i][k], cp[k][j], u);
                    }
                    a[i][j] = s;
                    nc[j] = -u;
                }
#pragma unroll
                for (int j = 0; j < M; ++j) c[i][j] = nc[j];
            }
#pragma unroll
            for (int i = 0; i < M; ++i) {
#pragma unroll
                for (int j = 0; j < M; ++j) {
                    ap[i][j] = a[i][j];
                    cp[i][j] = c[i][j];
                }
                dp[i] = dq[i];
            }
            st_blk<M>(AW + o, plane, ap);
            st_blk<M>(CW + o, plane, cp);
            st_vec<M>(D + o, plane, dp);
        }
    } else {
        ld_blk_rw<M>(ap, AW + rs, plane);
        ld_blk_rw<M>(cp, CW + rs, plane);
        ld_vec<M>(dp, D + rs, plane);
    }
    // Row 1: R = I - C'_1 A'_2; [A'_1|C'_1|d'_1] = R^{-1}[A'_1 | -C'_1 C'_2 | d'_1 - C'_1 d'_2].
    {
        double r[M][M], x[M][2 * M + 1];
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double c0[M];
#pragma unroll
            for (int k = 0; k < M; ++k) c0[k] = CW[(size_t)(i + M * k) * plane];
            double t = D[(size_t)i * plane];
#pragma unroll
            for (int k = 0; k < M; ++k) t = fma(-c0[k], dp[k], t);
            x[i][2 * M] = t;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double s = 0.0, u = 0.0;
#pragma unroll
                for (int k = 0; k < M; ++k) {
                    s = fma(c0[k], ap[k][j], s);
                    u = fma(c0[k], cp[k][j], u);
                }
                r[i][j] = (i == j ? 1.0 : 0.0) - s;
                x[i][M + j] = -u;
            }
            mem_fence_compiler();
        }
#pragma unroll
        for (int i = 0; i < M; ++i)
#pragma unroll
            for (int j = 0; j < M; ++j) x[i][j] = AW[(size_t)(i + M * j) * plane];
        gesv_pp<M, 2 * M + 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) {
                ap[i][j] = x[i][j];
                cp[i][j] = x[i][M + j];
            }
            dp[i] = x[i][2 * M];
        }
        st_blk<M>(AW, plane, ap);
        st_blk<M>(CW, plane, cp);
        st_vec<M>(D, plane, dp);
        const size_t ro = (size_t)sys + rs * (size_t)(2 * seg);
        st_blk<M>(g.ra + ro, rplane, ap);
        st_blk<M>(g.rc + ro, rplane, cp);
        st_vec<M>(g.rd + ro, rplane, dp);
    }
    if (bad) atomicAdd(g.status, 1ull);
}

// ---------------------------------------------------------------------------
// Stage 2: block Thomas on the R = 2P reduced rows (B = I).  Row 0's A and
// row R-1's C are never read.  C' overwrites rc, the solution overwrites rd.
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(128) k_reduced64(const SolveArgs g) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    const int R = 2 * g.nseg;
    const size_t plane0 = (size_t)g.nsys * R;
    const size_t plane = plane0;
    const size_t rs = (size_t)g.nsys;
    const double* RA = g.ra + sys;
    double* RC = g.rc + sys;
    double* RD = g.rd + sys;
    bool bad = false;

    double cp[M][M], y[M];
    // Row 0: B = I, so [C'|y] = [C|d] exactly.
    ld_blk_rw<M>(cp, RC, plane);
    ld_vec<M>(y, RD, plane);
    for (int q = 1; q < R - 1; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double a[M][M], r[M][M], x[M][M + 1];
        ld_blk_rw<M>(a, RA + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double t = RD[o + (size_t)i * plane];
#pragma unroll
            for (int k = 0; k < M; ++k) t = fma(-a[i][k], y[k], t);
            x[i][M] = t;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < M; ++k) s = fma(a[i][k], cp[k][j], s);
                r[i][j] = (i == j ? 1.0 : 0.0) - s;
                x[i][j] = RC[o + (size_t)(i + M * j) * plane];
            }
        }
        gesv_pp<M, M + 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) {
#pragma unroll
            for (int j = 0; j < M; ++j) cp[i][j] = x[i][j];
            y[i] = x[i][M];
        }
        st_blk<M>(RC + o, plane, cp);
        st_vec<M>(RD + o, plane, y);
    }
    {
        const size_t o = (size_t)(R - 1) * rs;
        double a[M][M], r[M][M], x[M][1];
        ld_blk_rw<M>(a, RA + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double t = RD[o + (size_t)i * plane];
#pragma unroll
            for (int k = 0; k < M; ++k) t = fma(-a[i][k], y[k], t);
            x[i][0] = t;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < M; ++k) s = fma(a[i][k], cp[k][j], s);
                r[i][j] = (i == j ? 1.0 : 0.0) - s;
            }
        }
        gesv_pp<M, 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) y[i] = x[i][0];
        st_vec<M>(RD + o, plane, y);
    }
    for (int q = R - 2; q >= 0; --q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double c[M][M], t[M];
        ld_blk_rw<M>(c, RC + o, plane);
        ld_vec<M>(t, RD + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double s = t[i];
#pragma unroll
            for (int k = 0; k < M; ++k) s = fma(-c[i][k], y[k], s);
            t[i] = s;
        }
#pragma unroll
        for (int i = 0; i < M; ++i) y[i] = t[i];
        st_vec<M>(RD + o, plane, y);
    }
    if (bad) atomicAdd(g.status, 1ull);
}

// ---------------------------------------------------------------------------
// Stage 2, cyclic: periodic block Thomas on the R = 2P reduced rows (B = I)
// with the fill-in column E, following btdma_many_cycl
// (Fortran_Original/src/mod_btdma_cpu.f90:80-183).  Needs R >= 4.
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(128) k_reduced_cyclic64(const SolveArgs g) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    const int R = 2 * g.nseg;
    const size_t plane0 = (size_t)g.nsys * R;
    const size_t plane = plane0;
    const size_t rs = (size_t)g.nsys;
    const double* RA = g.ra + sys;
    double* RC = g.rc + sys;
    double* RD = g.rd + sys;
    double* RE = g.re + sys;
    bool bad = false;

    // Row 1 (0-based): B = I, so [d'|e'|c'] = [d | -A_1 | C_1] exactly.
    double cp[M][M], ep[M][M], dp[M];
    {
        const size_t o = rs;
        double a1[M][M];
        ld_blk_rw<M>(a1, RA + o, plane);
        ld_blk_rw<M>(cp, RC + o, plane);
        ld_vec<M>(dp, RD + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i)
#pragma unroll
            for (int j = 0; j < M; ++j) ep[i][j] = -a1[i][j];
        st_blk<M>(RE + o, plane, ep);
    }
    // Rows 2..R-1: R_q = I - A_q C'_{q-1};
    // [d'|e'|c'] = R_q^{-1} [d - A_q d'_{q-1} | e_q - A_q e'_{q-1} | C_q],
    // with e_q = 0 except e_{R-1} = -C_{R-1}.
    for (int q = 2; q < R; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double a[M][M], r[M][M], x[M][2 * M + 1];
        ld_blk_rw<M>(a, RA + o, plane);
        const bool last = (q == R - 1);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double t = RD[o + (size_t)i * plane];
#pragma unroll
            for (int k = 0; k < M; ++k) t = fma(-a[i][k], dp[k], t);
            x[i][0] = t;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double s = 0.0, u = 0.0;
#pragma unroll
                for (int k = 0; k < M; ++k) {
                    s = fma(a[i][k], cp[k][j], s);
                    u = fma(a[i][k], ep[k][j], u);
                }
                const double cij = RC[o + (size_t)(i + M * j) * plane];
                r[i][j] = (i == j ? 1.0 : 0.0) - s;
                x[i][1 + j] = (last ? -cij : 0.0) - u;
                x[i][1 + M + j] = cij;
            }
        }
        gesv_pp<M, 2 * M + 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            dp[i] = x[i][0];
#pragma unroll
            for (int j = 0; j < M; ++j) {
                ep[i][j] = x[i][1 + j];
                cp[i][j] = x[i][1 + M + j];
            }
        }
        st_vec<M>(RD + o, plane, dp);
        st_blk<M>(RE + o, plane, ep);
        st_blk<M>(RC + o, plane, cp);
    }
    double elast[M][M], dlast[M];
#pragma unroll
    for (int i = 0; i < M; ++i) {
        dlast[i] = dp[i];
#pragma unroll
        for (int j = 0; j < M; ++j) elast[i][j] = ep[i][j];
    }
    // Backward, rows R-2..1: d'_q -= C'_q d'_{q+1}; e'_q -= C'_q e'_{q+1}.
    for (int q = R - 2; q >= 1; --q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double c[M][M], e[M][M], t[M];
        ld_blk_rw<M>(c, RC + o, plane);
        ld_blk_rw<M>(e, RE + o, plane);
        ld_vec<M>(t, RD + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double s = t[i];
#pragma unroll
            for (int k = 0; k < M; ++k) s = fma(-c[i][k], dp[k], s);
            t[i] = s;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double u = e[i][j];
#pragma unroll
                for (int k = 0; k < M; ++k) u = fma(-c[i][k], ep[k][j], u);
                e[i][j] = u;
            }
        }
#pragma unroll
        for (int i = 0; i < M; ++i) {
            dp[i] = t[i];
#pragma unroll
            for (int j = 0; j < M; ++j) ep[i][j] = e[i][j];
        }
        st_vec<M>(RD + o, plane, dp);
        st_blk<M>(RE + o, plane, ep);
    }
    // Row 0: (I + A_0 e'_{R-1} + C_0 e'_1) x_0 = d_0 - A_0 d'_{R-1} - C_0 d'_1.
    double x0[M];
    {
        double a0[M][M], c0[M][M], r[M][M], x[M][1];
        ld_blk_rw<M>(a0, RA, plane);
        ld_blk_rw<M>(c0, RC, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double t = RD[(size_t)i * plane];
#pragma unroll
            for (int k = 0; k < M; ++k) t = fma(-a0[i][k], dlast[k], t);
#pragma unroll
            for (int k = 0; k < M; ++k) t = fma(-c0[i][k], dp[k], t);
            x[i][0] = t;
#pragma unroll
            for (int j = 0; j < M; ++j) {
                double s = (i == j ? 1.0 : 0.0);
#pragma unroll
                for (int k = 0; k < M; ++k) s = fma(a0[i][k], elast[k][j], s);
#pragma unroll
                for (int k = 0; k < M; ++k) s = fma(c0[i][k], ep[k][j], s);
                r[i][j] = s;
            }
        }
        gesv_pp<M, 1>(r, x, bad);
#pragma unroll
        for (int i = 0; i < M; ++i) x0[i] = x[i][0];
        st_vec<M>(RD, plane, x0);
    }
    // Rows 1..R-1: x_q = d'_q + e'_q x_0.
    for (int q = 1; q < R; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double e[M][M], t[M];
        ld_blk_rw<M>(e, RE + o, plane);
        ld_vec<M>(t, RD + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double s = t[i];
#pragma unroll
            for (int k = 0; k < M; ++k) s = fma(e[i][k], x0[k], s);
            t[i] = s;
        }
        st_vec<M>(RD + o, plane, t);
    }
    if (bad) atomicAdd(g.status, 1ull);
}

// ---------------------------------------------------------------------------
// Stage 3: interior update of one segment from the reduced solution.
// ---------------------------------------------------------------------------
template <int M>
__global__ void __launch_bounds__(128) k_update64(const SolveArgs g) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= g.nsys) return;
    const int seg = blockIdx.y;
    int f, l;
    seg_rows(g.nrow, g.nseg, seg, f, l);
    const int n = l - f + 1;
    const size_t plane0 = (size_t)g.nsys * g.nrow;
    const size_t plane = plane0;
    const size_t rs = (size_t)g.nsys;
    const size_t fo = (size_t)f * rs + sys;
    const double* AW = g.aw + fo;
    const double* CW = g.cw + fo;
    double* D = g.d + fo;
    const int R = 2 * g.nseg;
    const size_t rplane = (size_t)g.nsys * R;
    double x0[M], xn[M];
    ld_vec<M>(x0, g.rd + sys + rs * (size_t)(2 * seg), rplane);
    ld_vec<M>(xn, g.rd + sys + rs * (size_t)(2 * seg + 1), rplane);
    st_vec<M>(D, plane, x0);
    st_vec<M>(D + (size_t)(n - 1) * rs, plane, xn);
    for (int q = 1; q < n - 1; ++q) {
        const size_t o = (size_t)q * rs;
        const size_t plane = opaque(plane0);
        double a[M][M], c[M][M], t[M];
        ld_blk_rw<M>(a, AW + o, plane);
        ld_blk_rw<M>(c, CW + o, plane);
        ld_vec<M>(t, D + o, plane);
#pragma unroll
        for (int i = 0; i < M; ++i) {
            double s = t[i];
#pragma unroll
            for (int k = 0; k < M; ++k) s = fma(-a[i][k], x0[k], s);
#pragma unroll
            for (int k = 0; k < M; ++k) s = fma(-c[i][k], xn[k], s);
            t[i] = s;
        }
        st_vec<M>(D + o, plane, t);
    }
}

// ---------------------------------------------------------------------------
// Launchers.
// ---------------------------------------------------------------------------
inline unsigned grid_x(int nsys, int tpb) { return (unsigned)((nsys + tpb - 1) / tpb); }

template <int M>
cudaError_t launch_fp64_thomas(const SolveArgs& g) {
    k_thomas64<M><<<grid_x(g.nsys, g.tpb), g.tpb, 0, g.stream>>>(g);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_fp64_modi(const SolveArgs& g) {
    dim3 grid(grid_x(g.nsys, g.tpb), (unsigned)g.nseg);
    k_modi64<M><<<grid, g.tpb, 0, g.stream>>>(g);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_fp64_reduced(const SolveArgs& g) {
    k_reduced64<M><<<grid_x(g.nsys, g.tpb), g.tpb, 0, g.stream>>>(g);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_fp64_reduced_cyclic(const SolveArgs& g) {
    k_reduced_cyclic64<M><<<grid_x(g.nsys, g.tpb), g.tpb, 0, g.stream>>>(g);
    return cudaGetLastError();
}
template <int M>
cudaError_t launch_fp64_update(const SolveArgs& g) {
    dim3 grid(grid_x(g.nsys, g.tpb), (unsigned)g.nseg);
    k_update64<M><<<grid, g.tpb, 0, g.stream>>>(g);
    return cudaGetLastError();
}

}  // namespace pbt
