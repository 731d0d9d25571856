/*
 * pbt_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the batched
 * modified block Thomas solver with two-stage reduction.
 *
 * Restates, stage by stage and in the same operation order, PaScaL_BTDMA's
 * MPI CPU path, Fortran_Original/src/mod_btdma_cpu.f90:
 *   btdma_many        :15-78    plain block Thomas (reduced solve)
 *   btdma_many_cycl   :80-183   cyclic block Thomas (cyclic reduced solve; also
 *                               applied to a whole periodic line, one segment)
 *   btdma_many_mpi    :242-271  stage sequence, non-cyclic
 *   btdma_many_cyclic_mpi :273-302  stage sequence, cyclic
 *   btdma_many_modi   :305-443  stage 1, modified elimination of a segment
 *   btdma_many_a2av_* :445-509  all-to-all of the reduced rows (here: a transpose)
 *   btdma_many_update :511-535  interior update
 * BLAS/LAPACK calls are restated as loops with the reference BLAS loop order
 * (dgemm 'N','N' and dgemv 'N': column-oriented, ascending inner index) and
 * LAPACK dgesv = dgetf2 (partial pivoting, multipliers scaled by the pivot's
 * reciprocal) + dgetrs (row swaps, unit-lower solve, non-unit-upper solve
 * dividing by the diagonal).  The external dependency is an unversioned
 * system BLAS/LAPACK (Fortran_Original/Makefile.inc:29); its published
 * reference algorithms are what is restated here.
 *
 * Internal layout is the reference CPU layout, X(m,m,nsys,nrow) column-major
 * (mod_btdma_cpu.f90:18): block (sys,row) is contiguous m*m doubles, and the
 * rows of one segment form exactly the rank-local array of the reference.
 * The exported entry points take the reference GPU layout
 * (CUDA_CXX_Port/include/pascal_btdma_cuda.hpp:46-65) and transpose at entry
 * and exit, except the *_cpu entry points, which take the CPU layout and are
 * what the CPU baseline times.
 *
 * Build with -ffp-contract=off so that no multiply-add is fused: results are
 * then identical on x86-64 and AArch64 hosts.
 */
#include "pbt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define MAXM 10

/* ------------------------------------------------------------------------- */
/* BLAS/LAPACK restatements (column-major, leading dimension = m)             */
/* ------------------------------------------------------------------------- */

/* c = a*b  (dgemm 'N','N', alpha=1, beta=0; reference loop order j, l, i) */
static void gemm_nn(int m, const double* a, const double* b, double* c) {
    for (int j = 0; j < m; ++j) {
        for (int i = 0; i < m; ++i) c[i + m * j] = 0.0;
        for (int l = 0; l < m; ++l) {
            const double t = b[l + m * j];
            for (int i = 0; i < m; ++i) c[i + m * j] += t * a[i + m * l];
        }
    }
}

/* y = a*x  (dgemv 'N', alpha=1, beta=0; reference loop order j, i) */
static void gemv_n(int m, const double* a, const double* x, double* y) {
    for (int i = 0; i < m; ++i) y[i] = 0.0;
    for (int j = 0; j < m; ++j) {
        const double t = x[j];
        for (int i = 0; i < m; ++i) y[i] += t * a[i + m * j];
    }
}

int pbto_dgesv(int m, int nrhs, double* a, int lda, double* b, int ldb) {
    int ipiv[MAXM];
    int info = 0;
    /* dgetf2: right-looking LU with partial pivoting */
    for (int j = 0; j < m; ++j) {
        int p = j;
        double amax = fabs(a[j + lda * j]);
        for (int i = j + 1; i < m; ++i) {
            const double v = fabs(a[i + lda * j]);
            if (v > amax) { amax = v; p = i; }
        }
        ipiv[j] = p;
        if (a[p + lda * j] != 0.0) {
            if (p != j) {
                for (int k = 0; k < m; ++k) {
                    const double t = a[j + lda * k];
                    a[j + lda * k] = a[p + lda * k];
                    a[p + lda * k] = t;
                }
            }
            const double r = 1.0 / a[j + lda * j];
            for (int i = j + 1; i < m; ++i) a[i + lda * j] *= r;
        } else if (info == 0) {
            info = j + 1;
        }
        for (int k = j + 1; k < m; ++k) {          /* dger rank-1 update */
            const double t = a[j + lda * k];
            if (t != 0.0)
                for (int i = j + 1; i < m; ++i) a[i + lda * k] -= a[i + lda * j] * t;
        }
    }
    if (info != 0) return info;
    /* dgetrs: dlaswp, then dtrsm L (unit) and dtrsm U (non-unit) */
    for (int j = 0; j < m; ++j) {
        const int p = ipiv[j];
        if (p != j)
            for (int k = 0; k < nrhs; ++k) {
                const double t = b[j + ldb * k];
                b[j + ldb * k] = b[p + ldb * k];
                b[p + ldb * k] = t;
            }
    }
    for (int k = 0; k < nrhs; ++k) {
        double* x = b + ldb * k;
        for (int j = 0; j < m; ++j)
            if (x[j] != 0.0)
                for (int i = j + 1; i < m; ++i) x[i] -= x[j] * a[i + lda * j];
        for (int j = m - 1; j >= 0; --j)
            if (x[j] != 0.0) {
                x[j] /= a[j + lda * j];
                for (int i = 0; i < j; ++i) x[i] -= x[j] * a[i + lda * j];
            }
    }
    return 0;
}

void pbto_partition(int N, int P, int seg, int* first, int* last) {
    const int base = N / P, rem = N % P;
    const int extra = seg < rem ? 1 : 0;
    const int a = seg < rem ? seg : rem;
    *first = seg * base + a;
    *last = *first + base + extra - 1;
}

/* ------------------------------------------------------------------------- */
/* Per-chunk kernels, reference CPU layout X(m,m,ns,n) with ns = row stride   */
/* in blocks; sys ranges over [s0, s1).                                       */
/* ------------------------------------------------------------------------- */

#define BLK(X, sys, row) ((X) + (size_t)mm * ((size_t)(sys) + (size_t)ns * (size_t)(row)))
#define VEC(X, sys, row) ((X) + (size_t)m * ((size_t)(sys) + (size_t)ns * (size_t)(row)))

/* btdma_many (mod_btdma_cpu.f90:15-78) on n rows; row 0's A and row n-1's C
 * are never read. */
static int many(int n, int ns, int m, int s0, int s1,
                double* a, double* b, double* c, double* d) {
    const int mm = m * m;
    double sol[MAXM * (MAXM + 1)], rr[MAXM * MAXM], akc[MAXM * MAXM], akd[MAXM], ckd[MAXM];
    int bad = 0;
    for (int sys = s0; sys < s1; ++sys) {                 /* q = 1 */
        memcpy(sol, VEC(d, sys, 0), sizeof(double) * m);
        memcpy(sol + m, BLK(c, sys, 0), sizeof(double) * mm);
        memcpy(rr, BLK(b, sys, 0), sizeof(double) * mm);
        bad |= pbto_dgesv(m, m + 1, rr, m, sol, m) != 0;
        memcpy(VEC(d, sys, 0), sol, sizeof(double) * m);
        memcpy(BLK(c, sys, 0), sol + m, sizeof(double) * mm);
    }
    for (int q = 1; q < n; ++q)
        for (int sys = s0; sys < s1; ++sys) {
            gemm_nn(m, BLK(a, sys, q), BLK(c, sys, q - 1), akc);
            gemv_n(m, BLK(a, sys, q), VEC(d, sys, q - 1), akd);
            const double* dq = VEC(d, sys, q);
            const double* bq = BLK(b, sys, q);
            for (int i = 0; i < m; ++i) sol[i] = dq[i] - akd[i];
            memcpy(sol + m, BLK(c, sys, q), sizeof(double) * mm);
            for (int k = 0; k < mm; ++k) rr[k] = bq[k] - akc[k];
            bad |= pbto_dgesv(m, m + 1, rr, m, sol, m) != 0;
            memcpy(VEC(d, sys, q), sol, sizeof(double) * m);
            memcpy(BLK(c, sys, q), sol + m, sizeof(double) * mm);
        }
    for (int q = n - 2; q >= 0; --q)
        for (int sys = s0; sys < s1; ++sys) {
            gemv_n(m, BLK(c, sys, q), VEC(d, sys, q + 1), ckd);
            double* dq = VEC(d, sys, q);
            for (int i = 0; i < m; ++i) dq[i] = dq[i] - ckd[i];
        }
    return bad;
}

/* btdma_many_cycl (mod_btdma_cpu.f90:80-183): periodic block Thomas with the
 * fill-in column e; row 0's A couples to row n-1, row n-1's C to row 0. */
static int many_cycl(int n, int ns, int m, int s0, int s1,
                     double* a, double* b, double* c, double* d, double* e) {
    const int mm = m * m;
    double sol[MAXM * (2 * MAXM + 1)], rr[MAXM * MAXM];
    double akc[MAXM * MAXM], ake[MAXM * MAXM], cke[MAXM * MAXM];
    double akd[MAXM], ckd[MAXM], ekd[MAXM];
    int bad = 0;
    for (int q = 0; q < n; ++q)
        for (int sys = s0; sys < s1; ++sys) memset(BLK(e, sys, q), 0, sizeof(double) * mm);
    for (int sys = s0; sys < s1; ++sys) {
        double* e1 = BLK(e, sys, 1);
        const double* a1 = BLK(a, sys, 1);
        for (int k = 0; k < mm; ++k) e1[k] = -a1[k];
        double* en = BLK(e, sys, n - 1);
        const double* cn = BLK(c, sys, n - 1);
        for (int k = 0; k < mm; ++k) en[k] = -cn[k];
    }
    for (int sys = s0; sys < s1; ++sys) {                 /* q = 2 (0-based 1) */
        memcpy(sol, VEC(d, sys, 1), sizeof(double) * m);
        memcpy(sol + m, BLK(e, sys, 1), sizeof(double) * mm);
        memcpy(sol + m + mm, BLK(c, sys, 1), sizeof(double) * mm);
        memcpy(rr, BLK(b, sys, 1), sizeof(double) * mm);
        bad |= pbto_dgesv(m, 2 * m + 1, rr, m, sol, m) != 0;
        memcpy(VEC(d, sys, 1), sol, sizeof(double) * m);
        memcpy(BLK(e, sys, 1), sol + m, sizeof(double) * mm);
        memcpy(BLK(c, sys, 1), sol + m + mm, sizeof(double) * mm);
    }
    for (int q = 2; q < n; ++q)
        for (int sys = s0; sys < s1; ++sys) {
            gemm_nn(m, BLK(a, sys, q), BLK(c, sys, q - 1), akc);
            gemv_n(m, BLK(a, sys, q), VEC(d, sys, q - 1), akd);
            gemm_nn(m, BLK(a, sys, q), BLK(e, sys, q - 1), ake);
            const double* dq = VEC(d, sys, q);
            const double* eq = BLK(e, sys, q);
            const double* bq = BLK(b, sys, q);
            for (int i = 0; i < m; ++i) sol[i] = dq[i] - akd[i];
            for (int k = 0; k < mm; ++k) sol[m + k] = eq[k] - ake[k];
            memcpy(sol + m + mm, BLK(c, sys, q), sizeof(double) * mm);
            for (int k = 0; k < mm; ++k) rr[k] = bq[k] - akc[k];
            bad |= pbto_dgesv(m, 2 * m + 1, rr, m, sol, m) != 0;
            memcpy(VEC(d, sys, q), sol, sizeof(double) * m);
            memcpy(BLK(e, sys, q), sol + m, sizeof(double) * mm);
            memcpy(BLK(c, sys, q), sol + m + mm, sizeof(double) * mm);
        }
    for (int q = n - 2; q >= 1; --q)
        for (int sys = s0; sys < s1; ++sys) {
            gemv_n(m, BLK(c, sys, q), VEC(d, sys, q + 1), ckd);
            gemm_nn(m, BLK(c, sys, q), BLK(e, sys, q + 1), cke);
            double* dq = VEC(d, sys, q);
            double* eq = BLK(e, sys, q);
            for (int i = 0; i < m; ++i) dq[i] = dq[i] - ckd[i];
            for (int k = 0; k < mm; ++k) eq[k] = eq[k] - cke[k];
        }
    for (int sys = s0; sys < s1; ++sys) {
        gemm_nn(m, BLK(a, sys, 0), BLK(e, sys, n - 1), ake);
        gemm_nn(m, BLK(c, sys, 0), BLK(e, sys, 1), cke);
        gemv_n(m, BLK(a, sys, 0), VEC(d, sys, n - 1), akd);
        gemv_n(m, BLK(c, sys, 0), VEC(d, sys, 1), ckd);
        const double* b0 = BLK(b, sys, 0);
        for (int k = 0; k < mm; ++k) rr[k] = b0[k] + ake[k] + cke[k];
        double* d0 = VEC(d, sys, 0);
        for (int i = 0; i < m; ++i) d0[i] = d0[i] - akd[i] - ckd[i];
        bad |= pbto_dgesv(m, 1, rr, m, d0, m) != 0;
    }
    for (int q = 1; q < n; ++q)
        for (int sys = s0; sys < s1; ++sys) {
            gemv_n(m, BLK(e, sys, q), VEC(d, sys, 0), ekd);
            double* dq = VEC(d, sys, q);
            for (int i = 0; i < m; ++i) dq[i] = dq[i] + ekd[i];
        }
    return bad;
}

/* btdma_many_modi (mod_btdma_cpu.f90:305-443) on one segment of n rows.
 * Writes the two reduced rows of each system into rows r0, r0+1 of the
 * transposed reduced arrays ta, tc, td (layout (m,m,tns,2P), system index
 * sys - s0); the reduced B is the identity and is written into tb. */
static int modi(int n, int ns, int m, int s0, int s1,
                double* a, const double* b, double* c, double* d,
                int tns, int r0, double* ta, double* tb, double* tc, double* td) {
    const int mm = m * m;
    double sol[MAXM * (2 * MAXM + 1)], rr[MAXM * MAXM];
    double aqd[MAXM], cqd[MAXM], aqa[MAXM * MAXM], aqc[MAXM * MAXM];
    double cqa[MAXM * MAXM], cqc[MAXM * MAXM];
    int bad = 0;
    for (int q = 0; q < 2 && q < n; ++q)                  /* q = 1, 2 */
        for (int sys = s0; sys < s1; ++sys) {
            memcpy(sol, VEC(d, sys, q), sizeof(double) * m);
            memcpy(sol + m, BLK(a, sys, q), sizeof(double) * mm);
            memcpy(sol + m + mm, BLK(c, sys, q), sizeof(double) * mm);
            memcpy(rr, BLK(b, sys, q), sizeof(double) * mm);
            bad |= pbto_dgesv(m, 2 * m + 1, rr, m, sol, m) != 0;
            memcpy(VEC(d, sys, q), sol, sizeof(double) * m);
            memcpy(BLK(a, sys, q), sol + m, sizeof(double) * mm);
            memcpy(BLK(c, sys, q), sol + m + mm, sizeof(double) * mm);
        }
    for (int q = 2; q < n; ++q)                           /* q = 3..nrow_sub */
        for (int sys = s0; sys < s1; ++sys) {
            gemv_n(m, BLK(a, sys, q), VEC(d, sys, q - 1), aqd);
            gemm_nn(m, BLK(a, sys, q), BLK(a, sys, q - 1), aqa);
            gemm_nn(m, BLK(a, sys, q), BLK(c, sys, q - 1), aqc);
            const double* dq = VEC(d, sys, q);
            const double* bq = BLK(b, sys, q);
            for (int i = 0; i < m; ++i) sol[i] = dq[i] - aqd[i];
            for (int k = 0; k < mm; ++k) sol[m + k] = -aqa[k];
            memcpy(sol + m + mm, BLK(c, sys, q), sizeof(double) * mm);
            for (int k = 0; k < mm; ++k) rr[k] = bq[k] - aqc[k];
            bad |= pbto_dgesv(m, 2 * m + 1, rr, m, sol, m) != 0;
            memcpy(VEC(d, sys, q), sol, sizeof(double) * m);
            memcpy(BLK(a, sys, q), sol + m, sizeof(double) * mm);
            memcpy(BLK(c, sys, q), sol + m + mm, sizeof(double) * mm);
        }
    for (int q = n - 3; q >= 1; --q)                      /* q = nrow_sub-2 .. 2 */
        for (int sys = s0; sys < s1; ++sys) {
            gemv_n(m, BLK(c, sys, q), VEC(d, sys, q + 1), cqd);
            gemm_nn(m, BLK(c, sys, q), BLK(a, sys, q + 1), cqa);
            gemm_nn(m, BLK(c, sys, q), BLK(c, sys, q + 1), cqc);
            double* dq = VEC(d, sys, q);
            double* aq = BLK(a, sys, q);
            double* cq = BLK(c, sys, q);
            for (int i = 0; i < m; ++i) dq[i] = dq[i] - cqd[i];
            for (int k = 0; k < mm; ++k) aq[k] = aq[k] - cqa[k];
            for (int k = 0; k < mm; ++k) cq[k] = -cqc[k];
        }
    for (int sys = s0; sys < s1; ++sys) {                 /* q = 1 */
        gemv_n(m, BLK(c, sys, 0), VEC(d, sys, 1), cqd);
        gemm_nn(m, BLK(c, sys, 0), BLK(c, sys, 1), cqc);
        gemm_nn(m, BLK(c, sys, 0), BLK(a, sys, 1), cqa);
        const double* d0 = VEC(d, sys, 0);
        for (int i = 0; i < m; ++i) sol[i] = d0[i] - cqd[i];
        memcpy(sol + m, BLK(a, sys, 0), sizeof(double) * mm);
        for (int k = 0; k < mm; ++k) sol[m + mm + k] = -cqc[k];
        for (int j = 0; j < m; ++j)
            for (int i = 0; i < m; ++i) rr[i + m * j] = (i == j ? 1.0 : 0.0) - cqa[i + m * j];
        bad |= pbto_dgesv(m, 2 * m + 1, rr, m, sol, m) != 0;
        memcpy(VEC(d, sys, 0), sol, sizeof(double) * m);
        memcpy(BLK(a, sys, 0), sol + m, sizeof(double) * mm);
        memcpy(BLK(c, sys, 0), sol + m + mm, sizeof(double) * mm);
    }
    /* reduced rows; the all-to-all of mod_btdma_cpu.f90:445-477 is this copy */
    for (int sys = s0; sys < s1; ++sys) {
        const int t = sys - s0;
        for (int r = 0; r < 2; ++r) {
            const int q = r == 0 ? 0 : n - 1;
            memcpy(ta + (size_t)mm * (t + (size_t)tns * (r0 + r)), BLK(a, sys, q), sizeof(double) * mm);
            memcpy(tc + (size_t)mm * (t + (size_t)tns * (r0 + r)), BLK(c, sys, q), sizeof(double) * mm);
            memcpy(td + (size_t)m * (t + (size_t)tns * (r0 + r)), VEC(d, sys, q), sizeof(double) * m);
            double* bb = tb + (size_t)mm * (t + (size_t)tns * (r0 + r));
            for (int j = 0; j < m; ++j)
                for (int i = 0; i < m; ++i) bb[i + m * j] = (i == j) ? 1.0 : 0.0;
        }
    }
    return bad;
}

/* btdma_many_update (mod_btdma_cpu.f90:511-535) on one segment. */
static void update(int n, int ns, int m, int s0, int s1,
                   const double* a, const double* c, double* d,
                   int tns, int r0, const double* td) {
    double aqd0[MAXM], cqdn[MAXM];
    const int mm = m * m;
    for (int sys = s0; sys < s1; ++sys) {
        const int t = sys - s0;
        memcpy(VEC(d, sys, 0), td + (size_t)m * (t + (size_t)tns * r0), sizeof(double) * m);
        memcpy(VEC(d, sys, n - 1), td + (size_t)m * (t + (size_t)tns * (r0 + 1)), sizeof(double) * m);
    }
    for (int q = 1; q < n - 1; ++q)
        for (int sys = s0; sys < s1; ++sys) {
            gemv_n(m, BLK(a, sys, q), VEC(d, sys, 0), aqd0);
            gemv_n(m, BLK(c, sys, q), VEC(d, sys, n - 1), cqdn);
            double* dq = VEC(d, sys, q);
            for (int i = 0; i < m; ++i) dq[i] = dq[i] - aqd0[i] - cqdn[i];
        }
    (void)mm;
}

/* ------------------------------------------------------------------------- */
/* Driver: one chunk of systems through the whole reference stage sequence.  */
/* ------------------------------------------------------------------------- */

typedef struct {
    int m, nsys, N, P, cyclic, thomas;
    double *A, *B, *C, *D;
    double* E;  /* whole-line periodic solve: the fill-in column, X(m,m,nsys,N) */
    int s0, s1;
    int bad;
    int err;
} chunk_job;

static void* run_chunk(void* arg) {
    chunk_job* jb = (chunk_job*)arg;
    const int m = jb->m, mm = m * m, ns = jb->nsys, P = jb->P;
    const int s0 = jb->s0, s1 = jb->s1, cnt = s1 - s0;
    if (cnt <= 0) return NULL;
    if (jb->thomas) {
        /* One segment per line: the reference's reduced-system solvers applied
         * to the original rows (btdma_many, or btdma_many_cycl for periodic
         * lines, which needs N >= 3). */
        if (jb->cyclic)
            jb->bad += many_cycl(jb->N, ns, m, s0, s1, jb->A, jb->B, jb->C, jb->D, jb->E);
        else
            jb->bad += many(jb->N, ns, m, s0, s1, jb->A, jb->B, jb->C, jb->D);
        return NULL;
    }
    const int R = 2 * P;
    double* ta = (double*)malloc(sizeof(double) * (size_t)mm * cnt * R);
    double* tb = (double*)malloc(sizeof(double) * (size_t)mm * cnt * R);
    double* tc = (double*)malloc(sizeof(double) * (size_t)mm * cnt * R);
    double* td = (double*)malloc(sizeof(double) * (size_t)m * cnt * R);
    double* te = jb->cyclic ? (double*)malloc(sizeof(double) * (size_t)mm * cnt * R) : NULL;
    if (!ta || !tb || !tc || !td || (jb->cyclic && !te)) {
        jb->err = 1;
        free(ta); free(tb); free(tc); free(td); free(te);
        return NULL;
    }
    for (int s = 0; s < P; ++s) {
        int f, l;
        pbto_partition(jb->N, P, s, &f, &l);
        const size_t off_m = (size_t)mm * ns * f, off_v = (size_t)m * ns * f;
        jb->bad += modi(l - f + 1, ns, m, s0, s1, jb->A + off_m, jb->B + off_m,
                        jb->C + off_m, jb->D + off_v, cnt, 2 * s, ta, tb, tc, td);
    }
    if (jb->cyclic)
        jb->bad += many_cycl(R, cnt, m, 0, cnt, ta, tb, tc, td, te);
    else
        jb->bad += many(R, cnt, m, 0, cnt, ta, tb, tc, td);
    for (int s = 0; s < P; ++s) {
        int f, l;
        pbto_partition(jb->N, P, s, &f, &l);
        const size_t off_m = (size_t)mm * ns * f, off_v = (size_t)m * ns * f;
        update(l - f + 1, ns, m, s0, s1, jb->A + off_m, jb->C + off_m, jb->D + off_v,
               cnt, 2 * s, td);
    }
    free(ta); free(tb); free(tc); free(td); free(te);
    return NULL;
}

int pbto_default_threads(void) {
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

static int run_cpu_layout(int m, int nsys, int N, int P, int cyclic, int thomas,
                          double* A, double* B, double* C, double* D, int nthreads) {
    if (m < 1 || m > MAXM || nsys < 1 || P < 1 || N < 2 * P) return -1;
    if (thomas && cyclic && N < 3) return -1;
    if (nthreads <= 0) nthreads = pbto_default_threads();
    if (nthreads > nsys) nthreads = nsys;
    chunk_job* jobs = (chunk_job*)calloc((size_t)nthreads, sizeof(chunk_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    double* E = (thomas && cyclic) ? (double*)malloc(sizeof(double) * (size_t)m * m * nsys * N) : NULL;
    if (!jobs || !th || (thomas && cyclic && !E)) { free(jobs); free(th); free(E); return -2; }
    for (int t = 0; t < nthreads; ++t) {
        int f, l;
        pbto_partition(nsys, nthreads, t, &f, &l);
        chunk_job j = {m, nsys, N, P, cyclic, thomas, A, B, C, D, E, f, l + 1, 0, 0};
        jobs[t] = j;
    }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, run_chunk, &jobs[t]);
    run_chunk(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    int bad = 0, err = 0;
    for (int t = 0; t < nthreads; ++t) { bad += jobs[t].bad; err |= jobs[t].err; }
    free(jobs); free(th); free(E);
    return err ? -2 : bad;
}

/* CPU-layout entry points: arrays X(m,m,nsys,N), D(m,nsys,N). */
int pbto_solve_noncyclic_cpu(int m, int nsys, int N, int P, double* A, double* B,
                             double* C, double* D, int nthreads) {
    return run_cpu_layout(m, nsys, N, P, 0, 0, A, B, C, D, nthreads);
}
int pbto_solve_cyclic_cpu(int m, int nsys, int N, int P, double* A, double* B,
                          double* C, double* D, int nthreads) {
    return run_cpu_layout(m, nsys, N, P, 1, 0, A, B, C, D, nthreads);
}
int pbto_block_thomas_cpu(int m, int nsys, int N, double* A, double* B, double* C,
                          double* D, int nthreads) {
    return run_cpu_layout(m, nsys, N, 1, 0, 1, A, B, C, D, nthreads);
}
int pbto_block_thomas_cyclic_cpu(int m, int nsys, int N, double* A, double* B, double* C,
                                 double* D, int nthreads) {
    return run_cpu_layout(m, nsys, N, 1, 1, 1, A, B, C, D, nthreads);
}

/* ------------------------------------------------------------------------- */
/* Layout conversion between the GPU layout (sys fastest, element planes) and */
/* the CPU layout (block fastest).                                            */
/* ------------------------------------------------------------------------- */

void pbto_gpu_to_cpu(int m, int nsys, int N, int is_matrix, const double* g, double* c) {
    const int w = is_matrix ? m * m : m;
    for (int row = 0; row < N; ++row)
        for (int e = 0; e < w; ++e) {
            const double* src = g + (size_t)nsys * (row + (size_t)N * e);
            for (int sys = 0; sys < nsys; ++sys)
                c[e + (size_t)w * (sys + (size_t)nsys * row)] = src[sys];
        }
}

void pbto_cpu_to_gpu(int m, int nsys, int N, int is_matrix, const double* c, double* g) {
    const int w = is_matrix ? m * m : m;
    for (int row = 0; row < N; ++row)
        for (int e = 0; e < w; ++e) {
            double* dst = g + (size_t)nsys * (row + (size_t)N * e);
            for (int sys = 0; sys < nsys; ++sys)
                dst[sys] = c[e + (size_t)w * (sys + (size_t)nsys * row)];
        }
}

static int run_gpu_layout(int m, int nsys, int N, int P, int cyclic, int thomas,
                          double* A, double* B, double* C, double* D, int nthreads) {
    if (m < 1 || m > MAXM || nsys < 1 || P < 1 || N < 2 * P) return -1;
    const size_t nm = (size_t)m * m * nsys * N, nv = (size_t)m * nsys * N;
    double* a = (double*)malloc(sizeof(double) * nm);
    double* b = (double*)malloc(sizeof(double) * nm);
    double* c = (double*)malloc(sizeof(double) * nm);
    double* d = (double*)malloc(sizeof(double) * nv);
    if (!a || !b || !c || !d) { free(a); free(b); free(c); free(d); return -2; }
    pbto_gpu_to_cpu(m, nsys, N, 1, A, a);
    pbto_gpu_to_cpu(m, nsys, N, 1, B, b);
    pbto_gpu_to_cpu(m, nsys, N, 1, C, c);
    pbto_gpu_to_cpu(m, nsys, N, 0, D, d);
    const int rc = run_cpu_layout(m, nsys, N, P, cyclic, thomas, a, b, c, d, nthreads);
    pbto_cpu_to_gpu(m, nsys, N, 1, a, A);
    pbto_cpu_to_gpu(m, nsys, N, 1, c, C);
    pbto_cpu_to_gpu(m, nsys, N, 0, d, D);
    free(a); free(b); free(c); free(d);
    return rc;
}

int pbto_solve_noncyclic(int m, int nsys, int N, int P, double* A, double* B, double* C,
                         double* D, int nthreads) {
    return run_gpu_layout(m, nsys, N, P, 0, 0, A, B, C, D, nthreads);
}
int pbto_solve_cyclic(int m, int nsys, int N, int P, double* A, double* B, double* C,
                      double* D, int nthreads) {
    return run_gpu_layout(m, nsys, N, P, 1, 0, A, B, C, D, nthreads);
}
int pbto_block_thomas(int m, int nsys, int N, double* A, double* B, double* C, double* D,
                      int nthreads) {
    return run_gpu_layout(m, nsys, N, 1, 0, 1, A, B, C, D, nthreads);
}
int pbto_block_thomas_cyclic(int m, int nsys, int N, double* A, double* B, double* C, double* D,
                             int nthreads) {
    return run_gpu_layout(m, nsys, N, 1, 1, 1, A, B, C, D, nthreads);
}
