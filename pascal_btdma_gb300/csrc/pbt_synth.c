/*
 * pbt_synth.c -- seeded synthetic workloads (see include/pbt_synth.h).
 * Compile with -ffp-contract=off: the generator must give identical bytes on
 * x86-64 and AArch64 hosts.
 */
#include "../../include/pbt_synth.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void pbt_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += PHILOX_W0;
            k1 += PHILOX_W1;
        }
        const uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        const uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

static inline void words(uint64_t seed, uint32_t stream, uint32_t sys, uint32_t row, uint32_t elem,
                         uint32_t w[4]) {
    const uint32_t ctr[4] = {sys, row, elem | (stream << 16), 0u};
    const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    pbt_philox4x32_10(ctr, key, w);
}

/* 53 bits -> [0, 1) exactly */
static inline double u01(uint32_t a, uint32_t b) {
    const uint64_t u = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
    return (double)u * 0x1p-53;
}

double pbt_synth_uniform(uint64_t seed, uint32_t stream, uint32_t sys, uint32_t row, uint32_t elem) {
    uint32_t w[4];
    words(seed, stream, sys, row, elem, w);
    const uint64_t u = ((uint64_t)(w[0] >> 5) << 26) | (uint64_t)(w[1] >> 6);
    return (double)u * 0x1p-52 - 1.0;
}

double pbt_synth_exp2(double t) {
    /* 2^t = 2^k * e^(f ln2), k = floor(t), f in [0,1); Taylor series of e^y
     * for y in [0, ln2) to degree 17 (remainder < 1e-17 relative). */
    const double k = floor(t);
    const double y = (t - k) * 0.69314718055994530942;
    double s = 1.0;
    for (int n = 17; n >= 1; --n) s = 1.0 + s * (y / (double)n);
    return ldexp(s, (int)k);
}

/* log2(x) for x > 0 by frexp (exact) and the atanh series of ln f, f in
 * [sqrt(1/2), sqrt(2)), to a fixed number of terms: identical on every IEEE
 * host. */
static double synth_log2(double x) {
    int k;
    double f = frexp(x, &k); /* x = f 2^k, f in [0.5, 1) */
    if (f < 0.70710678118654752440) {
        f = f * 2.0;
        k = k - 1;
    }
    const double z = (f - 1.0) / (f + 1.0), z2 = z * z;
    double s = 0.0;
    for (int n = 41; n >= 1; n -= 2) s = s * z2 + 1.0 / (double)n;
    return (double)k + 2.0 * z * s / 0.69314718055994530942;
}

typedef struct {
    int kind;
    unsigned flags;
    int m, nsys, N;
    uint64_t seed;
    double delta;
    double *A, *B, *C, *D, *X;
    int s0, s1;
} fill_job;

#define IDXM(sys, row, i, j) ((size_t)(sys) + (size_t)nsys * ((size_t)(row) + (size_t)N * ((size_t)(i) + (size_t)m * (size_t)(j))))
#define IDXV(sys, row, i) ((size_t)(sys) + (size_t)nsys * ((size_t)(row) + (size_t)N * (size_t)(i)))

static void* fill_chunk(void* arg) {
    const fill_job* jb = (const fill_job*)arg;
    const int m = jb->m, nsys = jb->nsys, N = jb->N;
    double* A = jb->A;
    double* B = jb->B;
    double* C = jb->C;
    double* D = jb->D;
    double* X = jb->X;
    const uint64_t seed = jb->seed;
    const int zero_ends = (jb->flags & PBT_SYNTH_ZERO_ENDS) != 0;
    for (int row = 0; row < N; ++row) {
        for (int sys = jb->s0; sys < jb->s1; ++sys) {
            if (jb->kind == PBT_SYNTH_DIAGONAL) {
                for (int j = 0; j < m; ++j) {
                    for (int i = 0; i < m; ++i) {
                        A[IDXM(sys, row, i, j)] = (i == j) ? 0.25 : 0.0;
                        B[IDXM(sys, row, i, j)] = (i == j) ? 2.0 : 0.0;
                        C[IDXM(sys, row, i, j)] = (i == j) ? 0.25 : 0.0;
                    }
                    D[IDXV(sys, row, j)] = 1.0;
                }
                continue;
            }
            const int a_zero = zero_ends && row == 0;
            const int c_zero = zero_ends && row == N - 1;
            if (jb->kind == PBT_SYNTH_MANUFACTURED) {
                for (int j = 0; j < m; ++j)
                    for (int i = 0; i < m; ++i) {
                        const int e = i + m * j;
                        const double a = a_zero ? 0.0 : 0.4 * pbt_synth_uniform(seed, 0, sys, row, e);
                        const double c = c_zero ? 0.0 : 0.4 * pbt_synth_uniform(seed, 2, sys, row, e);
                        A[IDXM(sys, row, i, j)] = a;
                        C[IDXM(sys, row, i, j)] = c;
                        B[IDXM(sys, row, i, j)] = ((i == j) ? 1.0 : 0.0) - (a + c);
                    }
                continue;
            }
            /* DOMINANT */
            double rs[16];
            for (int i = 0; i < m; ++i) rs[i] = 0.0;
            for (int j = 0; j < m; ++j)
                for (int i = 0; i < m; ++i) {
                    const int e = i + m * j;
                    const double a = a_zero ? 0.0 : pbt_synth_uniform(seed, 0, sys, row, e);
                    const double r = pbt_synth_uniform(seed, 1, sys, row, e);
                    const double c = c_zero ? 0.0 : pbt_synth_uniform(seed, 2, sys, row, e);
                    A[IDXM(sys, row, i, j)] = a;
                    B[IDXM(sys, row, i, j)] = r;
                    C[IDXM(sys, row, i, j)] = c;
                }
            for (int i = 0; i < m; ++i) {
                double s = 0.0;
                for (int j = 0; j < m; ++j) s = s + fabs(A[IDXM(sys, row, i, j)]);
                for (int j = 0; j < m; ++j) s = s + fabs(C[IDXM(sys, row, i, j)]);
                for (int j = 0; j < m; ++j) s = s + fabs(B[IDXM(sys, row, i, j)]);
                rs[i] = s;
            }
            for (int i = 0; i < m; ++i) {
                const double add = jb->delta * rs[i];
                B[IDXM(sys, row, i, i)] = B[IDXM(sys, row, i, i)] + add;
                D[IDXV(sys, row, i)] = pbt_synth_uniform(seed, 3, sys, row, (uint32_t)i);
            }
            if (jb->flags & PBT_SYNTH_ROW_SCALE) {
                uint32_t w[4];
                words(seed, 4, sys, row, 0, w);
                /* log-uniform in [1e-3, 1e3]: 2^t, t uniform in 3*log2(10)*[-1, 1) */
                const double t = (2.0 * u01(w[0], w[1]) - 1.0) * 9.965784284662087;
                const double s = pbt_synth_exp2(t);
                for (int j = 0; j < m; ++j)
                    for (int i = 0; i < m; ++i) {
                        A[IDXM(sys, row, i, j)] = A[IDXM(sys, row, i, j)] * s;
                        B[IDXM(sys, row, i, j)] = B[IDXM(sys, row, i, j)] * s;
                        C[IDXM(sys, row, i, j)] = C[IDXM(sys, row, i, j)] * s;
                    }
                for (int i = 0; i < m; ++i) D[IDXV(sys, row, i)] = D[IDXV(sys, row, i)] * s;
            }
        }
    }
    if (jb->kind == PBT_SYNTH_MANUFACTURED) {
        /* d = B x_q + A x_{q-1} + C x_{q+1}, with the out-of-line terms dropped */
        for (int row = 0; row < N; ++row)
            for (int sys = jb->s0; sys < jb->s1; ++sys)
                for (int i = 0; i < m; ++i) {
                    double s = 0.0;
                    for (int j = 0; j < m; ++j) {
                        const double xq = 100.0 * (row + 1) + (j + 1);
                        s = s + B[IDXM(sys, row, i, j)] * xq;
                    }
                    if (row > 0)
                        for (int j = 0; j < m; ++j) s = s + A[IDXM(sys, row, i, j)] * (100.0 * row + (j + 1));
                    if (row < N - 1)
                        for (int j = 0; j < m; ++j) s = s + C[IDXM(sys, row, i, j)] * (100.0 * (row + 2) + (j + 1));
                    D[IDXV(sys, row, i)] = s;
                    if (X) X[IDXV(sys, row, i)] = 100.0 * (row + 1) + (i + 1);
                }
    }
    return NULL;
}

int pbt_synth_fill(int kind, unsigned flags, int m, int nsys, int N, uint64_t seed, double delta, double* A,
                   double* B, double* C, double* D, double* x_ref, int nthreads) {
    if (m < 1 || m > 16 || nsys < 1 || N < 1 || !A || !B || !C || !D) return -1;
    if (kind < PBT_SYNTH_DOMINANT || kind > PBT_SYNTH_MANUFACTURED) return -1;
    if (nthreads <= 0) {
        long n = sysconf(_SC_NPROCESSORS_ONLN);
        nthreads = n > 0 ? (int)n : 1;
    }
    if (nthreads > nsys) nthreads = nsys;
    fill_job* jobs = (fill_job*)calloc((size_t)nthreads, sizeof(fill_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) {
        free(jobs);
        free(th);
        return -1;
    }
    for (int t = 0; t < nthreads; ++t) {
        const int base = nsys / nthreads, rem = nsys % nthreads;
        const int f = t * base + (t < rem ? t : rem);
        const int n = base + (t < rem ? 1 : 0);
        fill_job j = {kind, flags, m, nsys, N, seed, delta, A, B, C, D, x_ref, f, f + n};
        jobs[t] = j;
    }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, fill_chunk, &jobs[t]);
    fill_chunk(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(jobs);
    free(th);
    return 0;
}

typedef struct {
    int kind;
    unsigned flags;
    int nsys;
    const int* m;
    const int* nrow;
    const long long* mat_off;
    const long long* vec_off;
    uint64_t seed;
    double delta;
    double *A, *B, *C, *D;
    int s0, s1;
} batch_job;

/* One system s of a batch: the DOMINANT / DIAGONAL formulas of fill_chunk
 * with nsys = 1 storage at the system's own offsets and counter sys = s. */
static void* fill_batch_chunk(void* arg) {
    const batch_job* jb = (const batch_job*)arg;
    for (int s = jb->s0; s < jb->s1; ++s) {
        const int m = jb->m[s], N = jb->nrow[s];
        double* A = jb->A + jb->mat_off[s];
        double* B = jb->B + jb->mat_off[s];
        double* C = jb->C + jb->mat_off[s];
        double* D = jb->D + jb->vec_off[s];
        const int zero_ends = (jb->flags & PBT_SYNTH_ZERO_ENDS) != 0;
#define BM(row, i, j) ((size_t)(row) + (size_t)N * ((size_t)(i) + (size_t)m * (size_t)(j)))
#define BV(row, i) ((size_t)(row) + (size_t)N * (size_t)(i))
        for (int row = 0; row < N; ++row) {
            if (jb->kind == PBT_SYNTH_DIAGONAL) {
                for (int j = 0; j < m; ++j) {
                    for (int i = 0; i < m; ++i) {
                        A[BM(row, i, j)] = (i == j) ? 0.25 : 0.0;
                        B[BM(row, i, j)] = (i == j) ? 2.0 : 0.0;
                        C[BM(row, i, j)] = (i == j) ? 0.25 : 0.0;
                    }
                    D[BV(row, j)] = 1.0;
                }
                continue;
            }
            const int a_zero = zero_ends && row == 0;
            const int c_zero = zero_ends && row == N - 1;
            for (int j = 0; j < m; ++j)
                for (int i = 0; i < m; ++i) {
                    const int e = i + m * j;
                    A[BM(row, i, j)] = a_zero ? 0.0 : pbt_synth_uniform(jb->seed, 0, (uint32_t)s, row, e);
                    B[BM(row, i, j)] = pbt_synth_uniform(jb->seed, 1, (uint32_t)s, row, e);
                    C[BM(row, i, j)] = c_zero ? 0.0 : pbt_synth_uniform(jb->seed, 2, (uint32_t)s, row, e);
                }
            for (int i = 0; i < m; ++i) {
                double t = 0.0;
                for (int j = 0; j < m; ++j) t = t + fabs(A[BM(row, i, j)]);
                for (int j = 0; j < m; ++j) t = t + fabs(C[BM(row, i, j)]);
                for (int j = 0; j < m; ++j) t = t + fabs(B[BM(row, i, j)]);
                B[BM(row, i, i)] = B[BM(row, i, i)] + jb->delta * t;
                D[BV(row, i)] = pbt_synth_uniform(jb->seed, 3, (uint32_t)s, row, (uint32_t)i);
            }
        }
#undef BM
#undef BV
    }
    return NULL;
}

int pbt_synth_fill_batch(int kind, unsigned flags, int nsys, const int* m, const int* nrow, const long long* mat_off,
                         const long long* vec_off, uint64_t seed, double delta, double* A, double* B, double* C,
                         double* D, int nthreads) {
    if (nsys < 1 || !m || !nrow || !mat_off || !vec_off || !A || !B || !C || !D) return -1;
    if (kind != PBT_SYNTH_DOMINANT && kind != PBT_SYNTH_DIAGONAL) return -1;
    for (int s = 0; s < nsys; ++s)
        if (m[s] < 1 || m[s] > 16 || nrow[s] < 1) return -1;
    if (nthreads <= 0) {
        long n = sysconf(_SC_NPROCESSORS_ONLN);
        nthreads = n > 0 ? (int)n : 1;
    }
    if (nthreads > nsys) nthreads = nsys;
    batch_job* jobs = (batch_job*)calloc((size_t)nthreads, sizeof(batch_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) {
        free(jobs);
        free(th);
        return -1;
    }
    for (int t = 0; t < nthreads; ++t) {
        /* interleaved chunks balance long and short systems */
        const int base = nsys / nthreads, rem = nsys % nthreads;
        const int f = t * base + (t < rem ? t : rem);
        const int n = base + (t < rem ? 1 : 0);
        batch_job j = {kind, flags, nsys, m, nrow, mat_off, vec_off, seed, delta, A, B, C, D, f, f + n};
        jobs[t] = j;
    }
    for (int t = 1; t < nthreads; ++t) pthread_create(&th[t], NULL, fill_batch_chunk, &jobs[t]);
    fill_batch_chunk(&jobs[0]);
    for (int t = 1; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(jobs);
    free(th);
    return 0;
}

int pbt_synth_uneven_shapes(uint64_t seed, int nsys, int nmin, int nmax, int mmin, int mmax, int* n_out,
                            int* m_out) {
    if (nsys < 1 || nmin < 1 || nmax < nmin || mmin < 1 || mmax < mmin || !n_out || !m_out) return -1;
    const double lo = synth_log2((double)nmin), hi = synth_log2((double)nmax + 1.0);
    for (int s = 0; s < nsys; ++s) {
        uint32_t w[4];
        words(seed, 5, (uint32_t)s, 0, 0, w);
        const double u = u01(w[0], w[1]);
        int n = (int)floor(pbt_synth_exp2(lo + u * (hi - lo)));
        if (n < nmin) n = nmin;
        if (n > nmax) n = nmax;
        const double v = u01(w[2], w[3]);
        int mm = mmin + (int)floor(v * (double)(mmax - mmin + 1));
        if (mm > mmax) mm = mmax;
        n_out[s] = n;
        m_out[s] = mm;
    }
    return 0;
}
