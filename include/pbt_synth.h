/*
 * pbt_synth.h -- seeded synthetic block-tridiagonal workloads (libpbt_synth.so).
 *
 * Host-side generator for benchmarks and tests.  Every value is a pure
 * function of (seed, stream, system, row, element), drawn from a Philox4x32-10
 * counter-based stream (Salmon, Moraes, Dror, Shaw, "Parallel random numbers:
 * as easy as 1, 2, 3", SC'11), so the data does not depend on the thread
 * count, and all arithmetic is ordered IEEE double with no fused multiply-add,
 * so x86-64 and AArch64 hosts produce identical bytes.
 *
 * No counterpart in the reference's solver API; it replaces the initialisers
 * of its drivers: initialize_coefficients
 * (Study/example_cuda_cxx_btdma_profile.cu:53-74, the diagonal workload) and
 * demo_init (Fortran_Original/examples/btdma_cpu/sample_cpu.f90:115-176, a
 * manufactured solution).
 *
 * Layout: the reference GPU layout of include/pbt.h.
 */
#ifndef PBT_SYNTH_H
#define PBT_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Workload kinds for pbt_synth_fill. */
#define PBT_SYNTH_DOMINANT 0   /* A, C, d, R iid U[-1,1); B = R + diag(delta*rowsum(|A|+|C|+|R|)) */
#define PBT_SYNTH_DIAGONAL 1   /* A = 0.25 I, B = 2 I, C = 0.25 I, d = 1 (the reference Study workload) */
#define PBT_SYNTH_MANUFACTURED 2 /* x_ref(row,i) = 100*(row+1) + (i+1); A, C ~ U(-0.4,0.4); B = I - (A + C); d = M x_ref */

/* Flags for pbt_synth_fill. */
#define PBT_SYNTH_ZERO_ENDS 0x1u  /* A_0 = 0 and C_{N-1} = 0 explicitly (DOMINANT, MANUFACTURED) */
#define PBT_SYNTH_ROW_SCALE 0x2u  /* scale each block row (A, B, C, d) by a log-uniform factor in [1e-3, 1e3] */

/* Philox4x32-10 block function. */
void pbt_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* The uniform double in [-1, 1) the generator assigns to
 * (seed, stream, sys, row, elem): 53 random bits from words 0 and 1 of
 * Philox4x32-10 at counter (sys, row, elem | stream << 16, 0), key = seed. */
double pbt_synth_uniform(uint64_t seed, uint32_t stream, uint32_t sys, uint32_t row, uint32_t elem);

/* Fill A, B, C (nsys*N*m*m doubles each) and D (nsys*N*m) with a workload.
 * x_ref (nsys*N*m, may be NULL) receives the exact solution for
 * PBT_SYNTH_MANUFACTURED.  nthreads <= 0 uses all host cores.
 * Returns 0, or -1 on bad arguments. */
int pbt_synth_fill(int kind, unsigned flags, int m, int nsys, int N, uint64_t seed, double delta,
                   double* A, double* B, double* C, double* D, double* x_ref, int nthreads);

/* An uneven batch in the per-system layout of include/pbt_batch.h: system s
 * (block size m[s], length nrow[s]) at matrix offset mat_off[s] and vector
 * offset vec_off[s], each in the reference layout of a single system.  The
 * values of system s are those pbt_synth_fill gives system index s of a
 * uniform batch with the same m and nrow (counter sys = s), for the
 * DOMINANT and DIAGONAL kinds.  Threads split the systems. */
int pbt_synth_fill_batch(int kind, unsigned flags, int nsys, const int* m, const int* nrow,
                         const long long* mat_off, const long long* vec_off, uint64_t seed, double delta,
                         double* A, double* B, double* C, double* D, int nthreads);

/* Per-system shapes of the uneven batch: N log-uniform integer in
 * [nmin, nmax], m uniform in [mmin, mmax]; stream 5 of the seed. */
int pbt_synth_uneven_shapes(uint64_t seed, int nsys, int nmin, int nmax, int mmin, int mmax,
                            int* n_out, int* m_out);

/* 2^t for |t| < 1024, evaluated by a fixed Horner polynomial so that the
 * result is identical on every IEEE host (libm's exp2 is not). */
double pbt_synth_exp2(double t);

#ifdef __cplusplus
}
#endif
#endif
