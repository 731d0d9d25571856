/*
 * pbt_oracle.h -- CPU oracle for the batched block-tridiagonal solver.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of PaScaL_BTDMA's
 * MPI CPU path (Fortran_Original/src/mod_btdma_cpu.f90) run in one process:
 * the P MPI ranks of the reference become P contiguous segments of each line,
 * and its MPI_ALLTOALLV exchange becomes an index transpose in host memory.
 * Only tests/, the smoke check of __graft_entry__ and the CPU-baseline leg of
 * bench.py may load it, and only as the checker.  The product library never
 * links or calls it.
 *
 * Parity pins (see tests/test_oracle.py):
 *   - the Study "solution signatures" recorded by the reference itself
 *     (Study/result/btdma_solution_signature_260702_193138.csv), copied as
 *     numbers into tests/golden/signatures.json;
 *   - a dense LAPACK solve (numpy/scipy) of the assembled block-tridiagonal
 *     matrix on small cases;
 *   - the manufactured-solution workload of the reference samples
 *     (Fortran_Original/examples/btdma_cpu/sample_cpu.f90:115-176).
 *
 * Array layout (the reference GPU layout, Fortran column-major):
 *   matrix X(sys, row, i, j)  ->  X[sys + nsys*(row + N*(i + m*j))]
 *   vector D(sys, row, i)     ->  D[sys + nsys*(row + N*i)]
 * with i the row and j the column inside an m x m block
 * (CUDA_CXX_Port/include/pascal_btdma_cuda.hpp:46-65).
 */
#ifndef PBT_ORACLE_H
#define PBT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* LAPACK dgesv semantics on one column-major m x m system with nrhs columns:
 * LU with partial pivoting (first index of max |a| wins ties), row swaps
 * applied to the right-hand sides, unit-lower then non-unit-upper solves.
 * Returns info (0, or k>0 when U(k,k) is exactly zero; then b is untouched,
 * like dgesv). */
int pbto_dgesv(int m, int nrhs, double* a, int lda, double* b, int ldb);

/* Rows [first, last] (0-based, inclusive) of segment `seg` of a line of N rows
 * split into P segments; remainder rows go to the low segments.
 * Restates mpiutil_para (Fortran_Original/src/mpiutil.f90:27-48). */
void pbto_partition(int N, int P, int seg, int* first, int* last);

/* The full non-cyclic solve (mod_btdma_cpu.f90:242-271) for nsys systems of N
 * block rows split into P segments.  In place, like the reference:
 * D <- x, A <- A', C <- C' (modified-Thomas factors); B is not written.
 * nthreads <= 0 uses all host cores.  Returns 0, or a negative code for bad
 * arguments, or the number of systems in which some dgesv reported info>0. */
int pbto_solve_noncyclic(int m, int nsys, int N, int P,
                         double* A, double* B, double* C, double* D,
                         int nthreads);

/* The cyclic (periodic) solve (mod_btdma_cpu.f90:273-302): same local stage,
 * cyclic reduced solve btdma_many_cycl (mod_btdma_cpu.f90:80-183). */
int pbto_solve_cyclic(int m, int nsys, int N, int P,
                      double* A, double* B, double* C, double* D,
                      int nthreads);

/* Plain block Thomas on whole lines (btdma_many, mod_btdma_cpu.f90:15-78):
 * the P = 1 reduced-solve kernel applied directly to the data.  In place:
 * C <- C', D <- x. */
int pbto_block_thomas(int m, int nsys, int N,
                      double* A, double* B, double* C, double* D,
                      int nthreads);
/* A whole periodic line in one segment: btdma_many_cycl
 * (mod_btdma_cpu.f90:80-183) on the original rows, N >= 3. */
int pbto_block_thomas_cyclic(int m, int nsys, int N,
                             double* A, double* B, double* C, double* D,
                             int nthreads);

/* CPU-layout variants, X(m,m,nsys,N), D(m,nsys,N): what the CPU baseline times. */
int pbto_solve_noncyclic_cpu(int m, int nsys, int N, int P, double* A, double* B,
                             double* C, double* D, int nthreads);
int pbto_solve_cyclic_cpu(int m, int nsys, int N, int P, double* A, double* B,
                          double* C, double* D, int nthreads);
int pbto_block_thomas_cpu(int m, int nsys, int N, double* A, double* B, double* C,
                          double* D, int nthreads);
int pbto_block_thomas_cyclic_cpu(int m, int nsys, int N, double* A, double* B, double* C,
                                 double* D, int nthreads);

/* Layout transposes between the GPU layout and the CPU layout. */
void pbto_gpu_to_cpu(int m, int nsys, int N, int is_matrix, const double* g, double* c);
void pbto_cpu_to_gpu(int m, int nsys, int N, int is_matrix, const double* c, double* g);

/* Number of hardware threads the oracle uses when nthreads <= 0. */
int pbto_default_threads(void);

#ifdef __cplusplus
}
#endif
#endif
