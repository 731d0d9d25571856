/*
 * pbt_shared.h -- batches of lines that share one block-tridiagonal matrix,
 * solved in place in a strided field (part of libpbt.so).
 *
 * No single counterpart in the reference API; it replaces, for the
 * constant-coefficient ADI sweeps of the reference's heat3d example, the
 * sequence build matrix -> pack right-hand sides -> solve -> unpack:
 *   build_matrix_kernel  (Fortran_Original/examples/heat3d/heat3d_mpi_gpu.f90:439-509),
 *     which writes the same 2x2 blocks into A, B, C for every line,
 *   compute_rhs_*sweep_kernel / unpack_*sweep_kernel (same file), which copy
 *     between the field and the solver's (nsys, nblk, m) arrays,
 *   btdma_many_mpi_gpu_v2 on those arrays.
 * Here the matrix is given once (one system's blocks), factorised once on the
 * host in FP64 with partial pivoting, and a kernel solves every line directly
 * from a right-hand-side field into a solution field (which may be the same
 * array), addressing both with the caller's strides: no A, B, C arrays, no
 * packing.  Each row then moves 4*m doubles (d read, y written and read back,
 * x written) instead of 3m^2 + 2m.
 *
 * Line layout (pbt_lines): line s = s_in + nsys_inner * s_out, block row q,
 * unknown i of the row, at element offset
 *   s_in*stride_inner + s_out*stride_outer + q*row_stride + i*elem_stride
 * of the rhs and x arrays (double; offsets may not overlap between lines).
 * Threads go to consecutive s_in, so stride_inner = 1 gives coalesced access.
 * Example, heat3d's y-sweep over u(1-h:n1+h, 1-h:n2+h, 1-h:n3+h) with blocks
 * of two points (m = 2): lines over (i, k), stride_inner = 1,
 * stride_outer = (n1+2h)*(n2+2h), elem_stride = n1+2h, row_stride = 2*(n1+2h),
 * base pointer at u(1, 1, 1).
 */
#ifndef PBT_SHARED_H
#define PBT_SHARED_H

#include "pbt.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pbt_shared pbt_shared;

/* pbt_lines (pbt.h) gives where the m unknowns of each block row of each
 * line live in rhs and x. */
/* Factorise the matrix every line shares: a, b, c are HOST arrays of one
 * system, nrow*m*m doubles each, element (i, j) of row q at q + nrow*(i + m*j)
 * (the reference layout with nsys = 1); A_0 and C_{nrow-1} are ignored.  The
 * factorisation runs on the host in FP64; the factors go to device memory on
 * the current device.  precision: PBT_PREC_FP64 (the solve in FP64) or
 * PBT_PREC_FF (the solve in float-float arithmetic on the FP32 pipes, ~47
 * significant bits; factors must lie below 2^127 in magnitude, else
 * PBT_ERANGE), anything else PBT_EUNSUPPORTED.  Returns PBT_ESINGULAR (with
 * nothing created) if a zero pivot is met, PBT_EINVAL for bad sizes
 * (1 <= m <= PBT_MAX_BLOCK, nrow >= 2). */
int pbt_shared_create(pbt_shared** s, int m, int nrow, const double* a, const double* b, const double* c,
                      int precision);

/* x <- M^{-1} rhs for every line (device arrays; x may equal rhs).  The
 * solve uses x as its scratch: rows of x hold intermediate values until the
 * backward sweep overwrites them.  Asynchronous on `stream`. */
int pbt_shared_solve(const pbt_shared* s, const double* rhs, double* x, const pbt_lines* lines, void* stream);

/* Synchronises `stream` and reports the range check of the float-float
 * solves since the previous call (the rules of pbt_precision in pbt.h: a
 * right-hand-side value outside 2^-96 <= |x| < 2^96, an overflow, or a line
 * whose solution lies wholly below 2^-100): PBT_ERANGE if any line failed
 * (its solution is not valid), else PBT_OK.  Always PBT_OK for FP64. */
int pbt_shared_status(const pbt_shared* s, void* stream);

/* Block size and rows of the matrix. */
int pbt_shared_shape(const pbt_shared* s, int* m, int* nrow);

int pbt_shared_destroy(pbt_shared* s);

#ifdef __cplusplus
}
#endif
#endif
