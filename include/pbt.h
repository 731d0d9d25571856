/*
 * pbt.h -- C ABI of the GB300 batched block-tridiagonal solver (libpbt.so).
 *
 * Drop-in for PaScaL_BTDMA's plan / solve / destroy path:
 *
 *   reference (Fortran, Fortran_Original/src/mod_btdma_gpu_v2.f90)
 *     btdma_makeplan_gpu_v2(plan, m, nsys, nrow_sub, comm)   :70-109
 *     btdma_many_mpi_gpu_v2(A, B, C, D, m, nsys, nrow_sub, plan) :131-167
 *     btdma_many_mpi_gpu_v2_profiled(..., plan, timing)     :169-198
 *     btdma_many_cycl_mpi_gpu_v2(A, B, C, D, m, nsys, nrow_sub, plan) :200-239
 *     btdma_cleanplan_gpu_v2(plan)                          :111-129
 *   reference (C++, CUDA_CXX_Port/include/pascal_btdma_cuda.hpp)
 *     BtdmaGpuPlan::create(m, nsys, nrow, comm, mode)       :128-132
 *     solve_noncyclic(plan, a, b, c, d, m, nsys, nrow, stream) :137-145
 *     solve_noncyclic_profiled(..., timings, stream)        :147-156
 *     solve_cyclic(plan, a, b, c, d, m, nsys, nrow, stream) :158-166
 *     BtdmaGpuPlan::destroy()                               :134
 *
 * One GPU replaces the reference's MPI communicator: the `comm` argument
 * becomes `nseg`, the number P of segments each line is split into (one
 * segment per former MPI rank), and `nrow` is the FULL line length N (all P
 * segments live in the same arrays).  With nseg = 1 the call is identical to
 * a one-rank reference call.
 *
 * Arrays are device pointers in the reference GPU layout (column-major
 * Fortran A(nsys, nrow, m, m), D(nsys, nrow, m)):
 *   A[sys + nsys*(row + nrow*(i + m*j))],  D[sys + nsys*(row + nrow*i)]
 * or, for plans created with PBT_FLAG_CPU_LAYOUT, in the layout of the
 * reference CPU path (Fortran a(m, m, nsys, n), d(m, nsys, n),
 * Fortran_Original/src/mod_btdma_cpu.f90:18-19):
 *   A[i + m*(j + m*(sys + nsys*row))],  D[i + m*(sys + nsys*row)]
 * (such a plan converts on the device through workspace of the size of the
 * inputs; not with PBT_FLAG_INPLACE or the adjoint).
 * with (i, j) the row and column inside the m x m block
 * (pascal_btdma_cuda.hpp:46-65).  System `sys` solves
 *   A_q x_{q-1} + B_q x_q + C_q x_{q+1} = d_q,   q = 0 .. nrow-1,
 * where the non-cyclic solve never reads A_0 or C_{nrow-1} (they act as
 * zero, as in the reference) and the cyclic solve couples row 0 to row
 * nrow-1 through them.
 *
 * In-place contract (as in the reference, mod_btdma_gpu_v2.f90:618-919):
 * D is overwritten with the solution x.  B is never written.  A and C are
 * not written either unless the plan was created with PBT_FLAG_INPLACE, in
 * which case they receive the elimination factors (the reference's A', C')
 * and the plan needs no factor workspace.
 *
 * Errors: every entry point returns a pbt_status instead of throwing;
 * pbt_last_error_string() gives the message of the last failure on the
 * calling thread (the reference throws CudaError / std::invalid_argument /
 * std::runtime_error / std::logic_error, pascal_btdma_cuda.hpp:20-22 and
 * pascal_btdma_cuda.cu:862-870, 912-919, 956-967, 1063-1075).
 *
 * Threading: a plan owns device workspace; two solves on one plan must not
 * overlap on the GPU (same rule as the reference plan).  Solves are
 * asynchronous on `stream` (a cudaStream_t; NULL = legacy default stream)
 * and never synchronise the host, except the *_profiled entry, which
 * synchronises to read its event timings.
 */
#ifndef PBT_H
#define PBT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBT_MAX_BLOCK 10

typedef enum pbt_status {
    PBT_OK = 0,
    PBT_EINVAL = 1,       /* bad argument or plan/array mismatch (std::invalid_argument) */
    PBT_ECUDA = 2,        /* a CUDA runtime call failed (CudaError) */
    PBT_ESTATE = 3,       /* null or destroyed plan (std::runtime_error) */
    PBT_EUNSUPPORTED = 4, /* combination not provided (std::logic_error) */
    PBT_ENOMEM = 5,       /* device workspace allocation failed */
    PBT_ESINGULAR = 6,    /* a zero pivot was met in some block (pbt_plan_status) */
    PBT_ETIMEOUT = 7,     /* a bounded device-side wait ran out (pbt_plan_status); results invalid */
    PBT_ERANGE = 8,       /* a float-float / FP32 value left the arithmetic's range (pbt_plan_status);
                             results invalid: solve with PBT_PREC_FP64 */
    PBT_ENOCONV = 9       /* the refined solve did not reach desc.tol in desc.max_iter FP32 solves
                             (pbt_plan_status) */
} pbt_status;

/* Arithmetic of the solve.
 *
 * Range of the float-float method.  Its values are pairs of FP32 numbers, so
 * it has FP32's exponent range, not FP64's.  It accepts input entries (A, B,
 * C, D, and the adjoint's dL/dx) that are zero or of magnitude
 * 2^-96 <= |v| < 2^96 (about 1.3e-29 to 7.9e28).  Any other entry (a nonzero
 * entry below 2^-96, one at or above 2^96, Inf, NaN), any overflow on the way,
 * and any system whose solution lies wholly below 2^-100 in magnitude (where
 * the pairs lose their 47 bits) turn the solve into a reported failure:
 * pbt_plan_status returns PBT_ERANGE and the solution must not be used.  The
 * outcome is never a silently wrong number.  Solve such systems with
 * PBT_PREC_FP64, which has the reference's own range.
 * The FP32-refined method reads entries below 2^-126 as zero and fails on
 * entries at or above 2^128; its FP64 residual corrects the rest.  A
 * refinement that cannot converge is reported: PBT_ERANGE if a correction came
 * out Inf/NaN, else PBT_ENOCONV. */
typedef enum pbt_precision {
    PBT_PREC_FP64 = 0,        /* plain FP64 arithmetic, partial-pivot LU per block */
    PBT_PREC_FF = 1,          /* FP64 data, float-float (two-FP32) arithmetic on the FP32 pipes */
    PBT_PREC_FP32_REFINE = 2  /* FP32 factorisation + FP64-residual iterative refinement (non-cyclic) */
} pbt_precision;

/* Plan flags. */
#define PBT_FLAG_CYCLIC 0x1u           /* periodic lines: plan for pbt_solve_cyclic */
#define PBT_FLAG_INPLACE 0x2u          /* A, C receive the elimination factors; no factor workspace */
#define PBT_FLAG_REFERENCE_METHOD 0x4u /* always run the two-stage (modified Thomas) method on the nseg segments, even at nseg = 1 or for a batch that fills the GPU */
#define PBT_FLAG_DIRECT_LOADS 0x8u     /* single-segment solve: always direct global loads */
#define PBT_FLAG_STAGED_LOADS 0x10u    /* single-segment solve: TMA-staged loads wherever allowed (m <= 6,
                                          nsys >= 32 and even, 16-byte aligned arrays) */
/* Neither load flag: the library picks per solve (same results either way). */
#define PBT_FLAG_CPU_LAYOUT 0x20u      /* a, b, c, d are in the reference CPU layout (see below) */

typedef struct pbt_plan_desc {
    int m;                 /* block size, 1..PBT_MAX_BLOCK */
    int nsys;              /* number of independent systems */
    int nrow;              /* block rows per system (full line length N) */
    int nseg;              /* segments per line (P), 1..65535; >= 3 rows each when P > 1 */
    int precision;         /* pbt_precision */
    unsigned flags;        /* PBT_FLAG_* */
    double tol;            /* PBT_PREC_FP32_REFINE: target relative correction size */
    int max_iter;          /* PBT_PREC_FP32_REFINE: refinement iteration cap */
    int threads_per_block; /* 0 = choose automatically (float-float kernels whose
                              CTAs keep their warps on the same row take up to 256
                              threads); else a multiple of 32 in 32..128, used as is */
    int reserved[7];
} pbt_plan_desc;

/* Phase times of one solve in seconds; the same six fields as the
 * reference's BtdmaSolveTimings (pascal_btdma_cuda.hpp:24-39) and
 * BTDMA_TIMING_gpu_v2 (mod_btdma_gpu_v2.f90:38-45).  On one GPU the two
 * exchange phases move no data and read as the time of the (empty)
 * interval between the compute phases. */
typedef struct pbt_timings {
    double total;
    double local_compute;
    double forward_exchange;
    double reduced_compute;
    double backward_exchange;
    double update_compute;
} pbt_timings;

typedef struct pbt_plan pbt_plan;

/* Fill `desc` with defaults: nseg = 1, FP64, no flags, tol = 1e-12,
 * max_iter = 8. */
void pbt_plan_desc_init(pbt_plan_desc* desc);

/* Replaces BtdmaGpuPlan::create(m, nsys, nrow, comm) (pascal_btdma_cuda.cu:956-1005)
 * and btdma_makeplan_gpu_v2 (mod_btdma_gpu_v2.f90:70-109): validates the
 * sizes and allocates the device workspace on the current device.
 * Non-cyclic, FP64.
 * nseg stands for the reference's MPI ranks.  A batch large enough to fill
 * the GPU with one thread per system (nsys >= 128 * SMs, 19456 on a GB300)
 * is solved one segment per line whatever nseg says: the single-segment
 * method does ~40 % of the two-stage method's arithmetic and gives the same x
 * to rounding.  PBT_FLAG_REFERENCE_METHOD keeps the nseg segments (and the
 * reference's in-place A', C' with PBT_FLAG_INPLACE). */
int pbt_plan_create(pbt_plan** plan, int m, int nsys, int nrow, int nseg);

/* As pbt_plan_create with every option of pbt_plan_desc. */
int pbt_plan_create_ex(pbt_plan** plan, const pbt_plan_desc* desc);

/* Replaces BtdmaGpuPlan::destroy (pascal_btdma_cuda.cu:1007-1033) and
 * btdma_cleanplan_gpu_v2 (mod_btdma_gpu_v2.f90:111-129).  NULL is a no-op. */
int pbt_plan_destroy(pbt_plan* plan);

/* Replaces solve_noncyclic (pascal_btdma_cuda.cu:1035-1045, impl :853-908)
 * and btdma_many_mpi_gpu_v2 (mod_btdma_gpu_v2.f90:131-167).  m, nsys, nrow
 * must equal the plan's (PBT_EINVAL otherwise, like the reference's check at
 * pascal_btdma_cuda.cu:868-870).
 * Graph capture: the first solve of a kind (block size, arithmetic, method)
 * on a device loads its kernels there and sets their launch attributes
 * (register count query, shared-memory size); make one such solve before
 * capturing solves in a CUDA graph. */
int pbt_solve_noncyclic(pbt_plan* plan, double* a, double* b, double* c, double* d,
                        int m, int nsys, int nrow, void* stream);

/* Replaces solve_noncyclic_profiled (pascal_btdma_cuda.cu:1047-1061) and
 * btdma_many_mpi_gpu_v2_profiled (mod_btdma_gpu_v2.f90:169-198).  `timings`
 * may be NULL.  Synchronises `stream`. */
int pbt_solve_noncyclic_profiled(pbt_plan* plan, double* a, double* b, double* c, double* d,
                                 int m, int nsys, int nrow, pbt_timings* timings, void* stream);

/* Replaces solve_cyclic (pascal_btdma_cuda.cu:1063-1075, which throws in the
 * reference port) and btdma_many_cycl_mpi_gpu_v2 (mod_btdma_gpu_v2.f90:200-239).
 * The plan must carry PBT_FLAG_CYCLIC.  nseg >= 2 runs the two-stage method
 * with the cyclic reduced solve (btdma_many_cycl, mod_btdma_cpu.f90:80-183);
 * nseg = 1 (nrow >= 3) runs btdma_many_cycl's periodic block Thomas on the
 * whole line in one launch, with the fill-in column in plan workspace
 * (nsys * nrow * m * m doubles, also with PBT_FLAG_INPLACE, where C' goes into
 * C and A stays untouched).  FP64 and PBT_PREC_FF. */
int pbt_solve_cyclic(pbt_plan* plan, double* a, double* b, double* c, double* d,
                     int m, int nsys, int nrow, void* stream);

/* Lines addressed by strides: line s = s_in + nsys_inner * s_out, block row
 * q, element e of the row's block (e = i + m*j for A, B, C; e = i for D) at
 * element offset
 *   s_in*stride_inner + s_out*stride_outer + q*row_stride + e*elem_stride.
 * The reference GPU layout is {nsys, 1, 1, 0, nsys, nsys*nrow}.  Threads go
 * to consecutive s_in: stride_inner = 1 keeps the loads coalesced. */
typedef struct pbt_lines {
    int nsys_inner;         /* lines along the fast index (threads) */
    int nsys_outer;         /* lines along the slow index */
    long long stride_inner; /* element offset between consecutive inner lines */
    long long stride_outer; /* element offset between consecutive outer lines */
    long long row_stride;   /* element offset between block rows of a line */
    long long elem_stride;  /* element offset between the elements of a row */
} pbt_lines;

/* Non-cyclic solve of lines that live in the caller's own arrays, addressed
 * by `lines` (the same strides for A, B, C and D).
 *
 * No single counterpart in the reference API: it removes the transposes that
 * the reference's applications run around each solve to bring their arrays
 * into the solver layout, e.g. euler3d's transpose_jk / transpose_ik kernels
 * and their 5-D block versions (Fortran_Original/examples/euler3d/
 * euler3d_mpi_gpu.f90:931-1017) around btdma_many_mpi_gpu_v2: with
 * U(n1,n2,n3,m) and trA(n1,n2,n3,m,m) the y sweep is
 *   {n1, n3, 1, n1*n2, n1, n1*n2*n3}.
 * The plan must be a non-cyclic FP64 or PBT_PREC_FF plan solved one
 * segment per line (nseg = 1, or a batch that fills the GPU; no
 * PBT_FLAG_REFERENCE_METHOD / PBT_FLAG_CPU_LAYOUT) with
 * nsys = nsys_inner * nsys_outer; otherwise PBT_EUNSUPPORTED / PBT_EINVAL.
 * A PBT_FLAG_INPLACE plan writes C' into C, as the reference does; any other
 * plan keeps its factors in its workspace, addressed with the same strides,
 * so the lines must then fit in nsys*nrow*m*m elements (a dense layout, as
 * euler3d's), else PBT_EUNSUPPORTED.  Lines whose rows are contiguous
 * (row_stride 1, stride_inner != 1: a sweep along the array's fast index,
 * which one thread per line would read uncoalesced) are transposed into plan
 * workspace (the inputs' size, allocated on the first such call), solved in
 * the reference layout and transposed back; no extent rule applies there.
 * That first call allocates (cudaMalloc, which may synchronise the device and
 * is not allowed during stream capture): make one such call before capturing
 * a graph of these solves. */
int pbt_solve_noncyclic_lines(pbt_plan* plan, double* a, double* b, double* c, double* d,
                              const pbt_lines* lines, void* stream);

/* Solve without a plan and without allocating device memory.
 *
 * No counterpart in the reference.  It exists for callers that cannot call
 * cudaMalloc: applications that give all device memory to their own pool
 * allocator at start-up and forbid later allocations, and time-stepping loops
 * that must not call cudaMalloc / cudaFree (which can synchronise the device)
 * while other streams are busy.  Every plan-based entry allocates workspace
 * in pbt_plan_create; this one allocates nothing: it runs the two-stage method
 * (nseg segments per line; nseg = 1 runs it with one segment) in place --
 * A <- A', C <- C', D <- x, exactly the reference's side effects -- and keeps
 * its only scratch, the reduced system, in a fixed array of 4 Mi doubles
 * (32 MiB) compiled into the library, held on every GPU that loads the library
 * until the process exits.
 *
 * Limit: nsys * 2 * nseg * (2*m*m + m) doubles, each of the three reduced
 * arrays rounded up to a multiple of 32, must fit in 4 Mi doubles; larger
 * calls return PBT_EINVAL with the sizes in pbt_last_error_string().  Other
 * argument rules as pbt_plan_create (1 <= nseg <= 65535).  Every call looks
 * up the array's device address (cudaGetSymbolAddress) on the current device,
 * so a device reset between calls is harmless; the first call on a device
 * also loads the library's device code there, so make that first call before
 * any stream capture.  All calls share the array
 * and it keeps the previous call's contents (each call rewrites what it
 * reads), so two calls that overlap on the GPU race: serialise them on one
 * stream.  Zero pivots are not reported by this entry. */
int pbt_solve_noncyclic_noalloc(double* a, double* b, double* c, double* d,
                                int m, int nsys, int nrow, int nseg, void* stream);

/* Adjoint of the non-cyclic solve x = M^{-1} d (no counterpart in the
 * reference).  On entry g holds dL/dx for a scalar loss L; on return it holds
 * lambda = M^{-T} dL/dx = dL/dd, and da, db, dc (each nsys*nrow*m*m doubles,
 * reference layout; any may be NULL) receive
 *   dL/dA_q = -lambda_q x_{q-1}^T,  dL/dB_q = -lambda_q x_q^T,  dL/dC_q = -lambda_q x_{q+1}^T,
 * with dL/dA_0 = dL/dC_{nrow-1} = 0.  x is the forward solution and a, b, c
 * the forward blocks, unchanged (the plan must not be PBT_FLAG_INPLACE).
 * nseg = 1 (every m): one fused kernel solves M^T lambda = g by block Thomas
 * on the transposed blocks, read in place, and forms the gradient blocks in
 * its backward sweep.  nseg > 1: M^T's blocks are materialised in plan
 * workspace (allocated by the first such call), solved by the plan's forward
 * method, and the gradients formed in one more pass.  Precision fp64 or ff. */
int pbt_adjoint_noncyclic(pbt_plan* plan, const double* a, const double* b, const double* c,
                          const double* x, double* g, double* da, double* db, double* dc,
                          int m, int nsys, int nrow, void* stream);

/* Synchronises the plan's last stream and reports through *nsingular how
 * many zero pivots the solves since the previous call met (the reference has
 * no such report; its dgesv-less GPU path divides by zero silently).  Returns,
 * in this order of precedence: PBT_ETIMEOUT if a kernel's bounded wait for its
 * staged input ran out; PBT_ERANGE if a float-float or FP32 solve left its
 * arithmetic's range (see pbt_precision); PBT_ESINGULAR when *nsingular > 0;
 * PBT_ENOCONV if a refined solve did not reach its tolerance.  After
 * PBT_ETIMEOUT and PBT_ERANGE the solution of that solve is not valid.  The
 * call clears what it reports.  nsingular may be NULL. */
int pbt_plan_status(pbt_plan* plan, long long* nsingular);

/* Outcome of the last solve on a PBT_PREC_FP32_REFINE plan: the number of
 * FP32 solves it ran (the first solve plus the corrections) and the last
 * correction size c_k = max over systems of max|e| / max|x|.  The refined
 * solve stops once the estimated remaining error c_k^2 / c_{k-1} (c_0 = 1,
 * the first solve) is <= desc.tol, or after desc.max_iter solves, and
 * synchronises its stream once per solve to test it.  Zeros for other
 * precisions.  No counterpart in the reference. */
int pbt_plan_refine_info(const pbt_plan* plan, int* iterations, double* last_correction);

/* Copies the plan's creation parameters into *desc. */
int pbt_plan_get_desc(const pbt_plan* plan, pbt_plan_desc* desc);

/* Device workspace owned by the plan, in bytes. */
size_t pbt_plan_workspace_bytes(const pbt_plan* plan);

/* Message of the last failed call on this thread ("" if none). */
const char* pbt_last_error_string(void);

/* Rows [first, last] of part `part` of the inclusive range [start, end]
 * split into `nparts` parts, the remainder going to the low parts.
 * Replaces partition_1d (pascal_btdma_cuda.cu:921-930) and mpiutil_para
 * (Fortran_Original/src/mpiutil.f90:27-48, there 1-based). */
void pbt_partition_1d(int start, int end, int nparts, int part, int* first, int* last);

/* Library version as an integer, major*10000 + minor*100 + patch. */
int pbt_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PBT_H */
