// pbt_internal.h -- plan object and kernel-launch interface shared by the
// C ABI (pbt_api.cpp) and the per-block-size kernel objects (*_inst.cu).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>

#include "../../include/pbt.h"

namespace pbt {

// Arguments of one solve as the kernels see them.  All arrays use the
// reference GPU layout (see include/pbt.h); the reduced-system arrays use the
// same layout with nrow replaced by 2*nseg:
//   ra[sys + nsys*(r + 2*nseg*(i + m*j))], rd[sys + nsys*(r + 2*nseg*i)].
struct SolveArgs {
    const double* a;  // A (read; also written when aw == a)
    const double* b;  // B (read only)
    const double* c;  // C (read; also written when cw == c)
    double* d;        // D: right-hand side in, solution out
    double* aw;       // where the factors A' go: == a (in place) or workspace
    double* cw;       // where the factors C' go: == c (in place) or workspace
    double* ra;       // reduced rows: A'
    double* rc;       // reduced rows: C'
    double* rd;       // reduced rows: d', then the reduced solution
    double* re;       // cyclic fill-in column of the reduced system
    unsigned long long* status;  // zero pivots met
    int factors_raw;  // 1: aw/cw are workspace (raw arithmetic values); 0: caller's A/C (FP64)
    int nsys;
    int nrow;
    int nseg;
    int tpb;  // threads per block
    cudaStream_t stream;
    int sms = 0;       // SMs of the device (0: unknown)
    int tpb_auto = 0;  // 1: the CTA size is the library's choice (kernels may pick their own)
};

// Strided lines (pbt_solve_noncyclic_lines): line sys at
// (sys % lin)*in + (sys / lin)*out, rows `row` apart, elements `elem` apart,
// in A, B, C, D and the factor array alike.
struct LineStrides {
    int lin;
    long long in, out, row, elem;
};

// The arithmetics of pbt_num.cuh.
struct F64;
struct FF;
struct F32;

// Tensor maps of the TMA-staged single-segment solve (pbt_staged.cuh): A, B,
// C as {nsys, nrow, m*m} tensors, D as {nsys, nrow, m}, the factor
// workspace (or C when in place) as {nsys, nrow, m*m}; every box is one block
// column of 32 systems, {32, 1, m}.
struct ThomasMaps {
    CUtensorMap a, b, c, d, w;
};
// Largest block size with a staged kernel (larger blocks do not fit in the
// registers of one thread anyway and keep the direct-load kernel).
constexpr int kStagedMaxBlock = 6;
// A plan's status word: bits 0..46 count the threads that met a zero pivot,
// bit 47 is set (atomicOr) by a thread whose float-float / FP32 solution left
// the arithmetic's range, and kStallMark is added once per bounded wait that
// ran out.
constexpr unsigned long long kStallMark = 1ull << 48;
constexpr unsigned long long kRangeMark = 1ull << 47;
constexpr unsigned long long kPivotCountMask = kRangeMark - 1;

// Kernel launchers, explicitly instantiated per arithmetic and block size M
// (1..PBT_MAX_BLOCK) in pbt_inst.cu.  Each returns cudaGetLastError().
template <class Num, int M> cudaError_t launch_thomas(const SolveArgs& g);
template <class Num, int M> cudaError_t launch_thomas_lines(const SolveArgs& g, const LineStrides& ls);
// Lines with row stride 1 <-> the reference GPU layout, E element planes
// (dir 0: lines -> reference; dir 1: back).
cudaError_t launch_lines_layout(const double* src, double* dst, const LineStrides& ls, int E, int nsys, int nrow,
                                int dir, cudaStream_t s);
template <class Num, int M> cudaError_t launch_thomas_staged(const SolveArgs& g, const ThomasMaps& maps);
// Periodic lines in one segment (k_thomas_cyclic): the fill-in column in
// g.re, nsys * nrow * m * m raw values; nrow >= 3.
template <class Num, int M> cudaError_t launch_thomas_cyclic(const SolveArgs& g);
template <class Num, int M> cudaError_t launch_modi(const SolveArgs& g);
template <class Num, int M> cudaError_t launch_reduced(const SolveArgs& g);
template <class Num, int M> cudaError_t launch_reduced_cyclic(const SolveArgs& g);
template <class Num, int M> cudaError_t launch_update(const SolveArgs& g);
// Adjoint (pbt_kernels.cuh: k_adjoint, k_transpose_blocks, k_gradients).
struct AdjointArgs {
    const double* x;  // forward solution
    double* g;        // in: dL/dx; out: lambda = dL/dd
    double* da;       // gradient blocks (may be null)
    double* db;
    double* dc;
};
template <class Num, int M> cudaError_t launch_adjoint(const SolveArgs& g, const AdjointArgs& adj);
template <int M> cudaError_t launch_transpose_blocks(const SolveArgs& g, double* At, double* Bt, double* Ct);
template <int M> cudaError_t launch_gradients(const SolveArgs& g, const AdjointArgs& adj);
// FP64 parts of the refined solve (instantiated with the F64 kernels).
template <int M> cudaError_t launch_residual(const SolveArgs& g, const double* X, double* E);
template <int M> cudaError_t launch_accumulate(const SolveArgs& g, double* X, const double* E, unsigned* stat);

// One correction of the refined solve with stored FP32 factors
// (k_refine_step): lu = the factors the staged FP32 pass kept (per row and
// warp of 32 systems, m*m + 1 runs of 32 floats), y = float scratch of
// nsys*nrow*m, x = the FP64 solution (updated), stat = the convergence
// statistic.
struct RefineArgs {
    const float* lu;
    float* y;
    double* x;
    unsigned* stat;
};
template <int M> cudaError_t launch_refine_step(const SolveArgs& g, const RefineArgs& ra);
template <int M> cudaError_t launch_refine_staged(const SolveArgs& g, const ThomasMaps& maps, const RefineArgs& ra);

// Layout conversion for PBT_FLAG_CPU_LAYOUT plans (pbt_layout.cu): E elements
// per (system, row); dir 0: CPU layout src -> GPU layout dst, 1: back.
cudaError_t launch_layout(const double* src, double* dst, int E, int nsys, int nrow, int dir, cudaStream_t s);
// In place, n 8-byte slots: raw float-float pairs -> FP64 (to_f64 = 1; 2
// also zeroes values below 2^-96) or back (0).
cudaError_t launch_ff_raw_f64(double* x, size_t n, int to_f64, cudaStream_t s);
// The reduced solution rd (nsys systems, `rows` rows of m values) from FP64
// back to raw float-float pairs, with the line's range check into `status`.
cudaError_t launch_reduced_to_ff(double* rd, int nsys, int rows, int m, unsigned long long* status, cudaStream_t s);

// Records the message returned by pbt_last_error_string() on this thread and
// returns `code` (defined in pbt_api.cpp).
int set_last_error(int code, const char* msg);

}  // namespace pbt
