// pbt_api.cpp -- the C ABI of include/pbt.h: plan object, argument checks,
// workspace, stage dispatch and phase timing.
//
// Stage sequence of one solve (reference: btdma_many_mpi_gpu_v2,
// Fortran_Original/src/mod_btdma_gpu_v2.f90:131-167, and solve_noncyclic_impl,
// CUDA_CXX_Port/src/pascal_btdma_cuda.cu:853-908):
//   nseg == 1, non-cyclic, not forced to the reference method:
//       one launch, plain block Thomas on the whole line.
//   otherwise:
//       local (modified elimination of every segment, reduced rows written
//       into the reduced system) -> reduced solve (non-cyclic or cyclic) ->
//       update.  The reference's two all-to-all exchanges have no
//       counterpart: the reduced rows never leave device memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "pbt_internal.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(PBT_ECUDA, m);
}

}  // namespace

struct pbt_plan {
    pbt_plan_desc desc;
    int device = 0;
    int sms = 0;          // multiprocessors of `device`
    bool thomas = false;  // single-segment plain block Thomas path
    bool cyclic_thomas = false;  // single-segment periodic block Thomas (k_thomas_cyclic)
    double* aw = nullptr;  // factor workspace (nullptr when in place)
    double* cw = nullptr;
    double* ra = nullptr;
    double* rc = nullptr;
    double* rd = nullptr;
    double* re = nullptr;  // cyclic fill-in column: reduced rows, or every row (cyclic_thomas)
    unsigned long long* status = nullptr;
    // Iterative refinement (PBT_PREC_FP32_REFINE): iterate X, correction /
    // residual E, convergence statistic, and the outcome of the last solve.
    double* rx = nullptr;
    double* re_ = nullptr;
    // Two-stage plans over few, long lines: the reduced system (identity
    // diagonal blocks `rb`) is solved by the same two-stage method through a
    // plan of its own instead of one thread per system.
    pbt_plan* sub = nullptr;
    double* rb = nullptr;
    // PBT_FLAG_CPU_LAYOUT: the inputs in the GPU layout the kernels read.
    double* la = nullptr;
    double* lb = nullptr;
    double* lc = nullptr;
    double* ld = nullptr;
    // Adjoint of a segmented plan: M^T's blocks, allocated on first use.
    double* at = nullptr;
    double* bt = nullptr;
    double* ct = nullptr;
    unsigned* rstat = nullptr;
    int last_iters = 0;
    double last_correction = 0.0;
    int refine_fail = PBT_OK;  // a refined solve that failed, until pbt_plan_status reports it
    size_t bytes = 0;
    cudaStream_t last_stream = nullptr;
    unsigned magic = 0x50425450u;  // "PBTP"
};

namespace {

constexpr unsigned kMagic = 0x50425450u;

int check_plan(const pbt_plan* p) {
    if (p == nullptr) return fail(PBT_ESTATE, "solve called with a null plan");
    if (p->magic != kMagic) return fail(PBT_ESTATE, "solve called with a destroyed or corrupt plan");
    return PBT_OK;
}

int pick_tpb(const pbt_plan* p, int work_items) {
    if (p->desc.threads_per_block > 0) return p->desc.threads_per_block;
    // Enough CTAs to cover every SM when the batch is small: the FP64 pipe is
    // the bound, so one warp per SM already saturates it.
    const int sms = p->sms > 0 ? p->sms : 1;
    int tpb = 128;
    while (tpb > 32 && ((long long)work_items + tpb - 1) / tpb < 2LL * sms) tpb /= 2;
    return tpb;
}

#define PBT_DISPATCH_M(NUM, FN)                                            \
    switch (m) {                                                           \
        case 1: return pbt::FN<NUM, 1>(g);                                 \
        case 2: return pbt::FN<NUM, 2>(g);                                 \
        case 3: return pbt::FN<NUM, 3>(g);                                 \
        case 4: return pbt::FN<NUM, 4>(g);                                 \
        case 5: return pbt::FN<NUM, 5>(g);                                 \
        case 6: return pbt::FN<NUM, 6>(g);                                 \
        case 7: return pbt::FN<NUM, 7>(g);                                 \
        case 8: return pbt::FN<NUM, 8>(g);                                 \
        case 9: return pbt::FN<NUM, 9>(g);                                 \
        case 10: return pbt::FN<NUM, 10>(g);                               \
        default: return cudaErrorInvalidValue;                             \
    }

// Arithmetic of a kernel launch: the plan's precision, except that the
// refined solve factors in FP32.
enum Arith { kF64 = 0, kFF = 1, kF32 = 2 };

int arith_of(int precision) {
    return precision == PBT_PREC_FF ? kFF : (precision == PBT_PREC_FP32_REFINE ? kF32 : kF64);
}

#define PBT_DISPATCH(NAME, FN)                                             \
    cudaError_t NAME(int arith, int m, const pbt::SolveArgs& g) {         \
        if (arith == kFF) {                                                \
            PBT_DISPATCH_M(pbt::FF, FN)                                    \
        }                                                                  \
        if (arith == kF32) {                                               \
            PBT_DISPATCH_M(pbt::F32, FN)                                   \
        }                                                                  \
        PBT_DISPATCH_M(pbt::F64, FN)                                       \
    }

#define PBT_DISPATCH_PLAIN_M2(NUM, FN, ...)                                \
    switch (m) {                                                           \
        case 1: return pbt::FN<NUM, 1>(__VA_ARGS__);                       \
        case 2: return pbt::FN<NUM, 2>(__VA_ARGS__);                       \
        case 3: return pbt::FN<NUM, 3>(__VA_ARGS__);                       \
        case 4: return pbt::FN<NUM, 4>(__VA_ARGS__);                       \
        case 5: return pbt::FN<NUM, 5>(__VA_ARGS__);                       \
        case 6: return pbt::FN<NUM, 6>(__VA_ARGS__);                       \
        case 7: return pbt::FN<NUM, 7>(__VA_ARGS__);                       \
        case 8: return pbt::FN<NUM, 8>(__VA_ARGS__);                       \
        case 9: return pbt::FN<NUM, 9>(__VA_ARGS__);                       \
        case 10: return pbt::FN<NUM, 10>(__VA_ARGS__);                     \
        default: return cudaErrorInvalidValue;                             \
    }

#define PBT_DISPATCH_PLAIN_M(FN, ...)                                      \
    switch (m) {                                                           \
        case 1: return pbt::FN<1>(__VA_ARGS__);                            \
        case 2: return pbt::FN<2>(__VA_ARGS__);                            \
        case 3: return pbt::FN<3>(__VA_ARGS__);                            \
        case 4: return pbt::FN<4>(__VA_ARGS__);                            \
        case 5: return pbt::FN<5>(__VA_ARGS__);                            \
        case 6: return pbt::FN<6>(__VA_ARGS__);                            \
        case 7: return pbt::FN<7>(__VA_ARGS__);                            \
        case 8: return pbt::FN<8>(__VA_ARGS__);                            \
        case 9: return pbt::FN<9>(__VA_ARGS__);                            \
        case 10: return pbt::FN<10>(__VA_ARGS__);                          \
        default: return cudaErrorInvalidValue;                             \
    }

cudaError_t run_adjoint(int arith, int m, const pbt::SolveArgs& g, const pbt::AdjointArgs& adj) {
    if (arith == kFF) {
        PBT_DISPATCH_PLAIN_M2(pbt::FF, launch_adjoint, g, adj)
    }
    PBT_DISPATCH_PLAIN_M2(pbt::F64, launch_adjoint, g, adj)
}
cudaError_t run_transpose_blocks(int m, const pbt::SolveArgs& g, double* At, double* Bt, double* Ct) {
    PBT_DISPATCH_PLAIN_M(launch_transpose_blocks, g, At, Bt, Ct)
}
cudaError_t run_gradients(int m, const pbt::SolveArgs& g, const pbt::AdjointArgs& adj) {
    PBT_DISPATCH_PLAIN_M(launch_gradients, g, adj)
}
cudaError_t run_residual(int m, const pbt::SolveArgs& g, const double* X, double* E) {
    PBT_DISPATCH_PLAIN_M(launch_residual, g, X, E)
}
cudaError_t run_accumulate(int m, const pbt::SolveArgs& g, double* X, const double* E, unsigned* stat) {
    PBT_DISPATCH_PLAIN_M(launch_accumulate, g, X, E, stat)
}
cudaError_t run_refine_step(int m, const pbt::SolveArgs& g, const pbt::RefineArgs& ra) {
    PBT_DISPATCH_PLAIN_M(launch_refine_step, g, ra)
}
cudaError_t run_refine_staged(int m, const pbt::SolveArgs& g, const pbt::ThomasMaps& maps, const pbt::RefineArgs& ra) {
    switch (m) {
        case 1: return pbt::launch_refine_staged<1>(g, maps, ra);
        case 2: return pbt::launch_refine_staged<2>(g, maps, ra);
        case 3: return pbt::launch_refine_staged<3>(g, maps, ra);
        case 4: return pbt::launch_refine_staged<4>(g, maps, ra);
        case 5: return pbt::launch_refine_staged<5>(g, maps, ra);
        case 6: return pbt::launch_refine_staged<6>(g, maps, ra);
        default: return cudaErrorInvalidValue;
    }
}

PBT_DISPATCH(run_thomas, launch_thomas)
PBT_DISPATCH(run_thomas_cyclic, launch_thomas_cyclic)

cudaError_t run_thomas_lines(int arith, int m, const pbt::SolveArgs& g, const pbt::LineStrides& ls) {
    if (arith == kFF) {
        PBT_DISPATCH_PLAIN_M2(pbt::FF, launch_thomas_lines, g, ls)
    }
    PBT_DISPATCH_PLAIN_M2(pbt::F64, launch_thomas_lines, g, ls)
}

#define PBT_DISPATCH_STAGED_M(NUM)                                         \
    switch (m) {                                                           \
        case 1: return pbt::launch_thomas_staged<NUM, 1>(g, maps);         \
        case 2: return pbt::launch_thomas_staged<NUM, 2>(g, maps);         \
        case 3: return pbt::launch_thomas_staged<NUM, 3>(g, maps);         \
        case 4: return pbt::launch_thomas_staged<NUM, 4>(g, maps);         \
        case 5: return pbt::launch_thomas_staged<NUM, 5>(g, maps);         \
        case 6: return pbt::launch_thomas_staged<NUM, 6>(g, maps);         \
        default: return cudaErrorNotSupported;                             \
    }
static_assert(pbt::kStagedMaxBlock == 6, "PBT_DISPATCH_STAGED_M lists block sizes 1..6");

cudaError_t run_thomas_staged(int arith, int m, const pbt::SolveArgs& g, const pbt::ThomasMaps& maps) {
    if (arith == kFF) {
        PBT_DISPATCH_STAGED_M(pbt::FF)
    }
    if (arith == kF32) {
        PBT_DISPATCH_STAGED_M(pbt::F32)
    }
    PBT_DISPATCH_STAGED_M(pbt::F64)
}

// cuTensorMapEncodeTiled, looked up once through the runtime (the library
// links no driver library).  Null if the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
        else
            cudaGetLastError();
    });
    return fn;
}

// The {nsys, nrow, planes} FP64 tensor at `base` (reference layout), boxes of
// one block column of 32 systems: {32, 1, m}.  False if the address or the
// strides break the TMA rules (16-byte aligned base, strides multiples of 16
// bytes, i.e. nsys even) or the driver refuses.
bool encode_columns(CUtensorMap* tm, const double* base, int nsys, int nrow, int planes, int m) {
    const PFN_cuTensorMapEncodeTiled_v12000 fn = tensor_map_encoder();
    if (fn == nullptr || base == nullptr || (reinterpret_cast<std::uintptr_t>(base) & 15u) != 0 || (nsys & 1))
        return false;
    const cuuint64_t dims[3] = {(cuuint64_t)nsys, (cuuint64_t)nrow, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)nsys * 8u, (cuuint64_t)nsys * (cuuint64_t)nrow * 8u};
    const cuuint32_t box[3] = {32u, 1u, (cuuint32_t)m};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    return fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The FP32 staged solve keeps C' as floats: the same tensor over 4-byte
// elements (strides multiples of 16 bytes: nsys a multiple of 4).
bool encode_columns_f32(CUtensorMap* tm, const double* base, int nsys, int nrow, int planes, int m) {
    const PFN_cuTensorMapEncodeTiled_v12000 fn = tensor_map_encoder();
    if (fn == nullptr || base == nullptr || (reinterpret_cast<std::uintptr_t>(base) & 15u) != 0 || (nsys & 3))
        return false;
    const cuuint64_t dims[3] = {(cuuint64_t)nsys, (cuuint64_t)nrow, (cuuint64_t)planes};
    const cuuint64_t strides[2] = {(cuuint64_t)nsys * 4u, (cuuint64_t)nsys * (cuuint64_t)nrow * 4u};
    const cuuint32_t box[3] = {32u, 1u, (cuuint32_t)m};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    return fn(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<double*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Launch the single-segment block Thomas solve, with TMA-staged loads
// (k_thomas_staged) or direct loads (k_thomas); both give the same bits.
// The default follows GB300 measurements (float-float unless noted, N = 256
// or 512): staged loads win for the FP32 factorisation of the refined solve,
// which is bound by memory (m = 5, 65536 systems: 11.5 vs 12.2 ms); for
// float-float only at m = 4 (16384 systems: 4.48 vs 5.54 ms) -- elsewhere
// the direct kernel with rolled column loops is faster even on small batches
// (m = 5, 16384 systems: 4.37 vs 6.02 ms); for FP64 at m = 5, 6 on batches
// under 8 warps per SM (m = 5, 16384 systems: 4.98 vs 5.24 ms).  The plan
// flags force either; staging also needs m <= 6, nsys >= 32, nsys even and
// 16-byte aligned arrays (the tensor-map rules), else direct loads run.
bool prefer_staged(int arith, int m, int nsys, int sms) {
    const bool small = sms <= 0 || (nsys + 31) / 32 < 8 * sms;
    if (arith == kF32) return true;
    if (arith == kFF) return m == 4 && small;
    return (m == 5 || m == 6) && small;
}

// Whether the single-segment solve of g runs with TMA-staged loads; if so,
// the tensor maps are filled.
bool thomas_stages(const pbt_plan* p, int arith, int m, const pbt::SolveArgs& g, pbt::ThomasMaps* maps) {
    const pbt_plan_desc& ds = p->desc;
    bool staged;
    if (ds.flags & PBT_FLAG_DIRECT_LOADS)
        staged = false;
    else if (ds.flags & PBT_FLAG_STAGED_LOADS)
        staged = true;
    else
        staged = prefer_staged(arith, m, g.nsys, p->sms);
    if (!staged || m > pbt::kStagedMaxBlock || g.nsys < 32) return false;
    const int mm = m * m;
    return encode_columns(&maps->a, g.a, g.nsys, g.nrow, mm, m) && encode_columns(&maps->b, g.b, g.nsys, g.nrow, mm, m) &&
           encode_columns(&maps->c, g.c, g.nsys, g.nrow, mm, m) && encode_columns(&maps->d, g.d, g.nsys, g.nrow, m, m) &&
           (arith == kF32 ? encode_columns_f32(&maps->w, g.cw, g.nsys, g.nrow, mm, m)
                          : encode_columns(&maps->w, g.cw, g.nsys, g.nrow, mm, m));
}

cudaError_t thomas_launch(const pbt_plan* p, int arith, int m, const pbt::SolveArgs& g) {
    pbt::ThomasMaps maps;
    return thomas_stages(p, arith, m, g, &maps) ? run_thomas_staged(arith, m, g, maps) : run_thomas(arith, m, g);
}

// Whether a two-stage plan solves its reduced system (nsys lines of `rn`
// rows) by the two-stage method again: when the lines are long and so few
// that one thread per line would leave the GPU nearly idle (GB300, m = 4,
// 256 lines of 32768 rows, P = 128: the 256-row reduced solve took 1.3 of
// 6.1 ms with 8 warps on 152 SMs).  Its segments have kSubSegRows rows.
constexpr int kSubSegRows = 8;
bool recursive_reduced(int nsys, int rn, int sms) {
    const int warps = (nsys + 31) / 32;
    return rn >= 8 * kSubSegRows && warps < 4 * (sms > 0 ? sms : 152);
}

// Identity blocks for every (system, row) of a {nsys, rn, m*m} array in the
// reference GPU layout.
int fill_identity(double* rb, int m, int nsys, int rn) {
    const size_t plane = (size_t)nsys * rn;
    cudaError_t e = cudaMemset(rb, 0, plane * m * m * sizeof(double));
    if (e == cudaSuccess) {
        double* ones = static_cast<double*>(std::malloc(plane * sizeof(double)));
        if (!ones) return fail(PBT_ENOMEM, "plan: host buffer for the identity blocks");
        for (size_t i = 0; i < plane; ++i) ones[i] = 1.0;
        for (int i = 0; i < m && e == cudaSuccess; ++i)
            e = cudaMemcpy(rb + (size_t)(i + m * i) * plane, ones, plane * sizeof(double), cudaMemcpyHostToDevice);
        std::free(ones);
    }
    return e == cudaSuccess ? PBT_OK : cuda_fail(e, "plan: identity blocks of the reduced system");
}

PBT_DISPATCH(run_modi, launch_modi)
PBT_DISPATCH(run_reduced, launch_reduced)
PBT_DISPATCH(run_reduced_cyclic, launch_reduced_cyclic)
PBT_DISPATCH(run_update, launch_update)

// Whether a batch fills the GPU with one thread per system: at least 4 warps
// per SM.  Measured on GB300: the m = 5 pencil batch (65536 systems, 13.5
// warps per SM) solves in 6.2 ms as one segment per line against 18.7 ms in 16
// segments (float-float); m = 4, 16384 systems (3.4 warps per SM): 4.55 ms in
// one segment, 4.51 ms in 8.
bool fills_gpu(int nsys, int sms) {
    const long long warps = (nsys + 31) / 32;
    return warps >= 4LL * (sms > 0 ? sms : 152);
}

// The local-stage and update launches put the segments in gridDim.y.
constexpr int kMaxSegments = 65535;

int validate(const pbt_plan_desc& d) {
    char buf[256];
    if (d.m < 1 || d.m > PBT_MAX_BLOCK) {
        std::snprintf(buf, sizeof buf, "plan: block size m=%d outside 1..%d", d.m, PBT_MAX_BLOCK);
        return fail(PBT_EINVAL, buf);
    }
    if (d.nsys <= 0 || d.nrow < 2) {
        std::snprintf(buf, sizeof buf, "plan: requires nsys > 0 and nrow >= 2 (nsys=%d, nrow=%d)", d.nsys, d.nrow);
        return fail(PBT_EINVAL, buf);
    }
    if (d.nseg < 1 || d.nseg > kMaxSegments || d.nrow < 2 * d.nseg) {
        std::snprintf(buf, sizeof buf,
                      "plan: nseg=%d must be in 1..%d with at least 2 rows per segment (nrow=%d)", d.nseg,
                      kMaxSegments, d.nrow);
        return fail(PBT_EINVAL, buf);
    }
    if (d.nseg > 1 && d.nrow < 3 * d.nseg) {
        // A 2-row segment makes the reference's reduced row 1 couple to the
        // next segment's first row instead of its own last row, so the
        // two-stage method returns a wrong x; refuse instead.
        std::snprintf(buf, sizeof buf,
                      "plan: with nseg=%d > 1 every segment needs >= 3 rows (nrow=%d < %d)", d.nseg, d.nrow,
                      3 * d.nseg);
        return fail(PBT_EINVAL, buf);
    }
    if ((d.flags & PBT_FLAG_CYCLIC) && d.nseg == 1) {
        // One segment: the whole-line periodic block Thomas.  The reference
        // method (modified elimination + cyclic reduced solve) needs a reduced
        // system of at least 4 rows, i.e. nseg >= 2.
        if (d.flags & PBT_FLAG_REFERENCE_METHOD)
            return fail(PBT_EINVAL, "plan: the reference method of the cyclic solve needs nseg >= 2 (a reduced "
                                    "system of at least 4 rows)");
        if (d.nrow < 3)
            return fail(PBT_EINVAL, "plan: a periodic line needs nrow >= 3");
    }
    if (d.precision != PBT_PREC_FP64 && d.precision != PBT_PREC_FF && d.precision != PBT_PREC_FP32_REFINE) {
        return fail(PBT_EUNSUPPORTED, "plan: unknown precision");
    }
    if (d.precision == PBT_PREC_FP32_REFINE) {
        if (d.flags & PBT_FLAG_INPLACE)
            return fail(PBT_EINVAL, "plan: the refined solve needs A and C unchanged for its FP64 residual "
                                    "(PBT_FLAG_INPLACE not allowed with PBT_PREC_FP32_REFINE)");
        if (d.flags & PBT_FLAG_CYCLIC)
            return fail(PBT_EUNSUPPORTED, "plan: PBT_PREC_FP32_REFINE is provided for non-cyclic lines only");
        if (!(d.tol > 0.0) || d.max_iter < 1 || d.max_iter > 100)
            return fail(PBT_EINVAL, "plan: refinement needs tol > 0 and 1 <= max_iter <= 100");
    }
    if (d.threads_per_block != 0 &&
        (d.threads_per_block < 32 || d.threads_per_block > 128 || d.threads_per_block % 32 != 0)) {
        return fail(PBT_EINVAL, "plan: threads_per_block must be 0 or a multiple of 32 in 32..128");
    }
    const unsigned known = PBT_FLAG_CYCLIC | PBT_FLAG_INPLACE | PBT_FLAG_REFERENCE_METHOD | PBT_FLAG_DIRECT_LOADS |
                           PBT_FLAG_STAGED_LOADS | PBT_FLAG_CPU_LAYOUT;
    if (d.flags & ~known) return fail(PBT_EINVAL, "plan: unknown flag bits");
    if ((d.flags & PBT_FLAG_DIRECT_LOADS) && (d.flags & PBT_FLAG_STAGED_LOADS))
        return fail(PBT_EINVAL, "plan: PBT_FLAG_DIRECT_LOADS and PBT_FLAG_STAGED_LOADS exclude each other");
    if ((d.flags & PBT_FLAG_CPU_LAYOUT) && (d.flags & PBT_FLAG_INPLACE))
        return fail(PBT_EUNSUPPORTED, "plan: PBT_FLAG_CPU_LAYOUT works on converted copies, so PBT_FLAG_INPLACE "
                                      "(factors written into the caller's A and C) is not provided with it");
    return PBT_OK;
}

void free_plan(pbt_plan* p) {
    if (p->sub) pbt_plan_destroy(p->sub);
    p->sub = nullptr;
    cudaFree(p->rb);
    p->rb = nullptr;
    cudaFree(p->la);
    cudaFree(p->lb);
    cudaFree(p->lc);
    cudaFree(p->ld);
    p->la = p->lb = p->lc = p->ld = nullptr;
    cudaFree(p->at);
    cudaFree(p->bt);
    cudaFree(p->ct);
    p->at = p->bt = p->ct = nullptr;
    cudaFree(p->rx);
    cudaFree(p->re_);
    cudaFree(p->rstat);
    p->rx = p->re_ = nullptr;
    p->rstat = nullptr;
    cudaFree(p->aw);
    cudaFree(p->cw);
    cudaFree(p->ra);
    cudaFree(p->rc);
    cudaFree(p->rd);
    cudaFree(p->re);
    cudaFree(p->status);
    p->aw = p->cw = p->ra = p->rc = p->rd = p->re = nullptr;
    p->status = nullptr;
}

int alloc(pbt_plan* p, double** ptr, size_t n) {
    if (n == 0) return PBT_OK;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(ptr), n * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        char buf[160];
        std::snprintf(buf, sizeof buf, "plan: cudaMalloc of %zu bytes failed: %s", n * sizeof(double),
                      cudaGetErrorString(e));
        return fail(e == cudaErrorMemoryAllocation ? PBT_ENOMEM : PBT_ECUDA, buf);
    }
    p->bytes += n * sizeof(double);
    return PBT_OK;
}

pbt::SolveArgs make_args(pbt_plan* p, double* a, double* b, double* c, double* d, cudaStream_t s,
                         int work_items) {
    const bool inplace = (p->desc.flags & PBT_FLAG_INPLACE) != 0;
    pbt::SolveArgs g;
    g.a = a;
    g.b = b;
    g.c = c;
    g.d = d;
    g.aw = inplace ? a : p->aw;
    g.cw = inplace ? c : p->cw;
    g.ra = p->ra;
    g.rc = p->rc;
    g.rd = p->rd;
    g.re = p->re;
    g.status = p->status;
    g.factors_raw = inplace ? 0 : 1;
    g.nsys = p->desc.nsys;
    g.nrow = p->desc.nrow;
    g.nseg = p->desc.nseg;
    g.tpb = pick_tpb(p, work_items);
    g.stream = s;
    g.sms = p->sms;
    g.tpb_auto = p->desc.threads_per_block == 0;
    return g;
}

struct EventSet {
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool ok = false;
    explicit EventSet(bool make) {
        if (!make) return;
        ok = true;
        for (auto& e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) ok = false;
    }
    ~EventSet() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
    }
};

// The refined solve: keep the right-hand side d in p->rx; x_1 = the FP32
// solve of M x = d (same kernels, F32 arithmetic, in place in D); then repeat
// { r = d - M x in FP64; solve M e = r in FP32; x += e } until the estimated
// remaining error, c_k^2 / c_{k-1} with c_k = max over systems of
// max|e|/max|x| (c_1 = 1: the first solve is a correction of size 1), is <=
// tol, or after max_iter FP32 solves.  x lives in D throughout, so the
// result needs no copy.  Synchronises the stream once per correction to test
// convergence.
int solve_refined(pbt_plan* p, double* a, double* b, double* c, double* d, cudaStream_t s) {
    const pbt_plan_desc& ds = p->desc;
    const int m = ds.m;
    const size_t nv = (size_t)ds.nsys * ds.nrow * ds.m;
    p->last_iters = 0;
    p->last_correction = 0.0;
    auto fp32_solve = [&](double* rhs) -> cudaError_t {
        if (p->thomas) return thomas_launch(p, kF32, m, make_args(p, a, b, c, rhs, s, ds.nsys));
        pbt::SolveArgs g = make_args(p, a, b, c, rhs, s, ds.nsys * ds.nseg);
        cudaError_t e = run_modi(kF32, m, g);
        if (e == cudaSuccess) e = run_reduced(kF32, m, make_args(p, a, b, c, rhs, s, ds.nsys));
        if (e == cudaSuccess) e = run_update(kF32, m, g);
        return e;
    };
    double* const rhs = p->rx;
    // A single-segment plan whose first pass runs the staged kernel keeps the
    // FP32 factors (in p->aw) and copies d into rhs as it reads it; its
    // corrections are then one fused pass each.  Otherwise: d copied first,
    // and residual, FP32 solve, accumulate per correction.
    pbt::SolveArgs g1 = make_args(p, a, b, c, d, s, ds.nsys);
    pbt::ThomasMaps maps1;
    const bool fused = p->thomas && p->aw != nullptr && m <= pbt::kStagedMaxBlock && thomas_stages(p, kF32, m, g1, &maps1);
    cudaError_t e;
    if (fused) {
        g1.ra = rhs;
        e = run_thomas_staged(kF32, m, g1, maps1);
    } else {
        e = cudaMemcpyAsync(rhs, d, nv * sizeof(double), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e, "refined solve: set-up copy");
        e = p->thomas ? thomas_launch(p, kF32, m, g1) : fp32_solve(d);
    }
    if (e != cudaSuccess) return cuda_fail(e, "refined solve: FP32 solve launch");
    p->last_iters = 1;
    p->last_correction = 1.0;
    const pbt::SolveArgs g64 = make_args(p, a, b, c, rhs, s, ds.nsys);
    double prev_ratio = 1.0;
    bool converged = false;
    for (int it = 1; it < ds.max_iter; ++it) {
        if ((e = cudaMemsetAsync(p->rstat, 0, sizeof(unsigned), s)) != cudaSuccess)
            return cuda_fail(e, "refined solve: statistic reset");
        if (fused) {
            const pbt::RefineArgs ra{reinterpret_cast<const float*>(p->aw), reinterpret_cast<float*>(p->re_), d,
                                     p->rstat};
            // The forward sweep's FP64 inputs through the TMA ring when the
            // maps encode (k_refine_staged), else plain loads (k_refine_step).
            const int mm = m * m;
            pbt::ThomasMaps maps{};
            if (encode_columns(&maps.a, a, ds.nsys, ds.nrow, mm, m) &&
                encode_columns(&maps.b, b, ds.nsys, ds.nrow, mm, m) &&
                encode_columns(&maps.c, c, ds.nsys, ds.nrow, mm, m) &&
                encode_columns(&maps.d, rhs, ds.nsys, ds.nrow, m, m))
                e = run_refine_staged(m, g64, maps, ra);
            else
                e = run_refine_step(m, g64, ra);
            if (e != cudaSuccess) return cuda_fail(e, "refined solve: correction launch");
        } else {
            if ((e = run_residual(m, g64, d, p->re_)) != cudaSuccess)
                return cuda_fail(e, "refined solve: residual launch");
            if ((e = fp32_solve(p->re_)) != cudaSuccess)
                return cuda_fail(e, "refined solve: FP32 correction launch");
            if ((e = run_accumulate(m, g64, d, p->re_, p->rstat)) != cudaSuccess)
                return cuda_fail(e, "refined solve: accumulate launch");
        }
        unsigned bits = 0;
        if ((e = cudaMemcpyAsync(&bits, p->rstat, sizeof bits, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return cuda_fail(e, "refined solve: convergence read");
        float ratio;
        std::memcpy(&ratio, &bits, sizeof ratio);
        p->last_iters = it + 1;
        p->last_correction = ratio;
        // Stop when the estimated error left after this correction,
        // ratio * rho with the contraction rho = ratio / previous ratio, is
        // below tol.
        if ((double)ratio * ((double)ratio / prev_ratio) <= ds.tol) {
            converged = true;
            break;
        }
        prev_ratio = ratio > 0.f ? (double)ratio : 1e-300;
    }
    // Reported by pbt_plan_status: a correction that came out Inf/NaN (the
    // FP32 solve could not carry the system), or tol not reached.
    if (!converged) p->refine_fail = std::isfinite(p->last_correction) ? PBT_ENOCONV : PBT_ERANGE;
    return PBT_OK;
}

int solve_core(pbt_plan* p, double* a, double* b, double* c, double* d, int m, int nsys, int nrow, bool cyclic,
               pbt_timings* t, cudaStream_t s);

// Argument checks, then the solve; a PBT_FLAG_CPU_LAYOUT plan converts A, B,
// C, D into its GPU-layout workspace first and the solution back after
// (its profiled `total` includes both conversions).
int solve_impl(pbt_plan* p, double* a, double* b, double* c, double* d, int m, int nsys, int nrow,
               bool cyclic, pbt_timings* t, void* stream) {
    int rc = check_plan(p);
    if (rc) return rc;
    const pbt_plan_desc& ds = p->desc;
    if (m != ds.m || nsys != ds.nsys || nrow != ds.nrow) {
        char buf[200];
        std::snprintf(buf, sizeof buf, "solve dimensions (m=%d, nsys=%d, nrow=%d) do not match the plan (%d, %d, %d)",
                      m, nsys, nrow, ds.m, ds.nsys, ds.nrow);
        return fail(PBT_EINVAL, buf);
    }
    if (cyclic != ((ds.flags & PBT_FLAG_CYCLIC) != 0)) {
        return fail(PBT_EINVAL, cyclic ? "cyclic solve on a plan created without PBT_FLAG_CYCLIC"
                                       : "non-cyclic solve on a plan created with PBT_FLAG_CYCLIC");
    }
    if (!a || !b || !c || !d) return fail(PBT_EINVAL, "solve: null array pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    p->last_stream = s;
    if (!(ds.flags & PBT_FLAG_CPU_LAYOUT)) return solve_core(p, a, b, c, d, m, nsys, nrow, cyclic, t, s);

    EventSet span(t != nullptr);
    if (t && !span.ok) return fail(PBT_ECUDA, "solve_profiled: cudaEventCreate failed");
    cudaError_t e = t ? cudaEventRecord(span.ev[0], s) : cudaSuccess;
    const int mm = m * m;
    if (e == cudaSuccess) e = pbt::launch_layout(a, p->la, mm, nsys, nrow, 0, s);
    if (e == cudaSuccess) e = pbt::launch_layout(b, p->lb, mm, nsys, nrow, 0, s);
    if (e == cudaSuccess) e = pbt::launch_layout(c, p->lc, mm, nsys, nrow, 0, s);
    if (e == cudaSuccess) e = pbt::launch_layout(d, p->ld, m, nsys, nrow, 0, s);
    if (e != cudaSuccess) return cuda_fail(e, "CPU-layout conversion in");
    rc = solve_core(p, p->la, p->lb, p->lc, p->ld, m, nsys, nrow, cyclic, t, s);
    if (rc) return rc;
    if ((e = pbt::launch_layout(p->ld, d, m, nsys, nrow, 1, s)) != cudaSuccess)
        return cuda_fail(e, "CPU-layout conversion out");
    if (t) {
        float tot = 0.f;
        if ((e = cudaEventRecord(span.ev[1], s)) != cudaSuccess || (e = cudaEventSynchronize(span.ev[1])) != cudaSuccess)
            return cuda_fail(e, "solve_profiled");
        cudaEventElapsedTime(&tot, span.ev[0], span.ev[1]);
        t->total = tot * 1e-3;
    }
    return PBT_OK;
}

int solve_core(pbt_plan* p, double* a, double* b, double* c, double* d, int m, int nsys, int nrow, bool cyclic,
               pbt_timings* t, cudaStream_t s) {
    int rc = PBT_OK;
    const pbt_plan_desc& ds = p->desc;
    const bool timed = (t != nullptr);
    EventSet evs(timed);
    if (timed && !evs.ok) return fail(PBT_ECUDA, "solve_profiled: cudaEventCreate failed");
    auto mark = [&](int i) -> cudaError_t { return timed ? cudaEventRecord(evs.ev[i], s) : cudaSuccess; };

    cudaError_t e;
    if ((e = mark(0)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    if (ds.precision == PBT_PREC_FP32_REFINE) {
        rc = solve_refined(p, a, b, c, d, s);
        if (rc) return rc;
        for (int i = 1; i < 5; ++i)
            if ((e = mark(i)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    } else if (p->thomas || p->cyclic_thomas) {
        const pbt::SolveArgs g = make_args(p, a, b, c, d, s, nsys);
        e = p->thomas ? thomas_launch(p, arith_of(ds.precision), m, g)
                      : run_thomas_cyclic(arith_of(ds.precision), m, g);
        if (e != cudaSuccess) return cuda_fail(e, "block Thomas launch");
        for (int i = 1; i < 5; ++i)
            if ((e = mark(i)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    } else {
        pbt::SolveArgs g = make_args(p, a, b, c, d, s, nsys * ds.nseg);
        e = run_modi(arith_of(ds.precision), m, g);
        if (e != cudaSuccess) return cuda_fail(e, "local-stage launch");
        if ((e = mark(1)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
        if ((e = mark(2)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
        pbt::SolveArgs g2 = make_args(p, a, b, c, d, s, nsys);
        if (!cyclic && p->sub) {
            // The reduced rows are raw values of the arithmetic; the sub-plan
            // reads and writes FP64, so float-float pairs are widened first
            // and the reduced solution split back after (with the line's
            // range check).  The blocks' entries below the float-float input
            // window -- A' and C' decay along long segments -- are zeroed on
            // the way: negligible next to the identity diagonal blocks, they
            // would otherwise read as out of range in the float-float sub-plan.
            const bool ff = arith_of(ds.precision) == kFF;
            const size_t rr = (size_t)nsys * 2 * ds.nseg;
            if (ff) {
                if ((e = pbt::launch_ff_raw_f64(p->ra, rr * m * m, 2, s)) != cudaSuccess ||
                    (e = pbt::launch_ff_raw_f64(p->rc, rr * m * m, 2, s)) != cudaSuccess ||
                    (e = pbt::launch_ff_raw_f64(p->rd, rr * m, 1, s)) != cudaSuccess)
                    return cuda_fail(e, "reduced system to FP64");
            }
            rc = solve_core(p->sub, p->ra, p->rb, p->rc, p->rd, m, nsys, 2 * ds.nseg, false, nullptr, s);
            if (rc) return rc;
            if (ff && (e = pbt::launch_reduced_to_ff(p->rd, nsys, 2 * ds.nseg, m, p->status, s)) != cudaSuccess)
                return cuda_fail(e, "reduced solution to float-float");
        } else {
            e = cyclic ? run_reduced_cyclic(arith_of(ds.precision), m, g2) : run_reduced(arith_of(ds.precision), m, g2);
            if (e != cudaSuccess) return cuda_fail(e, "reduced-stage launch");
        }
        if ((e = mark(3)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
        e = run_update(arith_of(ds.precision), m, g);
        if (e != cudaSuccess) return cuda_fail(e, "update-stage launch");
        if ((e = mark(4)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    }
    if (timed) {
        if ((e = cudaEventSynchronize(evs.ev[4])) != cudaSuccess) return cuda_fail(e, "solve_profiled");
        float ms[4] = {0, 0, 0, 0};
        for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&ms[i], evs.ev[i], evs.ev[i + 1]);
        float tot = 0;
        cudaEventElapsedTime(&tot, evs.ev[0], evs.ev[4]);
        if (p->thomas || p->cyclic_thomas) {
            // One fused launch: all of it is local compute.
            t->local_compute = tot * 1e-3;
            t->forward_exchange = t->reduced_compute = t->backward_exchange = t->update_compute = 0.0;
        } else {
            t->local_compute = ms[0] * 1e-3;
            t->forward_exchange = ms[1] * 1e-3;
            t->reduced_compute = ms[2] * 1e-3;
            t->backward_exchange = 0.0;
            t->update_compute = ms[3] * 1e-3;
        }
        t->total = tot * 1e-3;
    }
    return PBT_OK;
}

}  // namespace

int pbt::set_last_error(int code, const char* msg) { return fail(code, msg ? msg : ""); }

extern "C" {

void pbt_plan_desc_init(pbt_plan_desc* d) {
    if (!d) return;
    std::memset(d, 0, sizeof *d);
    d->nseg = 1;
    d->precision = PBT_PREC_FP64;
    d->tol = 1e-12;
    d->max_iter = 8;
}

int pbt_plan_create_ex(pbt_plan** out, const pbt_plan_desc* desc) {
    if (!out || !desc) return fail(PBT_EINVAL, "plan_create: null argument");
    *out = nullptr;
    int rc = validate(*desc);
    if (rc) return rc;
    pbt_plan* p = new (std::nothrow) pbt_plan();
    if (!p) return fail(PBT_ENOMEM, "plan_create: host allocation failed");
    p->desc = *desc;
    cudaGetDevice(&p->device);
    if (cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess) {
        cudaGetLastError();
        p->sms = 0;
    }
    const auto& d = *desc;
    const bool inplace = (d.flags & PBT_FLAG_INPLACE) != 0;
    const bool cyclic = (d.flags & PBT_FLAG_CYCLIC) != 0;
    // nseg is the reference's decomposition of a line over MPI ranks.  On one
    // GPU, a batch with enough systems to fill it is solved one segment per
    // line (the method of nseg = 1: ~40 % of the two-stage method's
    // arithmetic, same x to rounding) unless PBT_FLAG_REFERENCE_METHOD asks for
    // the segments.
    const bool one_seg = d.nseg == 1 || (!(d.flags & PBT_FLAG_REFERENCE_METHOD) && fills_gpu(d.nsys, p->sms) &&
                                         (!cyclic || d.nrow >= 3));
    p->thomas = one_seg && !cyclic && !(d.flags & PBT_FLAG_REFERENCE_METHOD);
    p->cyclic_thomas = one_seg && cyclic;
    const size_t mm = (size_t)d.m * d.m;
    const size_t rows = (size_t)d.nsys * d.nrow;
    const size_t rrows = (size_t)d.nsys * 2 * d.nseg;
    if (!inplace) {
        if ((rc = alloc(p, &p->cw, mm * rows))) goto fail_out;
        // aw: A' for the two-stage method; for a single-segment refined plan,
        // the FP32 factors its first pass keeps: per row and warp of 32
        // systems, m*m + 1 runs of 32 floats.
        const bool keep_lu = p->thomas && d.precision == PBT_PREC_FP32_REFINE && d.m <= pbt::kStagedMaxBlock;
        const size_t lu_doubles = (size_t)d.nrow * ((d.nsys + 31) / 32) * 16 * (mm + 1);
        if (!p->thomas && !p->cyclic_thomas && (rc = alloc(p, &p->aw, mm * rows))) goto fail_out;
        if (keep_lu && (rc = alloc(p, &p->aw, lu_doubles))) goto fail_out;
    }
    if (p->cyclic_thomas) {
        // The fill-in column of every row (also with PBT_FLAG_INPLACE).
        if ((rc = alloc(p, &p->re, mm * rows))) goto fail_out;
    } else if (!p->thomas) {
        if ((rc = alloc(p, &p->ra, mm * rrows))) goto fail_out;
        if ((rc = alloc(p, &p->rc, mm * rrows))) goto fail_out;
        if ((rc = alloc(p, &p->rd, (size_t)d.m * rrows))) goto fail_out;
        if (cyclic && (rc = alloc(p, &p->re, mm * rrows))) goto fail_out;
    }
    if (d.flags & PBT_FLAG_CPU_LAYOUT) {
        if ((rc = alloc(p, &p->la, mm * rows))) goto fail_out;
        if ((rc = alloc(p, &p->lb, mm * rows))) goto fail_out;
        if ((rc = alloc(p, &p->lc, mm * rows))) goto fail_out;
        if ((rc = alloc(p, &p->ld, (size_t)d.m * rows))) goto fail_out;
    }
    if (!p->thomas && !cyclic && d.precision != PBT_PREC_FP32_REFINE &&
        recursive_reduced(d.nsys, 2 * d.nseg, p->sms)) {
        // The reduced system: nsys lines of 2*nseg rows, B = I.
        const int rn = 2 * d.nseg;
        if ((rc = alloc(p, &p->rb, mm * rrows))) goto fail_out;
        if ((rc = fill_identity(p->rb, d.m, d.nsys, rn))) goto fail_out;
        pbt_plan_desc sd = d;
        sd.nrow = rn;
        sd.nseg = rn / kSubSegRows;
        sd.flags = 0;
        if ((rc = pbt_plan_create_ex(&p->sub, &sd))) goto fail_out;
        p->bytes += p->sub->bytes;
    }
    if (d.precision == PBT_PREC_FP32_REFINE) {
        const size_t nv = (size_t)d.m * rows;
        if ((rc = alloc(p, &p->rx, nv))) goto fail_out;
        if ((rc = alloc(p, &p->re_, nv))) goto fail_out;
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p->rstat), sizeof(unsigned));
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "plan_create: refinement statistic");
            goto fail_out;
        }
    }
    {
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p->status), sizeof(unsigned long long));
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "plan_create: status word");
            goto fail_out;
        }
        e = cudaMemset(p->status, 0, sizeof(unsigned long long));
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "plan_create: status word");
            goto fail_out;
        }
    }
    *out = p;
    return PBT_OK;
fail_out:
    free_plan(p);
    p->magic = 0;
    delete p;
    return rc;
}

int pbt_plan_create(pbt_plan** out, int m, int nsys, int nrow, int nseg) {
    pbt_plan_desc d;
    pbt_plan_desc_init(&d);
    d.m = m;
    d.nsys = nsys;
    d.nrow = nrow;
    d.nseg = nseg;
    return pbt_plan_create_ex(out, &d);
}

int pbt_plan_destroy(pbt_plan* p) {
    if (!p) return PBT_OK;
    if (p->magic != kMagic) return fail(PBT_ESTATE, "plan_destroy: destroyed or corrupt plan");
    free_plan(p);
    p->magic = 0;
    delete p;
    return PBT_OK;
}

int pbt_solve_noncyclic(pbt_plan* p, double* a, double* b, double* c, double* d, int m, int nsys, int nrow,
                        void* stream) {
    return solve_impl(p, a, b, c, d, m, nsys, nrow, false, nullptr, stream);
}

int pbt_solve_noncyclic_profiled(pbt_plan* p, double* a, double* b, double* c, double* d, int m, int nsys,
                                 int nrow, pbt_timings* t, void* stream) {
    pbt_timings local;
    return solve_impl(p, a, b, c, d, m, nsys, nrow, false, t ? t : &local, stream);
}

int pbt_solve_cyclic(pbt_plan* p, double* a, double* b, double* c, double* d, int m, int nsys, int nrow,
                     void* stream) {
    return solve_impl(p, a, b, c, d, m, nsys, nrow, true, nullptr, stream);
}

int pbt_solve_noncyclic_lines(pbt_plan* p, double* a, double* b, double* c, double* d, const pbt_lines* L,
                              void* stream) {
    int rc = check_plan(p);
    if (rc) return rc;
    const pbt_plan_desc& ds = p->desc;
    if (!a || !b || !c || !d || !L) return fail(PBT_EINVAL, "solve_lines: null argument");
    if (!p->thomas || (ds.flags & PBT_FLAG_CPU_LAYOUT) || ds.precision == PBT_PREC_FP32_REFINE)
        return fail(PBT_EUNSUPPORTED,
                    "solve_lines: needs a single-segment, non-cyclic FP64 or float-float plan in the GPU layout");
    if (L->nsys_inner <= 0 || L->nsys_outer <= 0 || (long long)L->nsys_inner * L->nsys_outer != ds.nsys) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "solve_lines: %d x %d lines for a plan of %d systems", L->nsys_inner,
                      L->nsys_outer, ds.nsys);
        return fail(PBT_EINVAL, buf);
    }
    if (L->stride_inner < 0 || L->stride_outer < 0 || L->row_stride < 0 || L->elem_stride < 0)
        return fail(PBT_EINVAL, "solve_lines: negative stride");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const pbt::LineStrides ls{L->nsys_inner, L->stride_inner, L->stride_outer, L->row_stride, L->elem_stride};
    const bool inplace = (ds.flags & PBT_FLAG_INPLACE) != 0;
    if (L->row_stride == 1 && L->stride_inner != 1) {
        // Rows contiguous, lines not (a sweep along the array's fast index):
        // one thread per line would read 32 lines per warp load.  Tiled
        // transposes into plan workspace (allocated on first use), the
        // reference-layout solve, and the solution (and, in place, C') back.
        const int m = ds.m, nsys = ds.nsys, nrow = ds.nrow;
        const size_t rows = (size_t)nsys * nrow, mmz = (size_t)m * m;
        if (!p->la) {
            const size_t bytes0 = p->bytes;
            if ((rc = alloc(p, &p->la, mmz * rows)) || (rc = alloc(p, &p->lb, mmz * rows)) ||
                (rc = alloc(p, &p->lc, mmz * rows)) || (rc = alloc(p, &p->ld, (size_t)m * rows))) {
                cudaFree(p->la);
                cudaFree(p->lb);
                cudaFree(p->lc);
                cudaFree(p->ld);
                p->la = p->lb = p->lc = p->ld = nullptr;
                p->bytes = bytes0;
                return rc;
            }
        }
        p->last_stream = s;
        cudaError_t e = pbt::launch_lines_layout(a, p->la, ls, m * m, nsys, nrow, 0, s);
        if (e == cudaSuccess) e = pbt::launch_lines_layout(b, p->lb, ls, m * m, nsys, nrow, 0, s);
        if (e == cudaSuccess) e = pbt::launch_lines_layout(c, p->lc, ls, m * m, nsys, nrow, 0, s);
        if (e == cudaSuccess) e = pbt::launch_lines_layout(d, p->ld, ls, m, nsys, nrow, 0, s);
        if (e != cudaSuccess) return cuda_fail(e, "solve_lines: transpose in");
        rc = solve_core(p, p->la, p->lb, p->lc, p->ld, m, nsys, nrow, false, nullptr, s);
        if (rc) return rc;
        e = pbt::launch_lines_layout(p->ld, d, ls, m, nsys, nrow, 1, s);
        if (e == cudaSuccess && inplace) e = pbt::launch_lines_layout(p->lc, c, ls, m * m, nsys, nrow, 1, s);
        if (e != cudaSuccess) return cuda_fail(e, "solve_lines: transpose out");
        return PBT_OK;
    }
    const long long mm = (long long)ds.m * ds.m;
    // One past the last element a block array is addressed at.
    const long long extent = (long long)(L->nsys_inner - 1) * L->stride_inner +
                             (long long)(L->nsys_outer - 1) * L->stride_outer +
                             (long long)(ds.nrow - 1) * L->row_stride + (mm - 1) * L->elem_stride + 1;
    if (!inplace && extent > mm * ds.nsys * ds.nrow)
        return fail(PBT_EUNSUPPORTED,
                    "solve_lines: the lines span more than the plan's factor workspace (nsys*nrow*m*m); "
                    "use a PBT_FLAG_INPLACE plan for a non-dense layout");
    p->last_stream = s;
    cudaError_t e = run_thomas_lines(arith_of(ds.precision), ds.m, make_args(p, a, b, c, d, s, ds.nsys), ls);
    if (e != cudaSuccess) return cuda_fail(e, "block Thomas launch (strided lines)");
    return PBT_OK;
}

int pbt_plan_status(pbt_plan* p, long long* nsingular) {
    int rc = check_plan(p);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(p->last_stream);
    if (e != cudaSuccess) return cuda_fail(e, "plan_status: stream synchronize");
    // The plan's status word and those of its reduced-system plans (layout
    // in pbt_internal.h), and the host-side outcome of the refined solve.
    unsigned long long pivots = 0, stalls = 0;
    bool range = false;
    for (pbt_plan* q = p; q != nullptr; q = q->sub) {
        unsigned long long w = 0;
        e = cudaMemcpy(&w, q->status, sizeof w, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "plan_status: read");
        e = cudaMemset(q->status, 0, sizeof w);
        if (e != cudaSuccess) return cuda_fail(e, "plan_status: reset");
        pivots += w & pbt::kPivotCountMask;
        range |= (w & pbt::kRangeMark) != 0;
        stalls += w / pbt::kStallMark;
    }
    const int refine = p->refine_fail;
    p->refine_fail = PBT_OK;
    if (nsingular) *nsingular = (long long)pivots;
    if (stalls) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "%llu bounded device wait(s) ran out; the solution is not valid", stalls);
        return fail(PBT_ETIMEOUT, buf);
    }
    if (range || refine == PBT_ERANGE)
        return fail(PBT_ERANGE, "a float-float / FP32 value left the arithmetic's range (an input outside "
                                "2^-96 <= |x| < 2^96, an overflow, or a solution below 2^-100); the solution is "
                                "not valid: solve with PBT_PREC_FP64");
    if (pivots) return fail(PBT_ESINGULAR, "a zero pivot was met in at least one block");
    if (refine == PBT_ENOCONV) {
        char buf[200];
        std::snprintf(buf, sizeof buf,
                      "the refined solve did not reach tol = %.3g in %d FP32 solves (last correction %.3g)",
                      p->desc.tol, p->last_iters, p->last_correction);
        return fail(PBT_ENOCONV, buf);
    }
    return PBT_OK;
}

int pbt_adjoint_noncyclic(pbt_plan* p, const double* a, const double* b, const double* c, const double* x,
                          double* g, double* da, double* db, double* dc, int m, int nsys, int nrow, void* stream) {
    int rc = check_plan(p);
    if (rc) return rc;
    const pbt_plan_desc& ds = p->desc;
    if (m != ds.m || nsys != ds.nsys || nrow != ds.nrow) {
        char buf[200];
        std::snprintf(buf, sizeof buf, "adjoint dimensions (m=%d, nsys=%d, nrow=%d) do not match the plan (%d, %d, %d)",
                      m, nsys, nrow, ds.m, ds.nsys, ds.nrow);
        return fail(PBT_EINVAL, buf);
    }
    if (!a || !b || !c || !x || !g) return fail(PBT_EINVAL, "adjoint: null array pointer");
    if (ds.flags & (PBT_FLAG_CYCLIC | PBT_FLAG_INPLACE | PBT_FLAG_CPU_LAYOUT))
        return fail(PBT_EUNSUPPORTED,
                    "adjoint: needs a non-cyclic plan without PBT_FLAG_INPLACE and without PBT_FLAG_CPU_LAYOUT");
    if (ds.precision == PBT_PREC_FP32_REFINE)
        return fail(PBT_EUNSUPPORTED, "adjoint: provided for the fp64 and ff precisions");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    p->last_stream = s;
    pbt::AdjointArgs adj;
    adj.x = x;
    adj.g = g;
    adj.da = da;
    adj.db = db;
    adj.dc = dc;
    const int arith = arith_of(ds.precision);
    cudaError_t e;
    if (p->thomas) {
        e = run_adjoint(arith, m, make_args(p, const_cast<double*>(a), const_cast<double*>(b),
                                            const_cast<double*>(c), g, s, ds.nsys), adj);
        if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
        return PBT_OK;
    }
    // Segmented plans: materialise M^T and solve it with the plan's own
    // forward method.
    if (!p->at) {
        const size_t n = (size_t)ds.m * ds.m * ds.nsys * ds.nrow;
        if ((rc = alloc(p, &p->at, n)) || (rc = alloc(p, &p->bt, n)) || (rc = alloc(p, &p->ct, n))) return rc;
    }
    const pbt::SolveArgs g0 = make_args(p, const_cast<double*>(a), const_cast<double*>(b), const_cast<double*>(c),
                                        g, s, ds.nsys);
    if ((e = run_transpose_blocks(m, g0, p->at, p->bt, p->ct)) != cudaSuccess)
        return cuda_fail(e, "adjoint: transpose launch");
    if (p->thomas) {
        e = thomas_launch(p, arith, m, make_args(p, p->at, p->bt, p->ct, g, s, ds.nsys));
        if (e != cudaSuccess) return cuda_fail(e, "adjoint: transposed solve launch");
    } else {
        pbt::SolveArgs gs = make_args(p, p->at, p->bt, p->ct, g, s, ds.nsys * ds.nseg);
        if ((e = run_modi(arith, m, gs)) != cudaSuccess ||
            (e = run_reduced(arith, m, make_args(p, p->at, p->bt, p->ct, g, s, ds.nsys))) != cudaSuccess ||
            (e = run_update(arith, m, gs)) != cudaSuccess)
            return cuda_fail(e, "adjoint: transposed solve launch");
    }
    if ((e = run_gradients(m, g0, adj)) != cudaSuccess) return cuda_fail(e, "adjoint: gradient launch");
    return PBT_OK;
}

int pbt_plan_refine_info(const pbt_plan* p, int* iterations, double* last_correction) {
    int rc = check_plan(p);
    if (rc) return rc;
    if (iterations) *iterations = p->last_iters;
    if (last_correction) *last_correction = p->last_correction;
    return PBT_OK;
}

int pbt_plan_get_desc(const pbt_plan* p, pbt_plan_desc* d) {
    int rc = check_plan(p);
    if (rc) return rc;
    if (!d) return fail(PBT_EINVAL, "plan_get_desc: null desc");
    *d = p->desc;
    return PBT_OK;
}

size_t pbt_plan_workspace_bytes(const pbt_plan* p) {
    if (!p || p->magic != kMagic) return 0;
    return p->bytes + sizeof(unsigned long long);
}

const char* pbt_last_error_string(void) { return g_last_error.c_str(); }

void pbt_partition_1d(int start, int end, int nparts, int part, int* first, int* last) {
    const int n = end - start + 1;
    const int base = n / nparts, rem = n % nparts;
    const int f = part * base + start + (part < rem ? part : rem);
    if (first) *first = f;
    if (last) *last = f + base - 1 + (rem > part ? 1 : 0);
}

int pbt_version(void) { return 100; }

}  // extern "C"
