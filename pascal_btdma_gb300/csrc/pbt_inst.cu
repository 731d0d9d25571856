// pbt_inst.cu -- explicit instantiation of the solver kernels for one
// arithmetic and one block size.  The build compiles this file once per
// (PBT_NUM, PBT_M), PBT_NUM in {F64, FF, F32} and PBT_M in 1..PBT_MAX_BLOCK, so the
// unrolled variants compile in parallel.
#if !defined(PBT_M) || !defined(PBT_NUM)
#error "compile with -DPBT_M=<block size> -DPBT_NUM=<F64|FF>"
#endif

#if PBT_M > 6
#define PBT_UNROLL _Pragma("unroll 1")
#endif

#include "pbt_kernels.cuh"
#if PBT_M <= 6
#include "pbt_staged.cuh"
#endif
#if defined(PBT_NUM_IS_F64) || defined(PBT_NUM_IS_FF)
#include "pbt_batch.cuh"
#endif

namespace pbt {
template cudaError_t launch_thomas<PBT_NUM, PBT_M>(const SolveArgs&);
template cudaError_t launch_thomas_lines<PBT_NUM, PBT_M>(const SolveArgs&, const LineStrides&);
template cudaError_t launch_thomas_cyclic<PBT_NUM, PBT_M>(const SolveArgs&);
#if PBT_M <= 6
template cudaError_t launch_thomas_staged<PBT_NUM, PBT_M>(const SolveArgs&, const ThomasMaps&);
#endif
template cudaError_t launch_modi<PBT_NUM, PBT_M>(const SolveArgs&);
template cudaError_t launch_reduced<PBT_NUM, PBT_M>(const SolveArgs&);
template cudaError_t launch_reduced_cyclic<PBT_NUM, PBT_M>(const SolveArgs&);
template cudaError_t launch_update<PBT_NUM, PBT_M>(const SolveArgs&);
template cudaError_t launch_adjoint<PBT_NUM, PBT_M>(const SolveArgs&, const AdjointArgs&);
#if defined(PBT_NUM_IS_F64) || defined(PBT_NUM_IS_FF)
template cudaError_t launch_batch<PBT_NUM, PBT_M>(const BatchArgs&, int, cudaStream_t, int*);
#endif
#ifdef PBT_NUM_IS_F64
template cudaError_t launch_transpose_blocks<PBT_M>(const SolveArgs&, double*, double*, double*);
template cudaError_t launch_gradients<PBT_M>(const SolveArgs&, const AdjointArgs&);
template cudaError_t launch_residual<PBT_M>(const SolveArgs&, const double*, double*);
template cudaError_t launch_accumulate<PBT_M>(const SolveArgs&, double*, const double*, unsigned*);
template cudaError_t launch_refine_step<PBT_M>(const SolveArgs&, const RefineArgs&);
#if PBT_M <= 6
template cudaError_t launch_refine_staged<PBT_M>(const SolveArgs&, const ThomasMaps&, const RefineArgs&);
#endif
#endif
}  // namespace pbt
