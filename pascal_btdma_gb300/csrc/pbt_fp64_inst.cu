// pbt_fp64_inst.cu -- explicit instantiation of the FP64 kernels for one block
// size.  The build compiles this file once per M in 1..PBT_MAX_BLOCK with
// -DPBT_M=<M>, so the ten unrolled variants compile in parallel.
#include "pbt_fp64.cuh"

#ifndef PBT_M
#error "compile with -DPBT_M=<block size>"
#endif

namespace pbt {
template cudaError_t launch_fp64_thomas<PBT_M>(const SolveArgs&);
template cudaError_t launch_fp64_modi<PBT_M>(const SolveArgs&);
template cudaError_t launch_fp64_reduced<PBT_M>(const SolveArgs&);
template cudaError_t launch_fp64_reduced_cyclic<PBT_M>(const SolveArgs&);
template cudaError_t launch_fp64_update<PBT_M>(const SolveArgs&);
}  // namespace pbt
