// pbt_util.cuh -- small code-generation helpers shared by the kernels.
#pragma once

#include <cstddef>

namespace pbt {

// Hides a value from the optimiser.  Called once per row iteration (or
// phase) on the plane stride, it stops the compiler from hoisting the m*m
// 64-bit element addresses of a block out of the loop, where they would hold
// ~2*m*m registers for the whole kernel and force the blocks to spill.
__device__ __forceinline__ size_t opaque(size_t v) {
    asm volatile("" : "+l"(v));
    return v;
}

// Compiler barrier for memory operations: the front end does not move loads
// across it.  It emits no instruction, so the PTX assembler's own scheduler
// may still reorder; only a real memory operation (an mbarrier wait, a fence)
// constrains that.
__device__ __forceinline__ void mem_fence_compiler() { asm volatile("" ::: "memory"); }

// Barrier of the whole CTA for kernels whose warps go through the rows in
// step.  The form without .aligned (sm_70 and later): the threads of one warp
// may reach it from different instructions -- in a partial last CTA, the
// threads without a system take the same number of barriers on a path of
// their own -- and arrivals at barrier 0 count wherever they come from.
__device__ __forceinline__ void cta_row_barrier() { asm volatile("barrier.sync 0;" ::: "memory"); }

}  // namespace pbt
