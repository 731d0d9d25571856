// pbt_batch_ff.cu -- the persistent batch kernel for the FF arithmetic
// (one translation unit per arithmetic so the two compile in parallel).
#include "pbt_batch.cuh"

namespace pbt {
template cudaError_t launch_batch<FF>(const BatchArgs&, int, cudaStream_t, int*);
}  // namespace pbt
