// pbt_batch_f64.cu -- the persistent batch kernel for the F64 arithmetic
// (one translation unit per arithmetic so the two compile in parallel).
#include "pbt_batch.cuh"

namespace pbt {
template cudaError_t launch_batch<F64>(const BatchArgs&, int, cudaStream_t, int*);
cudaError_t launch_pack(const PackArgs& pa, const double* ua, const double* ub, const double* uc, const double* ud,
                        double* ta, double* tb, double* tc, double* td, double* ud_out, int dir, cudaStream_t s) {
    return launch_pack_impl(pa, ua, ub, uc, ud, ta, tb, tc, td, ud_out, dir, s);
}
}  // namespace pbt
