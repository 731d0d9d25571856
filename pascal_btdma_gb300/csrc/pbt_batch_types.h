// pbt_batch_types.h -- descriptors shared by the batch host code
// (pbt_batch.cpp) and the persistent batch kernel (pbt_batch.cuh).
#pragma once

#include <cuda_runtime.h>

namespace pbt {

struct BatchTile {
    int m;
    int lanes;              // systems in the tile (<= 32)
    int rows;               // rows of the tile layout (largest N of its systems)
    int nseg;               // segments per system
    long long mat_off;      // doubles, in A/B/C and the factor workspace
    long long vec_off;      // doubles, in D
    long long red_mat_off;  // doubles, in the reduced A'/C' workspace
    long long red_vec_off;  // doubles, in the reduced d' workspace
};

struct BatchArgs {
    const double* a;
    const double* b;
    const double* c;
    double* d;
    double* aw;
    double* cw;
    double* ra;
    double* rc;
    double* rd;
    const BatchTile* tiles;
    const int* lane_rows;  // [tile*32 + lane]: N of that system, 0 for an empty lane
    const int2* items1;    // (tile, segment or -1 for a whole-line Thomas item)
    const int2* items3;    // (tile, segment)
    int n1, n3;
    int* head1;            // queue heads, zeroed before every solve
    int* head3;
    int* seg_done;         // per tile: segments done (zeroed before every solve)
    unsigned long long* status;  // zero pivots, range flag
};

// Packing between the caller's per-system layout and the tiled layout.
struct PackArgs {
    const BatchTile* tiles;
    const int* lane_rows;
    const int* sys_of;              // [tile*32 + lane]: system index, -1 = empty lane
    const long long* user_mat_off;  // per system
    const long long* user_vec_off;
    const long long* row_start;     // per tile: prefix sum of 32*rows
    int ntiles;
    long long total;                // sum over tiles of 32*rows
};

// The launches of block size M (pbt_batch.cuh; instantiated with the other
// kernels of (Num, M) in pbt_inst.cu).
template <class Num, int M>
cudaError_t launch_batch(const BatchArgs& ba, int warps, cudaStream_t s, int* grid_out);
cudaError_t launch_pack(const PackArgs& pa, const double* ua, const double* ub, const double* uc, const double* ud,
                        double* ta, double* tb, double* tc, double* td, double* ud_out, int dir, cudaStream_t s);

}  // namespace pbt
