// pbt_batch_pack.cu -- the batch's layout conversion between the caller's
// per-system arrays and the packed tiles (pbt_batch_pack / pbt_batch_unpack).
#include "pbt_batch_types.h"

namespace pbt {

// Packing between the caller's per-system layout (system s at its own
// offset, in the reference layout of a single system: X_s[row + N_s*e],
// e = i + m*j, D_s[row + N_s*i]) and the tiled layout.  One thread per
// (tile, row, lane); `sys_of` maps a tile lane to its system (-1 = empty).
__device__ __forceinline__ int find_tile(const long long* row_start, int ntiles, long long idx) {
    int lo = 0, hi = ntiles - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (row_start[mid] <= idx) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// dir = 0: user -> tiled (matrices and D); dir = 1: tiled D -> user D.
__global__ void k_pack(const PackArgs pa, const double* ua, const double* ub, const double* uc, const double* ud,
                       double* ta, double* tb, double* tc, double* td, double* ud_out, int dir) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= pa.total) return;
    const int t = find_tile(pa.row_start, pa.ntiles, idx);
    const long long local = idx - pa.row_start[t];
    const BatchTile tl = pa.tiles[t];
    const int row = (int)(local / 32), lane = (int)(local % 32);
    const int s = pa.sys_of[t * 32 + lane];
    const int n = pa.lane_rows[t * 32 + lane];
    const bool live = s >= 0 && row < n;
    const int m = tl.m;
    if (dir == 0) {
        // A system shorter than its tile is padded to the tile's rows with
        // rows that decouple (A = C = 0, B = I, d = 0: x = 0 there), and its
        // last real row's C is zeroed (the non-cyclic solve treats it as zero):
        // every lane of a tile then has the tile's rows and the same segment
        // boundaries, so a warp's accesses stay coalesced.
        const bool pad = s >= 0 && row >= n;
        for (int e = 0; e < m * m; ++e) {
            const size_t dst = (size_t)tl.mat_off + lane + (size_t)32 * (row + (size_t)tl.rows * e);
            const size_t src = live ? (size_t)pa.user_mat_off[s] + row + (size_t)n * e : 0;
            ta[dst] = live ? ua[src] : 0.0;
            tb[dst] = live ? ub[src] : ((pad && e % (m + 1) == 0) ? 1.0 : 0.0);
            tc[dst] = (live && row < n - 1) ? uc[src] : 0.0;
        }
        for (int i = 0; i < m; ++i) {
            const size_t dst = (size_t)tl.vec_off + lane + (size_t)32 * (row + (size_t)tl.rows * i);
            td[dst] = live ? ud[(size_t)pa.user_vec_off[s] + row + (size_t)n * i] : 0.0;
        }
    } else if (live) {
        for (int i = 0; i < m; ++i) {
            const size_t src = (size_t)tl.vec_off + lane + (size_t)32 * (row + (size_t)tl.rows * i);
            ud_out[(size_t)pa.user_vec_off[s] + row + (size_t)n * i] = td[src];
        }
    }
}

cudaError_t launch_pack(const PackArgs& pa, const double* ua, const double* ub, const double* uc, const double* ud,
                        double* ta, double* tb, double* tc, double* td, double* ud_out, int dir, cudaStream_t s) {
    if (pa.total <= 0) return cudaSuccess;
    k_pack<<<(unsigned)((pa.total + 255) / 256), 256, 0, s>>>(pa, ua, ub, uc, ud, ta, tb, tc, td, ud_out, dir);
    return cudaGetLastError();
}

}  // namespace pbt
