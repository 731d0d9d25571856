// pbt_batch.cuh -- one persistent launch for a batch of systems of uneven
// length N and mixed block size m (include/pbt_batch.h).
//
// Packed layout: the host sorts the systems by (m, N descending) and packs
// them into tiles of up to 32 systems of equal m.  A tile is the reference
// layout with 32 interleaved systems: element (i, j) of row r of lane l at
//   tile.mat_off + l + 32*(r + tile.rows*(i + m*j)),
// so a warp's accesses are contiguous 256-byte runs as in the uniform solve.
// Lanes keep their own N (<= tile.rows); rows beyond a lane's N are unused.
//
// Work: a tile with nseg = 1 is one item (block Thomas, thomas_body).  A tile
// with nseg = P > 1 gives P stage-1 items (modified elimination of segment s
// of every lane, modi_body) and P stage-3 items (update_body); the warp that
// completes a tile's last stage-1 item solves its reduced system
// (reduced_body) and publishes the tile as ready.  Stage-1 items are ordered
// by decreasing cost on the host (size-sorted queue); every warp pulls items
// from it, then from the stage-3 list, whose items wait -- boundedly -- for
// their tile to be ready.  Every warp of the persistent grid is resident, and
// every stage-1 item has been claimed by a running warp before any warp
// reaches stage 3, so the waits always end; a wait that runs past its limit
// sets the error word and the kernel returns.
#pragma once

#include "pbt_batch_types.h"
#include "pbt_kernels.cuh"

namespace pbt {

__device__ __forceinline__ int warp_claim(int* head) {
    int v = 0;
    if ((threadIdx.x & 31) == 0) v = atomicAdd(head, 1);
    return __shfl_sync(0xffffffffu, v, 0);
}

// The single-segment items of the float-float (and FP32) batch run the split
// form with rolled column loops (thomas_body_lu): one kernel holds the code
// of every block size, so code size matters even more than in k_thomas.
#ifndef PBT_BATCH_LU
#define PBT_BATCH_LU 1
#endif
template <class Num>
__host__ __device__ constexpr bool batch_uses_lu() {
    return PBT_BATCH_LU && Num::kConv;
}
// Shared memory a lane needs for thomas_body_lu at the largest batch block size.
constexpr int kBatchLuSlots = 5 * 5 + 5;

template <class Num, int M>
__device__ __forceinline__ void batch_stage1(const BatchArgs& ba, const BatchTile& tl, int t, int seg, unsigned& bad) {
    const int lane = threadIdx.x & 31;
    const size_t plane = (size_t)32 * tl.rows, rs = 32;
    const int n_lane = ba.lane_rows[t * 32 + lane];
    const bool active = lane < tl.lanes && n_lane >= 2;
    const size_t mo = (size_t)tl.mat_off + lane, vo = (size_t)tl.vec_off + lane;
    if (seg < 0) {
        if (active) {
            if constexpr (batch_uses_lu<Num>()) {
                extern __shared__ double batch_cps[];
                thomas_body_lu<Num, M>(ba.a + mo, ba.b + mo, ba.c + mo, ba.d + vo, ba.cw + mo,
                                       batch_cps + threadIdx.x, blockDim.x, plane, rs, n_lane, true, bad);
            } else {
                thomas_body<Num, M>(ba.a + mo, ba.b + mo, ba.c + mo, ba.d + vo, ba.cw + mo, plane, rs, n_lane, true,
                                    bad);
            }
        }
        return;
    }
    const size_t rplane = (size_t)32 * 2 * tl.nseg;
    if (active) {
        int f, l;
        seg_rows(n_lane, tl.nseg, seg, f, l);
        const size_t fo = (size_t)f * rs;
        modi_body<Num, M>(ba.a + mo + fo, ba.b + mo + fo, ba.c + mo + fo, ba.d + vo + fo, ba.aw + mo + fo,
                          ba.cw + mo + fo, plane, rs, l - f + 1, true, ba.ra + tl.red_mat_off + lane,
                          ba.rc + tl.red_mat_off + lane, ba.rd + tl.red_vec_off + lane, rplane, rs, seg, bad);
    }
    // Publish this segment; the warp completing the tile solves its reduced system.
    __threadfence();
    __syncwarp();
    int done = 0;
    if (lane == 0) done = atomicAdd(&ba.seg_done[t], 1);
    done = __shfl_sync(0xffffffffu, done, 0);
    if (done == tl.nseg - 1) {
        __threadfence();
        if (active)
            reduced_body<Num, M>(ba.ra + tl.red_mat_off + lane, ba.rc + tl.red_mat_off + lane,
                                 ba.rd + tl.red_vec_off + lane, rplane, rs, 2 * tl.nseg, bad);
        __threadfence();
        __syncwarp();
        if (lane == 0) atomicExch(&ba.ready[t], 1);
    }
}

template <class Num, int M>
__device__ __forceinline__ void batch_stage3(const BatchArgs& ba, const BatchTile& tl, int t, int seg, unsigned& bad) {
    const int lane = threadIdx.x & 31;
    const size_t plane = (size_t)32 * tl.rows, rs = 32;
    const int n_lane = ba.lane_rows[t * 32 + lane];
    if (lane >= tl.lanes || n_lane < 2) return;
    const size_t mo = (size_t)tl.mat_off + lane, vo = (size_t)tl.vec_off + lane;
    int f, l;
    seg_rows(n_lane, tl.nseg, seg, f, l);
    const size_t fo = (size_t)f * rs;
    unsigned amax = 0;
    update_body<Num, M>(ba.aw + mo + fo, ba.cw + mo + fo, ba.d + vo + fo, plane, rs, l - f + 1, true,
                        ba.rd + tl.red_vec_off + lane, (size_t)32 * 2 * tl.nseg, rs, seg, amax);
    bad |= range_bits<Num>(amax, false);
}

// Block sizes of the batch kernel: 1..kBatchMaxBlock (the host refuses
// larger m for batches).
constexpr int kBatchMaxBlock = 5;
#define PBT_BATCH_SWITCH(CALL)                                  \
    switch (tl.m) {                                             \
        case 1: CALL(1); break;                                 \
        case 2: CALL(2); break;                                 \
        case 3: CALL(3); break;                                 \
        case 4: CALL(4); break;                                 \
        default: CALL(5); break;                                \
    }

template <class Num>
__global__ void __launch_bounds__(128) k_batch(const BatchArgs ba) {
    unsigned bad = 0;
    // Stage 1 (and the reduced solves).
    while (true) {
        const int item = warp_claim(ba.head1);
        if (item >= ba.n1) break;
        const int2 it = ba.items1[item];
        const BatchTile tl = ba.tiles[it.x];
#define PBT_S1(MM) batch_stage1<Num, MM>(ba, tl, it.x, it.y, bad)
        PBT_BATCH_SWITCH(PBT_S1)
#undef PBT_S1
    }
    // Stage 3: wait (boundedly) until the item's tile is reduced, then update.
    while (true) {
        const int item = warp_claim(ba.head3);
        if (item >= ba.n3) break;
        const int2 it = ba.items3[item];
        int ok = 1;
        if ((threadIdx.x & 31) == 0) {
            long long spins = 0;
            while (atomicAdd(&ba.ready[it.x], 0) == 0) {
                if (++spins > ba.spin_limit || atomicAdd(ba.error, 0) != 0) {
                    ok = 0;
                    break;
                }
                __nanosleep(256);
            }
            if (!ok) atomicExch(ba.error, 1);
        }
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) break;
        __threadfence();
        const BatchTile tl = ba.tiles[it.x];
#define PBT_S3(MM) batch_stage3<Num, MM>(ba, tl, it.x, it.y, bad)
        PBT_BATCH_SWITCH(PBT_S3)
#undef PBT_S3
    }
    report_status(ba.status, bad);
}

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
static __global__ void k_pack(const PackArgs pa, const double* ua, const double* ub, const double* uc, const double* ud,
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
        for (int e = 0; e < m * m; ++e) {
            const size_t dst = (size_t)tl.mat_off + lane + (size_t)32 * (row + (size_t)tl.rows * e);
            const size_t src = live ? (size_t)pa.user_mat_off[s] + row + (size_t)n * e : 0;
            ta[dst] = live ? ua[src] : 0.0;
            tb[dst] = live ? ub[src] : 0.0;
            tc[dst] = live ? uc[src] : 0.0;
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

static inline cudaError_t launch_pack_impl(const PackArgs& pa, const double* ua, const double* ub, const double* uc,
                                    const double* ud, double* ta, double* tb, double* tc, double* td, double* ud_out,
                                    int dir, cudaStream_t s) {
    if (pa.total <= 0) return cudaSuccess;
    k_pack<<<(unsigned)((pa.total + 255) / 256), 256, 0, s>>>(pa, ua, ub, uc, ud, ta, tb, tc, td, ud_out, dir);
    return cudaGetLastError();
}

// Persistent launch: as many CTAs of `warps` warps as fit on the device.
template <class Num>
cudaError_t launch_batch(const BatchArgs& ba, int warps, cudaStream_t s, int* grid_out) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = batch_uses_lu<Num>() ? (size_t)32 * warps * kBatchLuSlots * sizeof(double) : 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<Num>, 32 * warps, smem);
    if (e != cudaSuccess) return e;
    const int grid = sms * (per_sm > 0 ? per_sm : 1);
    if (grid_out) *grid_out = grid;
    k_batch<Num><<<grid, 32 * warps, smem, s>>>(ba);
    return cudaGetLastError();
}

}  // namespace pbt
