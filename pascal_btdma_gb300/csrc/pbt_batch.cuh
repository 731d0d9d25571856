// pbt_batch.cuh -- persistent launches for a batch of systems of uneven
// length N and mixed block size m (include/pbt_batch.h).
//
// Packed layout: the host sorts the systems by (m, N descending) and packs
// them into tiles of up to 32 systems of equal m.  A tile is the reference
// layout with 32 interleaved systems: element (i, j) of row r of lane l at
//   tile.mat_off + l + 32*(r + tile.rows*(i + m*j)),
// so a warp's accesses are contiguous 256-byte runs as in the uniform solve.
// The packing pads every system to its tile's rows with decoupled rows
// (B = I, A = C = 0, d = 0), so all lanes share the tile's row partition.
//
// Work, per block size M present, in two launches on the caller's stream
// (float-float m = 5, 6 keep each CTA's warps in step in the first: a CTA
// claims one item per warp at a time, and every thread takes the same number
// of barriers each round):
//   k_batch_local   persistent over the stage-1 items, ordered by decreasing
//                   cost on the host (size-sorted queue): a tile with
//                   nseg = 1 is one item (block Thomas on every lane); a
//                   tile with nseg = P > 1 gives P items (the modified
//                   elimination of one segment of every lane), each writing
//                   its two reduced rows; the warp that completes a tile's
//                   last segment solves its 2P-row reduced system;
//   k_batch_update  persistent over the stage-3 items (the interior update of
//                   one segment of every lane).
// The kernel boundaries order the stages, so no warp ever waits on another
// (a tile's reduced system is solved by the warp that finishes it last, found
// with an atomic counter).
// Each launch carries one block size's code, with the bodies and register
// budget k_thomas / k_modi use for that size.
#pragma once

#include "pbt_batch_types.h"
#include "pbt_kernels.cuh"

namespace pbt {

__device__ __forceinline__ int warp_claim(int* head) {
    int v = 0;
    if ((threadIdx.x & 31) == 0) v = atomicAdd(head, 1);
    return __shfl_sync(0xffffffffu, v, 0);
}

// Shared memory slots a lane needs for the bodies of block size M: the split
// single-segment body keeps C'_{q-1} and y_{q-1} (M*M + M), the split local
// stage also A'_{q-1} (2*M*M + M).
template <class Num, int M>
__host__ __device__ constexpr int batch_slots() {
    return modi_uses_lu<Num, M>() ? cyclic_slots<Num, M>() : (thomas_uses_lu<M>() ? M * M + M : 0);
}


template <class Num, int M, bool InStep = false>
__device__ __forceinline__ void batch_modi(const BatchArgs& ba, const BatchTile& tl, int seg, int lane, size_t plane,
                                           size_t rplane, unsigned& bad) {
    extern __shared__ double batch_cps[];
    const size_t rs = 32;
    const size_t mo = (size_t)tl.mat_off + lane, vo = (size_t)tl.vec_off + lane;
    int f, l;
    seg_rows(tl.rows, tl.nseg, seg, f, l);
    const size_t fo = (size_t)f * rs;
    if constexpr (modi_uses_lu<Num, M>()) {
        modi_body_lu<Num, M, InStep>(ba.a + mo + fo, ba.b + mo + fo, ba.c + mo + fo, ba.d + vo + fo, ba.aw + mo + fo,
                             ba.cw + mo + fo, batch_cps + threadIdx.x, blockDim.x, plane, rs, l - f + 1, true,
                             ba.ra + tl.red_mat_off + lane, ba.rc + tl.red_mat_off + lane,
                             ba.rd + tl.red_vec_off + lane, rplane, rs, seg, bad);
    } else {
        modi_body<Num, M>(ba.a + mo + fo, ba.b + mo + fo, ba.c + mo + fo, ba.d + vo + fo, ba.aw + mo + fo,
                          ba.cw + mo + fo, plane, rs, l - f + 1, true, ba.ra + tl.red_mat_off + lane,
                          ba.rc + tl.red_mat_off + lane, ba.rd + tl.red_vec_off + lane, rplane, rs, seg, bad);
    }
}

// Whether the local stage of block size M keeps each CTA's warps in step
// (as the uniform float-float kernels do): float-float with the split bodies
// (m = 5, 6), in CTAs of kBatchStepWarps warps.  Uneven batch of 32768
// systems, N 16..4096, m 2..5: float-float 17.25 -> 16.78 ms per sweep with
// 4-warp CTAs, 16.70 ms with 8.
template <class Num, int M>
__host__ __device__ constexpr bool batch_in_step() {
    return rows_in_step<Num>() && modi_uses_lu<Num, M>();
}
constexpr int kBatchStepWarps = 8;

// Barriers an item's body takes in step: block Thomas (seg < 0) one per
// forward row and one per backward row (2N - 1), the local stage of a
// segment of n rows one per forward row and one per backward row (n - 3).
__device__ __forceinline__ int item_barriers(const BatchTile& tl, int seg) {
    if (seg < 0) return 2 * tl.rows - 1;
    int f, l;
    seg_rows(tl.rows, tl.nseg, seg, f, l);
    const int n = l - f + 1;
    return n + (n > 3 ? n - 3 : 0);
}

template <class Num, int M, bool InStep = false>
__device__ __forceinline__ void batch_stage1(const BatchArgs& ba, const BatchTile& tl, int t, int seg, unsigned& bad) {
    const int lane = threadIdx.x & 31;
    const size_t plane = (size_t)32 * tl.rows, rs = 32;
    const int n_lane = tl.rows;  // every system of the tile is padded to its rows
    const bool active = lane < tl.lanes;
    const size_t mo = (size_t)tl.mat_off + lane, vo = (size_t)tl.vec_off + lane;
    extern __shared__ double batch_cps[];
    if (seg < 0) {
        if (!active) {
            // In step, a lane without a system takes the body's barriers;
            // otherwise it rejoins at the next claim.
            if constexpr (InStep) thomas_idle_rows(n_lane);
            return;
        }
        if constexpr (thomas_uses_lu<M>()) {
            // d solved apart: in this kernel, beside the local stage's
            // body, the merged column loop raises the spills (uneven batch
            // of 32768 systems, N 16..4096, m 2..5: float-float 17.90 vs
            // 18.43 ms per sweep).
            thomas_body_lu<Num, M, false, InStep>(ba.a + mo, ba.b + mo, ba.c + mo, ba.d + vo, ba.cw + mo,
                                                  batch_cps + threadIdx.x, blockDim.x, plane, rs, n_lane, true,
                                                  bad);
        } else {
            thomas_body<Num, M>(ba.a + mo, ba.b + mo, ba.c + mo, ba.d + vo, ba.cw + mo, plane, rs, n_lane, true, bad);
        }
        return;
    }
    const size_t rplane = (size_t)32 * 2 * tl.nseg;
    if (active) {
        batch_modi<Num, M, InStep>(ba, tl, seg, lane, plane, rplane, bad);
    } else if constexpr (InStep) {
        int f, l;
        seg_rows(tl.rows, tl.nseg, seg, f, l);
        modi_idle_rows(l - f + 1);
    }
    {
        // Publish this segment; the warp completing the tile solves its
        // reduced system while the other warps go on with their items (no
        // warp waits: the update is the next launch).  Measured against a
        // launch of its own, one warp per segmented tile (the uneven batch
        // above, segments of 64 rows): float-float 17.94 vs 18.43 ms per
        // sweep, FP64 24.60 vs 25.84 ms.
        __threadfence();
        __syncwarp();
        int done = 0;
        if (lane == 0) done = atomicAdd(&ba.seg_done[t], 1);
        done = __shfl_sync(0xffffffffu, done, 0);
        if (done == tl.nseg - 1) {
            __threadfence();
            if (active) {
                if constexpr (modi_uses_lu<Num, M>()) {
                    reduced_body_lu<Num, M>(ba.ra + tl.red_mat_off + lane, ba.rc + tl.red_mat_off + lane,
                                            ba.rd + tl.red_vec_off + lane, batch_cps + threadIdx.x, blockDim.x,
                                            rplane, rs, 2 * tl.nseg, bad);
                } else {
                    reduced_body<Num, M>(ba.ra + tl.red_mat_off + lane, ba.rc + tl.red_mat_off + lane,
                                         ba.rd + tl.red_vec_off + lane, rplane, rs, 2 * tl.nseg, bad);
                }
            }
        }
    }
}


// Registers of the local stage: the split bodies (m = 5, 6 in FP64 and
// float-float) are built for 128 registers (4 CTAs of 128 threads an SM);
// the fused local stage of the other sizes keeps up to 255.
template <class Num, int M>
__host__ __device__ constexpr int batch_min_ctas() {
    return batch_slots<Num, M>() > 0 ? 4 : 1;
}

template <class Num, int M>
__global__ void __launch_bounds__(batch_in_step<Num, M>() ? 32 * kBatchStepWarps : 128,
                                  batch_in_step<Num, M>() ? 2 : batch_min_ctas<Num, M>())
    k_batch_local(const BatchArgs ba) {
    unsigned bad = 0;
    if constexpr (batch_in_step<Num, M>()) {
        // In step: the CTA claims one item per warp at a time; every thread
        // takes the same barriers each round -- two around the claim, then
        // as many as the round's longest item takes (a warp whose item is
        // shorter, or that has none, adds the difference), so the rows of
        // the CTA's warps stay in step.
        __shared__ int claim;
        const int nw = blockDim.x >> 5, w = threadIdx.x >> 5;
        while (true) {
            cta_row_barrier();
            if (threadIdx.x == 0) claim = atomicAdd(ba.head1, nw);
            cta_row_barrier();
            const int base = claim;
            if (base >= ba.n1) break;
            int most = 0, mine = 0;
            for (int k = 0; k < nw && base + k < ba.n1; ++k) {
                const int2 it = ba.items1[base + k];
                const int c = item_barriers(ba.tiles[it.x], it.y);
                most = c > most ? c : most;
                if (k == w) mine = c;
            }
            if (base + w < ba.n1) {
                const int2 it = ba.items1[base + w];
                const BatchTile tl = ba.tiles[it.x];
                batch_stage1<Num, M, true>(ba, tl, it.x, it.y, bad);
            }
            for (int k = mine; k < most; ++k) cta_row_barrier();
        }
    } else {
        while (true) {
            const int item = warp_claim(ba.head1);
            if (item >= ba.n1) break;
            const int2 it = ba.items1[item];
            const BatchTile tl = ba.tiles[it.x];
            batch_stage1<Num, M>(ba, tl, it.x, it.y, bad);
        }
    }
    report_status(ba.status, bad);
}

template <class Num, int M>
__global__ void __launch_bounds__(128) k_batch_update(const BatchArgs ba) {
    unsigned bad = 0;
    while (true) {
        const int item = warp_claim(ba.head3);
        if (item >= ba.n3) break;
        const int2 it = ba.items3[item];
        const BatchTile tl = ba.tiles[it.x];
        const int t = it.x, seg = it.y;
        const int lane = threadIdx.x & 31;
        const int n_lane = tl.rows;
        if (lane < tl.lanes) {
            const size_t plane = (size_t)32 * tl.rows, rs = 32;
            const size_t mo = (size_t)tl.mat_off + lane, vo = (size_t)tl.vec_off + lane;
            int f, l;
            seg_rows(n_lane, tl.nseg, seg, f, l);
            const size_t fo = (size_t)f * rs;
            unsigned amax = 0;
            update_body<Num, M>(ba.aw + mo + fo, ba.cw + mo + fo, ba.d + vo + fo, plane, rs, l - f + 1, true,
                                ba.rd + tl.red_vec_off + lane, (size_t)32 * 2 * tl.nseg, rs, seg, amax);
            bad |= range_bits<Num>(amax, false);
        }
    }
    report_status(ba.status, bad);
}

// The two launches of block size M on stream s, both persistent (as many
// CTAs of `warps` warps as fit the device): the local stage with the reduced
// solves, then the update.
template <class Num, int M>
cudaError_t launch_batch(const BatchArgs& ba, int warps, cudaStream_t s, int* grid_out) {
    if constexpr (std::is_same<Num, F32>::value) {
        return cudaErrorInvalidValue;  // FP64 and float-float batches only
    } else {
        if (batch_in_step<Num, M>()) warps = kBatchStepWarps;  // the tuned CTA size is for the other sizes
        int dev = 0, sms = 0, per_sm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const size_t smem = (size_t)32 * warps * batch_slots<Num, M>() * sizeof(double);
        if (e == cudaSuccess && smem > 48u * 1024u)
            e = cudaFuncSetAttribute(k_batch_local<Num, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_local<Num, M>, 32 * warps, smem);
        if (e != cudaSuccess) return e;
        const int grid = sms * (per_sm > 0 ? per_sm : 1);
        if (grid_out) *grid_out = grid;
        if (ba.n1 > 0) k_batch_local<Num, M><<<grid, 32 * warps, smem, s>>>(ba);
        if (ba.n3 > 0) {
            int per_sm3 = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm3, k_batch_update<Num, M>, 128, 0);
            if (e != cudaSuccess) return e;
            k_batch_update<Num, M><<<sms * (per_sm3 > 0 ? per_sm3 : 1), 128, 0, s>>>(ba);
        }
        return cudaGetLastError();
    }
}

}  // namespace pbt
