/*
 * pbt_batch.h -- uneven batches: thousands of block-tridiagonal systems of
 * different length N and block size m solved by persistent launches
 * (part of libpbt.so).  No counterpart in the reference, whose plan fixes
 * one (m, nsys, nrow) per call (pascal_btdma_cuda.hpp:128-145).
 *
 * Caller layout ("per-system"): system s occupies its own contiguous range,
 * in the reference layout of a single system --
 *   A_s[row + N_s*(i + m_s*j)] at offset mat_off[s],  D_s[row + N_s*i] at vec_off[s],
 * with the offsets of pbt_batch_user_offsets (prefix sums of N_s*m_s^2 and
 * N_s*m_s).  pbt_batch_pack rearranges such arrays into the batch's packed
 * layout (tiles of 32 systems of equal m, sorted by N); pbt_batch_solve works
 * on packed arrays; pbt_batch_unpack brings the solution back.  Non-cyclic
 * lines; A_0 and C_{N-1} of every system act as zero.  In the packed layout a
 * system shorter than its tile's longest is extended to that length with rows
 * that decouple from it (B = I, A = C = 0, d = 0); unpack returns only the
 * system's own rows.
 *
 * The solve runs, per block size present (largest total cost first), a
 * persistent launch over the local-stage items (the warp that completes a
 * tile's last segment also solves the tile's reduced system) and a
 * persistent launch over the update items, on the caller's stream; each
 * launch carries one block size's code.
 *
 * Tuning (pbt_batch_tuning): the number of segments of each tile is
 * round(N_max / seg_len[m]) (one segment when seg_len[m] <= 0), so long lines
 * use the two-stage method and no single warp's chain of rows dominates the
 * launch; warps_per_cta sets the persistent CTA size (float-float m = 5, 6,
 * whose local stage keeps a CTA's warps on the same row, always runs 8-warp
 * CTAs there).  An autotuner picks these per (m, N, nsys) bucket
 * (pascal_btdma_gb300/batch.py).
 */
#ifndef PBT_BATCH_H
#define PBT_BATCH_H

#include "pbt.h"

#ifdef __cplusplus
extern "C" {
#endif

#define PBT_BATCH_MAX_BLOCK 10

typedef struct pbt_batch pbt_batch;

typedef struct pbt_batch_tuning {
    int seg_len[PBT_MAX_BLOCK + 1]; /* target rows per segment, indexed by m; <= 0: one segment */
    int warps_per_cta;              /* 1..4; 0 = 4 */
    int reserved[8];
} pbt_batch_tuning;

/* Defaults: seg_len[m] = 256 for every m, 4 warps per CTA. */
void pbt_batch_tuning_init(pbt_batch_tuning* tuning);

/* Plan a batch of nsys systems with block sizes m[s] (1..PBT_BATCH_MAX_BLOCK)
 * and lengths nrow[s] (>= 2); precision PBT_PREC_FP64 or PBT_PREC_FF;
 * tuning may be NULL.  Allocates the device workspace. */
int pbt_batch_create(pbt_batch** batch, int nsys, const int* m, const int* nrow, int precision,
                     const pbt_batch_tuning* tuning);

int pbt_batch_destroy(pbt_batch* batch);

/* Element counts (doubles): per-system layout of A (= B = C) and D, and the
 * packed layout of A (= B = C) and D. */
int pbt_batch_sizes(const pbt_batch* batch, long long* user_mat, long long* user_vec,
                    long long* packed_mat, long long* packed_vec);

/* Per-system offsets of the caller layout (host arrays of nsys entries). */
int pbt_batch_user_offsets(const pbt_batch* batch, long long* mat_off, long long* vec_off);

/* Per-system layout -> packed layout (device arrays, on `stream`). */
int pbt_batch_pack(pbt_batch* batch, const double* ua, const double* ub, const double* uc, const double* ud,
                   double* pa, double* pb, double* pc, double* pd, void* stream);

/* Packed D -> per-system D. */
int pbt_batch_unpack(pbt_batch* batch, const double* pd, double* ud, void* stream);

/* Solve every system of the batch in place on packed arrays: one memset of
 * the queue state and up to two launches per block size present, no host
 * synchronisation. */
int pbt_batch_solve(pbt_batch* batch, const double* pa, const double* pb, const double* pc, double* pd,
                    void* stream);

/* Synchronises the last stream; reports zero pivots met.  *timed_out is
 * always 0: the stages are separate launches, so no kernel waits on another
 * (the argument stays for callers of the earlier single-launch form).
 * Returns PBT_ERANGE (a float-float batch left the arithmetic's range, as
 * pbt_plan_status; the result is invalid) or PBT_ESINGULAR accordingly, in
 * that order. */
int pbt_batch_status(pbt_batch* batch, long long* nsingular, int* timed_out);

/* Shape of the schedule: tiles, stage-1 and stage-3 items, CTAs of the
 * largest persistent launch of the last solve (0 before the first). */
int pbt_batch_info(const pbt_batch* batch, int* ntiles, int* n_items1, int* n_items3, int* grid_ctas);

#ifdef __cplusplus
}
#endif
#endif
