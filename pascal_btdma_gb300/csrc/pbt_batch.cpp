// pbt_batch.cpp -- host side of include/pbt_batch.h: tiling, work queues,
// workspace and launches of the persistent batch kernel (pbt_batch.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/pbt_batch.h"
#include "pbt_batch_types.h"
#include "pbt_internal.h"

struct pbt_batch {
    int nsys = 0, precision = 0, ntiles = 0, n1 = 0, n3 = 0, warps = 4, last_grid = 0;
    // Items of block size m: items1[off1[m] .. off1[m] + cnt1[m]), likewise
    // items3; one persistent launch per block size present, in `order`.
    int off1[PBT_MAX_BLOCK + 1] = {}, cnt1[PBT_MAX_BLOCK + 1] = {};
    int off3[PBT_MAX_BLOCK + 1] = {}, cnt3[PBT_MAX_BLOCK + 1] = {};
    std::vector<int> order;
    std::vector<long long> user_mat_off, user_vec_off;
    long long user_mat = 0, user_vec = 0, packed_mat = 0, packed_vec = 0, red_mat = 0, red_vec = 0;
    // device
    pbt::BatchTile* tiles = nullptr;
    int* lane_rows = nullptr;
    int* sys_of = nullptr;
    int2* items1 = nullptr;
    int2* items3 = nullptr;
    long long* d_user_mat_off = nullptr;
    long long* d_user_vec_off = nullptr;
    long long* row_start = nullptr;
    long long pack_total = 0;
    int* state = nullptr;  // error (always 0), pad, head1[m], head3[m] (kHeads each), seg_done[ntiles]
    unsigned long long* status = nullptr;
    double *aw = nullptr, *cw = nullptr, *ra = nullptr, *rc = nullptr, *rd = nullptr;
    cudaStream_t last_stream = nullptr;
    unsigned magic = 0x50425442u;  // "PBTB"
};

namespace {

constexpr unsigned kBatchMagic = 0x50425442u;
constexpr int kHeads = PBT_MAX_BLOCK + 1;

size_t state_ints(int ntiles) { return (size_t)2 + 2 * kHeads + (size_t)ntiles; }

// One launch of the batch kernel for block size m (pbt_inst.cu instantiates
// launch_batch per arithmetic and block size).
cudaError_t launch_m(int precision, int m, const pbt::BatchArgs& ba, int warps, cudaStream_t s, int* grid) {
#define PBT_BATCH_CASE(MM)                                                                        \
    case MM:                                                                                      \
        return precision == PBT_PREC_FF ? pbt::launch_batch<pbt::FF, MM>(ba, warps, s, grid)    \
                                        : pbt::launch_batch<pbt::F64, MM>(ba, warps, s, grid);
    switch (m) {
        PBT_BATCH_CASE(1)
        PBT_BATCH_CASE(2)
        PBT_BATCH_CASE(3)
        PBT_BATCH_CASE(4)
        PBT_BATCH_CASE(5)
        PBT_BATCH_CASE(6)
        PBT_BATCH_CASE(7)
        PBT_BATCH_CASE(8)
        PBT_BATCH_CASE(9)
        PBT_BATCH_CASE(10)
        default:
            return cudaErrorInvalidValue;
    }
#undef PBT_BATCH_CASE
}
static_assert(PBT_BATCH_MAX_BLOCK == 10, "launch_m lists block sizes 1..10");

int bfail(int code, const std::string& msg) { return pbt::set_last_error(code, msg.c_str()); }

int bcuda(cudaError_t e, const char* what) {
    return bfail(PBT_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class T>
int upload(T** dst, const std::vector<T>& src) {
    if (src.empty()) return PBT_OK;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), src.size() * sizeof(T));
    if (e == cudaSuccess) e = cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? PBT_OK : bcuda(e, "batch_create: upload");
}

int dalloc(double** p, long long n) {
    if (n <= 0) return PBT_OK;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), (size_t)n * sizeof(double));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bfail(e == cudaErrorMemoryAllocation ? PBT_ENOMEM : PBT_ECUDA,
                     std::string("batch_create: workspace allocation: ") + cudaGetErrorString(e));
    }
    return PBT_OK;
}

void free_batch(pbt_batch* b) {
    cudaFree(b->tiles);
    cudaFree(b->lane_rows);
    cudaFree(b->sys_of);
    cudaFree(b->items1);
    cudaFree(b->items3);
    cudaFree(b->d_user_mat_off);
    cudaFree(b->d_user_vec_off);
    cudaFree(b->row_start);
    cudaFree(b->state);
    cudaFree(b->status);
    cudaFree(b->aw);
    cudaFree(b->cw);
    cudaFree(b->ra);
    cudaFree(b->rc);
    cudaFree(b->rd);
}

int check(const pbt_batch* b) {
    if (!b || b->magic != kBatchMagic) return bfail(PBT_ESTATE, "batch: null, destroyed or corrupt handle");
    return PBT_OK;
}

}  // namespace

extern "C" {

void pbt_batch_tuning_init(pbt_batch_tuning* t) {
    if (!t) return;
    std::memset(t, 0, sizeof *t);
    for (int m = 0; m <= PBT_MAX_BLOCK; ++m) t->seg_len[m] = 256;
    t->warps_per_cta = 4;
}

int pbt_batch_create(pbt_batch** out, int nsys, const int* m, const int* nrow, int precision,
                     const pbt_batch_tuning* tuning) {
    if (!out) return bfail(PBT_EINVAL, "batch_create: null output handle");
    *out = nullptr;
    if (nsys <= 0 || !m || !nrow) return bfail(PBT_EINVAL, "batch_create: needs nsys > 0 and the m, nrow arrays");
    if (precision != PBT_PREC_FP64 && precision != PBT_PREC_FF)
        return bfail(PBT_EUNSUPPORTED, "batch_create: precision fp64 or ff");
    for (int s = 0; s < nsys; ++s) {
        if (m[s] < 1 || m[s] > PBT_BATCH_MAX_BLOCK || nrow[s] < 2) {
            char buf[160];
            std::snprintf(buf, sizeof buf, "batch_create: system %d has m=%d, nrow=%d (needs 1 <= m <= %d, nrow >= 2)",
                          s, m[s], nrow[s], PBT_BATCH_MAX_BLOCK);
            return bfail(PBT_EINVAL, buf);
        }
    }
    pbt_batch_tuning tu;
    if (tuning) tu = *tuning; else pbt_batch_tuning_init(&tu);
    if (tu.warps_per_cta == 0) tu.warps_per_cta = 4;
    if (tu.warps_per_cta < 1 || tu.warps_per_cta > 4) return bfail(PBT_EINVAL, "batch_create: warps_per_cta in 1..4");

    pbt_batch* b = new (std::nothrow) pbt_batch();
    if (!b) return bfail(PBT_ENOMEM, "batch_create: host allocation");
    b->nsys = nsys;
    b->precision = precision;
    b->warps = tu.warps_per_cta;
    // Caller layout offsets.
    b->user_mat_off.resize(nsys);
    b->user_vec_off.resize(nsys);
    long long om = 0, ov = 0;
    for (int s = 0; s < nsys; ++s) {
        b->user_mat_off[s] = om;
        b->user_vec_off[s] = ov;
        om += (long long)nrow[s] * m[s] * m[s];
        ov += (long long)nrow[s] * m[s];
    }
    b->user_mat = om;
    b->user_vec = ov;
    // Tiles: systems sorted by (m, N descending), 32 per tile.
    std::vector<int> order(nsys);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return m[x] != m[y] ? m[x] < m[y] : nrow[x] > nrow[y];
    });
    std::vector<pbt::BatchTile> tiles;
    std::vector<int> lane_rows, sys_of;
    std::vector<long long> row_start;
    long long mat_off = 0, vec_off = 0, red_m = 0, red_v = 0, rowacc = 0;
    for (int k = 0; k < nsys;) {
        const int mm = m[order[k]];
        int lanes = 0;
        while (lanes < 32 && k + lanes < nsys && m[order[k + lanes]] == mm) ++lanes;
        pbt::BatchTile t{};
        t.m = mm;
        t.lanes = lanes;
        t.rows = nrow[order[k]];
        // Systems are padded to the tile's rows (pbt_batch_pack), so the
        // segments split t.rows.
        int P = 1;
        const int L = tu.seg_len[mm];
        if (L > 0) {
            P = (t.rows + L / 2) / L;
            P = std::max(1, std::min(P, t.rows / 3));
        }
        t.nseg = P;
        t.mat_off = mat_off;
        t.vec_off = vec_off;
        t.red_mat_off = red_m;
        t.red_vec_off = red_v;
        mat_off += 32LL * t.rows * mm * mm;
        vec_off += 32LL * t.rows * mm;
        if (P > 1) {
            red_m += 32LL * 2 * P * mm * mm;
            red_v += 32LL * 2 * P * mm;
        }
        row_start.push_back(rowacc);
        rowacc += 32LL * t.rows;
        for (int l = 0; l < 32; ++l) {
            lane_rows.push_back(l < lanes ? nrow[order[k + l]] : 0);
            sys_of.push_back(l < lanes ? order[k + l] : -1);
        }
        tiles.push_back(t);
        k += lanes;
    }
    b->ntiles = (int)tiles.size();
    b->packed_mat = mat_off;
    b->packed_vec = vec_off;
    b->red_mat = red_m;
    b->red_vec = red_v;
    b->pack_total = rowacc;
    // Work items, per block size.  Stage 1 by decreasing cost (m^3 * rows of
    // the item; the two-stage elimination costs ~2.4x block Thomas per row);
    // stage 3 in the order stage 1 first reaches each tile.  The launches run
    // the block sizes in decreasing total cost.
    struct It {
        int t, s;
        double cost;
    };
    std::vector<int2> items1, items3;
    std::vector<char> seen(b->ntiles, 0);
    std::vector<std::pair<double, int>> by_cost;
    for (int mm = 1; mm <= PBT_BATCH_MAX_BLOCK; ++mm) {
        std::vector<It> it1;
        double total = 0.0;
        for (int t = 0; t < b->ntiles; ++t) {
            const auto& tl = tiles[t];
            if (tl.m != mm) continue;
            const double w = (double)tl.m * tl.m * tl.m;
            if (tl.nseg == 1) {
                it1.push_back({t, -1, w * tl.rows});
            } else {
                for (int sg = 0; sg < tl.nseg; ++sg) it1.push_back({t, sg, 2.4 * w * tl.rows / tl.nseg});
            }
            total += it1.back().cost * (tl.nseg == 1 ? 1 : tl.nseg);
        }
        if (it1.empty()) continue;
        std::stable_sort(it1.begin(), it1.end(), [](const It& x, const It& y) { return x.cost > y.cost; });
        b->off1[mm] = (int)items1.size();
        b->off3[mm] = (int)items3.size();
        for (const auto& i : it1) {
            items1.push_back(make_int2(i.t, i.s));
            if (i.s >= 0 && !seen[i.t]) {
                seen[i.t] = 1;
                for (int sg = 0; sg < tiles[i.t].nseg; ++sg) items3.push_back(make_int2(i.t, sg));
            }
        }
        b->cnt1[mm] = (int)items1.size() - b->off1[mm];
        b->cnt3[mm] = (int)items3.size() - b->off3[mm];
        by_cost.push_back({total, mm});
    }
    std::stable_sort(by_cost.begin(), by_cost.end(), [](const std::pair<double, int>& x, const std::pair<double, int>& y) {
        return x.first > y.first;
    });
    for (const auto& c : by_cost) b->order.push_back(c.second);
    b->n1 = (int)items1.size();
    b->n3 = (int)items3.size();
    int rc = PBT_OK;
    if ((rc = upload(&b->tiles, tiles)) || (rc = upload(&b->lane_rows, lane_rows)) || (rc = upload(&b->sys_of, sys_of)) ||
        (rc = upload(&b->items1, items1)) || (rc = upload(&b->items3, items3)) ||
        (rc = upload(&b->d_user_mat_off, b->user_mat_off)) || (rc = upload(&b->d_user_vec_off, b->user_vec_off)) ||
        (rc = upload(&b->row_start, row_start)))
        goto fail_out;
    {
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&b->state), sizeof(int) * state_ints(b->ntiles));
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&b->status), sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMemset(b->status, 0, sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMemset(b->state, 0, sizeof(int) * state_ints(b->ntiles));
        if (e != cudaSuccess) {
            rc = bcuda(e, "batch_create: queue state");
            goto fail_out;
        }
    }
    if ((rc = dalloc(&b->cw, b->packed_mat)) || (rc = dalloc(&b->aw, b->red_mat > 0 ? b->packed_mat : 0)) ||
        (rc = dalloc(&b->ra, b->red_mat)) || (rc = dalloc(&b->rc, b->red_mat)) || (rc = dalloc(&b->rd, b->red_vec)))
        goto fail_out;
    *out = b;
    return PBT_OK;
fail_out:
    free_batch(b);
    b->magic = 0;
    delete b;
    return rc;
}

int pbt_batch_destroy(pbt_batch* b) {
    if (!b) return PBT_OK;
    int rc = check(b);
    if (rc) return rc;
    free_batch(b);
    b->magic = 0;
    delete b;
    return PBT_OK;
}

int pbt_batch_sizes(const pbt_batch* b, long long* um, long long* uv, long long* pm, long long* pv) {
    int rc = check(b);
    if (rc) return rc;
    if (um) *um = b->user_mat;
    if (uv) *uv = b->user_vec;
    if (pm) *pm = b->packed_mat;
    if (pv) *pv = b->packed_vec;
    return PBT_OK;
}

int pbt_batch_user_offsets(const pbt_batch* b, long long* mo, long long* vo) {
    int rc = check(b);
    if (rc) return rc;
    if (mo) std::copy(b->user_mat_off.begin(), b->user_mat_off.end(), mo);
    if (vo) std::copy(b->user_vec_off.begin(), b->user_vec_off.end(), vo);
    return PBT_OK;
}

static pbt::PackArgs pack_args(const pbt_batch* b) {
    pbt::PackArgs pa;
    pa.tiles = b->tiles;
    pa.lane_rows = b->lane_rows;
    pa.sys_of = b->sys_of;
    pa.user_mat_off = b->d_user_mat_off;
    pa.user_vec_off = b->d_user_vec_off;
    pa.row_start = b->row_start;
    pa.ntiles = b->ntiles;
    pa.total = b->pack_total;
    return pa;
}

int pbt_batch_pack(pbt_batch* b, const double* ua, const double* ub, const double* uc, const double* ud, double* pa,
                   double* pb, double* pc, double* pd, void* stream) {
    int rc = check(b);
    if (rc) return rc;
    if (!ua || !ub || !uc || !ud || !pa || !pb || !pc || !pd) return bfail(PBT_EINVAL, "batch_pack: null pointer");
    cudaError_t e = pbt::launch_pack(pack_args(b), ua, ub, uc, ud, pa, pb, pc, pd, nullptr, 0,
                                     static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? PBT_OK : bcuda(e, "batch_pack");
}

int pbt_batch_unpack(pbt_batch* b, const double* pd, double* ud, void* stream) {
    int rc = check(b);
    if (rc) return rc;
    if (!pd || !ud) return bfail(PBT_EINVAL, "batch_unpack: null pointer");
    cudaError_t e = pbt::launch_pack(pack_args(b), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                     const_cast<double*>(pd), ud, 1, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? PBT_OK : bcuda(e, "batch_unpack");
}

int pbt_batch_solve(pbt_batch* b, const double* pa, const double* pb, const double* pc, double* pd, void* stream) {
    int rc = check(b);
    if (rc) return rc;
    if (!pa || !pb || !pc || !pd) return bfail(PBT_EINVAL, "batch_solve: null pointer");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    b->last_stream = s;
    cudaError_t e = cudaMemsetAsync(b->state, 0, sizeof(int) * state_ints(b->ntiles), s);
    if (e != cudaSuccess) return bcuda(e, "batch_solve: queue reset");
    pbt::BatchArgs ba;
    ba.a = pa;
    ba.b = pb;
    ba.c = pc;
    ba.d = pd;
    ba.aw = b->aw;
    ba.cw = b->cw;
    ba.ra = b->ra;
    ba.rc = b->rc;
    ba.rd = b->rd;
    ba.tiles = b->tiles;
    ba.lane_rows = b->lane_rows;
    ba.status = b->status;
    ba.seg_done = b->state + 2 + 2 * kHeads;
    b->last_grid = 0;
    for (int mm : b->order) {
        ba.items1 = b->items1 + b->off1[mm];
        ba.items3 = b->items3 + b->off3[mm];
        ba.n1 = b->cnt1[mm];
        ba.n3 = b->cnt3[mm];
        ba.head1 = b->state + 2 + mm;
        ba.head3 = b->state + 2 + kHeads + mm;
        int grid = 0;
        e = launch_m(b->precision, mm, ba, b->warps, s, &grid);
        if (e != cudaSuccess) return bcuda(e, "batch_solve: launch");
        b->last_grid = std::max(b->last_grid, grid);
    }
    return PBT_OK;
}

int pbt_batch_status(pbt_batch* b, long long* nsingular, int* timed_out) {
    int rc = check(b);
    if (rc) return rc;
    cudaError_t e = cudaStreamSynchronize(b->last_stream);
    if (e != cudaSuccess) return bcuda(e, "batch_status: synchronize");
    unsigned long long v = 0;
    int err = 0;
    if ((e = cudaMemcpy(&v, b->status, sizeof v, cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(&err, b->state, sizeof err, cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemset(b->status, 0, sizeof v)) != cudaSuccess)
        return bcuda(e, "batch_status: read");
    const unsigned long long pivots = v & pbt::kPivotCountMask;
    if (nsingular) *nsingular = (long long)pivots;
    if (timed_out) *timed_out = err;
    if (err) return bfail(PBT_ECUDA, "batch_status: a wait of the persistent kernel ran out; the result is invalid");
    if (v & pbt::kRangeMark)
        return bfail(PBT_ERANGE, "a float-float value left the arithmetic's range (an input outside "
                                 "2^-96 <= |x| < 2^96, an overflow, or a solution below 2^-100); the result is invalid");
    if (pivots) return bfail(PBT_ESINGULAR, "a zero pivot was met in at least one block");
    return PBT_OK;
}

int pbt_batch_info(const pbt_batch* b, int* ntiles, int* n1, int* n3, int* grid) {
    int rc = check(b);
    if (rc) return rc;
    if (ntiles) *ntiles = b->ntiles;
    if (n1) *n1 = b->n1;
    if (n3) *n3 = b->n3;
    if (grid) *grid = b->last_grid;
    return PBT_OK;
}

}  // extern "C"
