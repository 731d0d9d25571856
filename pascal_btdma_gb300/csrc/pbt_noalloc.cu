// pbt_noalloc.cu -- a solve entry point that allocates no device memory.
//
// Every other entry point works through a plan, and creating a plan calls
// cudaMalloc for its workspace.  Some callers cannot do that: applications
// that hand the whole device memory to their own pool allocator at start-up
// and forbid later allocations, and time-stepping loops that must not call
// cudaMalloc / cudaFree between kernels because those calls can synchronise
// the device while other streams are busy.  pbt_solve_noncyclic_noalloc
// serves them: it runs the two-stage method in place (A <- A', C <- C',
// D <- x, like the reference) and keeps the only scratch it needs -- the
// reduced system of two block rows per segment and a zero-pivot counter -- in
// a fixed-size array compiled into this library.
//
// The array lives for as long as the library is loaded, on every GPU that
// loads it: kScratchDoubles doubles (32 MiB) plus one 256-byte status slot.
// All calls share it and it keeps the last call's contents; the status slot is
// cleared on every call and the reduced rows are fully rewritten before they
// are read.  Two calls whose work overlaps on the GPU (on different streams, or
// from different host threads) race on the array.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "pbt_internal.h"

namespace {

// Capacity of the reduced-system scratch in doubles (4 Mi doubles = 32 MiB).
constexpr size_t kScratchDoubles = size_t(4) << 20;
constexpr size_t kStatusSlot = 32;  // doubles: one 256-byte slot after the scratch

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles + kStatusSlot];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_addr[kMaxDevices] = {};  // device address of g_noalloc_scratch, per device

// 256-byte alignment of every sub-array keeps warp accesses on whole segments.
size_t round_up32(size_t n) { return (n + 31) & ~size_t(31); }

// Device address of the scratch array on the current device.  In host code
// `g_noalloc_scratch` names a host-side stand-in, not device memory, so the
// address is fetched once per device, with that device current.
int scratch_on_current_device(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "solve_noncyclic_noalloc: cudaGetDevice failed: %s", cudaGetErrorString(e));
        return pbt::set_last_error(PBT_ECUDA, buf);
    }
    if (dev < 0 || dev >= kMaxDevices) return pbt::set_last_error(PBT_EINVAL, "solve_noncyclic_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            char buf[200];
            std::snprintf(buf, sizeof buf, "solve_noncyclic_noalloc: cudaGetSymbolAddress of the static scratch failed: %s",
                          cudaGetErrorString(e));
            return pbt::set_last_error(PBT_ECUDA, buf);
        }
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return PBT_OK;
}

#define PBT_NOALLOC_DISPATCH(FN)                            \
    switch (m) {                                            \
        case 1: e = pbt::FN<pbt::F64, 1>(g); break;                   \
        case 2: e = pbt::FN<pbt::F64, 2>(g); break;                   \
        case 3: e = pbt::FN<pbt::F64, 3>(g); break;                   \
        case 4: e = pbt::FN<pbt::F64, 4>(g); break;                   \
        case 5: e = pbt::FN<pbt::F64, 5>(g); break;                   \
        case 6: e = pbt::FN<pbt::F64, 6>(g); break;                   \
        case 7: e = pbt::FN<pbt::F64, 7>(g); break;                   \
        case 8: e = pbt::FN<pbt::F64, 8>(g); break;                   \
        case 9: e = pbt::FN<pbt::F64, 9>(g); break;                   \
        default: e = pbt::FN<pbt::F64, 10>(g); break;                 \
    }

}  // namespace

extern "C" int pbt_solve_noncyclic_noalloc(double* a, double* b, double* c, double* d, int m, int nsys, int nrow,
                                           int nseg, void* stream) {
    char buf[256];
    if (m < 1 || m > PBT_MAX_BLOCK) {
        std::snprintf(buf, sizeof buf, "solve_noncyclic_noalloc: block size m=%d outside 1..%d", m, PBT_MAX_BLOCK);
        return pbt::set_last_error(PBT_EINVAL, buf);
    }
    if (nsys <= 0 || nrow < 2 || nseg < 1 || nrow < 2 * nseg || (nseg > 1 && nrow < 3 * nseg)) {
        std::snprintf(buf, sizeof buf,
                      "solve_noncyclic_noalloc: needs nsys > 0, nrow >= 2, nseg >= 1 and >= 3 rows per segment "
                      "when nseg > 1 (nsys=%d, nrow=%d, nseg=%d)", nsys, nrow, nseg);
        return pbt::set_last_error(PBT_EINVAL, buf);
    }
    if (!a || !b || !c || !d) return pbt::set_last_error(PBT_EINVAL, "solve_noncyclic_noalloc: null array pointer");
    const size_t rrows = (size_t)nsys * 2 * (size_t)nseg;
    const size_t mat = round_up32(rrows * m * m), vec = round_up32(rrows * m);
    const size_t need = 2 * mat + vec;
    if (need > kScratchDoubles) {
        std::snprintf(buf, sizeof buf,
                      "solve_noncyclic_noalloc: the reduced system needs %zu doubles of scratch "
                      "(nsys*2*nseg*(2m^2+m) = %zu), more than the static capacity of %zu doubles (32 MiB); "
                      "use fewer systems per call or a plan", need, rrows * (2 * (size_t)m * m + m),
                      kScratchDoubles);
        return pbt::set_last_error(PBT_EINVAL, buf);
    }
    double* base = nullptr;
    int rc = scratch_on_current_device(&base);
    if (rc != PBT_OK) return rc;

    pbt::SolveArgs g;
    g.a = a;
    g.b = b;
    g.c = c;
    g.d = d;
    g.aw = a;  // in place: A <- A', C <- C'
    g.cw = c;
    g.ra = base;
    g.rc = base + mat;
    g.rd = base + 2 * mat;
    g.re = nullptr;
    g.status = reinterpret_cast<unsigned long long*>(base + kScratchDoubles);
    g.factors_raw = 0;
    g.nsys = nsys;
    g.nrow = nrow;
    g.nseg = nseg;
    int tpb = 128;
    while (tpb > 32 && ((long long)nsys * nseg + tpb - 1) / tpb < 2 * 152) tpb /= 2;
    g.tpb = tpb;
    g.stream = static_cast<cudaStream_t>(stream);

    cudaError_t e = cudaMemsetAsync(g.status, 0, sizeof(unsigned long long), g.stream);
    if (e == cudaSuccess) PBT_NOALLOC_DISPATCH(launch_modi)
    if (e == cudaSuccess) {
        pbt::SolveArgs g2 = g;
        int t2 = 128;
        while (t2 > 32 && (nsys + t2 - 1) / t2 < 2 * 152) t2 /= 2;
        g2.tpb = t2;
        {
            const pbt::SolveArgs& g = g2;
            PBT_NOALLOC_DISPATCH(launch_reduced)
        }
    }
    if (e == cudaSuccess) PBT_NOALLOC_DISPATCH(launch_update)
    if (e != cudaSuccess) {
        std::snprintf(buf, sizeof buf, "solve_noncyclic_noalloc: launch failed: %s", cudaGetErrorString(e));
        return pbt::set_last_error(PBT_ECUDA, buf);
    }
    return PBT_OK;
}
