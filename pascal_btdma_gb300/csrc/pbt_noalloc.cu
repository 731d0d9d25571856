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

#include "pbt_internal.h"

namespace {

// Capacity of the reduced-system scratch in doubles (4 Mi doubles = 32 MiB).
constexpr size_t kScratchDoubles = size_t(4) << 20;
constexpr size_t kStatusSlot = 32;  // doubles: one 256-byte slot after the scratch

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles + kStatusSlot];

// 256-byte alignment of every sub-array keeps warp accesses on whole segments.
size_t round_up32(size_t n) { return (n + 31) & ~size_t(31); }

// gridDim.y of the local-stage and update launches is the segment count.
constexpr int kMaxSegments = 65535;

// Device address of the scratch array on the current device.  In host code
// `g_noalloc_scratch` names a host-side stand-in, not device memory, so the
// address is looked up with the device current.  It is looked up on every
// call (a table lookup once the module is loaded; it allocates nothing), so a
// context that was reset and made again never sees a stale address.  The
// first call on a device loads the library's device code there (lazy module
// loading), which is why that first call must come before any stream capture.
int scratch_on_current_device(double** out, int* sms) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "solve_noncyclic_noalloc: cudaGetDevice failed: %s", cudaGetErrorString(e));
        return pbt::set_last_error(PBT_ECUDA, buf);
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        char buf[200];
        std::snprintf(buf, sizeof buf, "solve_noncyclic_noalloc: cudaGetSymbolAddress of the static scratch failed: %s",
                      cudaGetErrorString(e));
        return pbt::set_last_error(PBT_ECUDA, buf);
    }
    *out = static_cast<double*>(p);
    if (cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || *sms <= 0) {
        cudaGetLastError();
        *sms = 1;
    }
    return PBT_OK;
}

// Threads per block for `items` threads of work: enough CTAs to give every
// SM two.
int pick_threads(long long items, int sms) {
    int tpb = 128;
    while (tpb > 32 && (items + tpb - 1) / tpb < 2LL * sms) tpb /= 2;
    return tpb;
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
    if (nsys <= 0 || nrow < 2 || nseg < 1 || nseg > kMaxSegments || nrow < 2 * nseg ||
        (nseg > 1 && nrow < 3 * nseg)) {
        std::snprintf(buf, sizeof buf,
                      "solve_noncyclic_noalloc: needs nsys > 0, nrow >= 2, 1 <= nseg <= %d and >= 3 rows per "
                      "segment when nseg > 1 (nsys=%d, nrow=%d, nseg=%d)", kMaxSegments, nsys, nrow, nseg);
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
    int sms = 1;
    int rc = scratch_on_current_device(&base, &sms);
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
    g.tpb = pick_threads((long long)nsys * nseg, sms);
    g.stream = static_cast<cudaStream_t>(stream);
    g.sms = sms;
    g.tpb_auto = 1;

    cudaError_t e = cudaMemsetAsync(g.status, 0, sizeof(unsigned long long), g.stream);
    if (e == cudaSuccess) PBT_NOALLOC_DISPATCH(launch_modi)
    if (e == cudaSuccess) {
        pbt::SolveArgs g2 = g;
        g2.tpb = pick_threads(nsys, sms);
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
