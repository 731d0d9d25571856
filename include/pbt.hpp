/*
 * pbt.hpp -- C++ layer over the C ABI of pbt.h, with the reference C++ port's
 * names and error behaviour (CUDA_CXX_Port/include/pascal_btdma_cuda.hpp):
 *
 *   reference                                   here
 *   pascal_btdma::BtdmaGpuPlan (hpp:88-135)     pbt::BtdmaGpuPlan (move-only, frees in its destructor)
 *     create(m, nsys, nrow, comm, mode)         create(m, nsys, nrow, nseg [, desc options])
 *     destroy()                                 destroy()
 *   solve_noncyclic(plan, a, b, c, d, m, nsys, nrow, stream)            (hpp:137-145)
 *   solve_noncyclic_profiled(..., timings, stream)                      (hpp:147-156)
 *   solve_cyclic(plan, a, b, c, d, m, nsys, nrow, stream)               (hpp:158-166)
 *   BtdmaSolveTimings (hpp:24-39)               pbt::BtdmaSolveTimings (same six fields)
 *   partition_1d (hpp:67)                       pbt::partition_1d
 *   CudaError (hpp:20-22)                       pbt::CudaError
 *
 * Status codes become the reference's exception types: PBT_EINVAL ->
 * std::invalid_argument, PBT_ECUDA -> CudaError, PBT_ESTATE and
 * PBT_ETIMEOUT -> std::runtime_error, PBT_EUNSUPPORTED -> std::logic_error,
 * PBT_ENOMEM -> std::bad_alloc, PBT_ESINGULAR -> pbt::SingularBlock (a
 * std::runtime_error; the reference has no such report), PBT_ERANGE ->
 * pbt::ArithmeticRange (a std::range_error: a float-float / FP32 solve left its
 * arithmetic's range), PBT_ENOCONV -> std::runtime_error.  Header only; link
 * libpbt.so.
 */
#ifndef PBT_HPP
#define PBT_HPP

#include <new>
#include <stdexcept>
#include <string>
#include <utility>

#include "pbt.h"

namespace pbt {

class CudaError : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

class SingularBlock : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

class ArithmeticRange : public std::range_error {
public:
    using std::range_error::range_error;
};

inline void check(int status, const char* where) {
    if (status == PBT_OK) return;
    const std::string msg = std::string(where) + ": " + pbt_last_error_string();
    switch (status) {
        case PBT_EINVAL: throw std::invalid_argument(msg);
        case PBT_ECUDA: throw CudaError(msg);
        case PBT_EUNSUPPORTED: throw std::logic_error(msg);
        case PBT_ENOMEM: throw std::bad_alloc();
        case PBT_ESINGULAR: throw SingularBlock(msg);
        case PBT_ERANGE: throw ArithmeticRange(msg);
        default: throw std::runtime_error(msg);  // PBT_ESTATE, PBT_ETIMEOUT, PBT_ENOCONV
    }
}

struct BtdmaSolveTimings {
    double total = 0.0;
    double local_compute = 0.0;
    double forward_exchange = 0.0;
    double reduced_compute = 0.0;
    double backward_exchange = 0.0;
    double update_compute = 0.0;

    double computation() const { return local_compute + reduced_compute + update_compute; }
    double communication() const { return forward_exchange + backward_exchange; }
};

class BtdmaGpuPlan {
public:
    BtdmaGpuPlan() = default;
    BtdmaGpuPlan(int m, int nsys, int nrow, int nseg = 1) { create(m, nsys, nrow, nseg); }
    explicit BtdmaGpuPlan(const pbt_plan_desc& desc) { create(desc); }
    ~BtdmaGpuPlan() { pbt_plan_destroy(plan_); }
    BtdmaGpuPlan(const BtdmaGpuPlan&) = delete;
    BtdmaGpuPlan& operator=(const BtdmaGpuPlan&) = delete;
    BtdmaGpuPlan(BtdmaGpuPlan&& o) noexcept : plan_(std::exchange(o.plan_, nullptr)) {}
    BtdmaGpuPlan& operator=(BtdmaGpuPlan&& o) noexcept {
        if (this != &o) {
            pbt_plan_destroy(plan_);
            plan_ = std::exchange(o.plan_, nullptr);
        }
        return *this;
    }

    void create(int m, int nsys, int nrow, int nseg = 1) {
        pbt_plan_desc d;
        pbt_plan_desc_init(&d);
        d.m = m;
        d.nsys = nsys;
        d.nrow = nrow;
        d.nseg = nseg;
        create(d);
    }
    void create(const pbt_plan_desc& desc) {
        destroy();
        pbt_plan* p = nullptr;
        check(pbt_plan_create_ex(&p, &desc), "BtdmaGpuPlan::create");
        plan_ = p;
    }
    void destroy() {
        if (plan_) {
            pbt_plan* p = std::exchange(plan_, nullptr);
            check(pbt_plan_destroy(p), "BtdmaGpuPlan::destroy");
        }
    }
    bool created() const { return plan_ != nullptr; }
    pbt_plan* get() const { return plan_; }

    /* Zero pivots met since the last call (synchronises). */
    long long singular_count() {
        long long n = 0;
        const int rc = pbt_plan_status(plan_, &n);
        if (rc != PBT_ESINGULAR) check(rc, "BtdmaGpuPlan::singular_count");
        return n;
    }

private:
    pbt_plan* plan_ = nullptr;
};

inline void solve_noncyclic(BtdmaGpuPlan& plan, double* a, double* b, double* c, double* d, int m, int nsys,
                            int nrow, void* stream = nullptr) {
    check(pbt_solve_noncyclic(plan.get(), a, b, c, d, m, nsys, nrow, stream), "solve_noncyclic");
}

inline void solve_noncyclic_profiled(BtdmaGpuPlan& plan, double* a, double* b, double* c, double* d, int m,
                                     int nsys, int nrow, BtdmaSolveTimings* timings, void* stream = nullptr) {
    pbt_timings t{};
    check(pbt_solve_noncyclic_profiled(plan.get(), a, b, c, d, m, nsys, nrow, &t, stream),
          "solve_noncyclic_profiled");
    if (timings) {
        timings->total = t.total;
        timings->local_compute = t.local_compute;
        timings->forward_exchange = t.forward_exchange;
        timings->reduced_compute = t.reduced_compute;
        timings->backward_exchange = t.backward_exchange;
        timings->update_compute = t.update_compute;
    }
}

inline void solve_cyclic(BtdmaGpuPlan& plan, double* a, double* b, double* c, double* d, int m, int nsys, int nrow,
                         void* stream = nullptr) {
    check(pbt_solve_cyclic(plan.get(), a, b, c, d, m, nsys, nrow, stream), "solve_cyclic");
}

// Lines in the caller's own arrays (pbt_solve_noncyclic_lines; no reference
// counterpart: it replaces the transposes around each solve).
inline void solve_noncyclic_lines(BtdmaGpuPlan& plan, double* a, double* b, double* c, double* d,
                                  const pbt_lines& lines, void* stream = nullptr) {
    check(pbt_solve_noncyclic_lines(plan.get(), a, b, c, d, &lines, stream), "solve_noncyclic_lines");
}

inline std::pair<int, int> partition_1d(int start, int end, int nparts, int part) {
    int first = 0, last = -1;
    pbt_partition_1d(start, end, nparts, part, &first, &last);
    return {first, last};
}

}  // namespace pbt

#endif /* PBT_HPP */
