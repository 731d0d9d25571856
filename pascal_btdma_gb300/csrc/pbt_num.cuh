// pbt_num.cuh -- the arithmetics the solver kernels are written over.
//
//   F64: plain IEEE double on the FP64 pipe (1/63 of the FP32 rate on GB300).
//   FF:  float-float ("double-single") arithmetic on the FP32 pipes.  A value
//        is an unevaluated sum h + l of two floats with |l| <= ulp(h)/2, which
//        carries ~47 significant bits.  The operations are built from the
//        error-free transformations TwoSum (Knuth, TAOCP vol. 2, 4.2.2),
//        FastTwoSum (Dekker 1971) and the FMA form of TwoProduct (Ogita, Rump,
//        Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005).
//        Each multiply-accumulate costs 12 FP32 instructions, i.e. ~5x the
//        FP64 pipe's rate.
//   F32: plain float, the factorisation arithmetic of the iteratively refined
//        solve (see k_residual64 in pbt_kernels.cuh).
//
// Every kernel uses the same small interface:
//   T            register value;  Acc: an accumulator for sums of products
//   in(p)        load an FP64 matrix element (A, B, C) and convert to T
//   in_rhs(p)    the same for a right-hand-side element (D)
//   out(p, v)    convert T to FP64 and store (f64(v): the converted value)
//   lds/sts      raw 8-byte workspace slots (no conversion); from_raw: a slot's
//                8 bytes already in a register
//   acc(x), mac(acc, x, y) (acc += x*y), msub(acc, x, y) (acc -= x*y), fin(acc)
//   mul, rcp, neg, zero, one, key (|x| as an ordered integer), sel, is_zero
//   nonfinite(v), mag(v), kTinyMag: the solution range check (no-ops for F64)
//
// FP64 <-> FF conversion uses integer bit operations only, so the FF path
// issues no FP64 instruction except one DADD per FP64 value it writes.
// FF and F32 take matrix entries of magnitude 2^-96 <= |x| < 2^96 (and zero);
// any other entry converts to NaN and the solve reports it (kBadRange).
// Right-hand sides convert without the lower edge (split_wide): entries tiny
// next to the rest of the system's are negligible, and a whole solution too
// small to carry is caught by the output check.
#pragma once

#include <cstdint>

#include "pbt_internal.h"

namespace pbt {

__device__ __forceinline__ float fsel(unsigned s, float x, float y) {
    float r;
    asm("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %3, 0;\n\tselp.f32 %0, %1, %2, p;\n\t}"
        : "=f"(r)
        : "f"(x), "f"(y), "r"(s));
    return r;
}

__device__ __forceinline__ double dsel(unsigned s, double x, double y) {
    double r;
    asm("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %3, 0;\n\tselp.f64 %0, %1, %2, p;\n\t}"
        : "=d"(r)
        : "d"(x), "d"(y), "r"(s));
    return r;
}

// ---------------------------------------------------------------------------
struct F64 {
    using T = double;
    struct Acc {
        double v;
    };
    static constexpr bool kConv = false;  // raw workspace values differ from FP64?

    __device__ static __forceinline__ T in(const double* p) { return *p; }
    __device__ static __forceinline__ T in_ro(const double* p) { return __ldg(p); }
    __device__ static __forceinline__ T in_rhs(const double* p) { return *p; }
    __device__ static __forceinline__ void out(double* p, T v) { *p = v; }
    __device__ static __forceinline__ double f64(T v) { return v; }
    __device__ static __forceinline__ T lds(const double* p) { return *p; }
    __device__ static __forceinline__ void sts(double* p, T v) { *p = v; }
    // A raw 8-byte slot already loaded into a register.
    __device__ static __forceinline__ T from_raw(double v) { return v; }

    __device__ static __forceinline__ Acc acc(T x) { return {x}; }
    __device__ static __forceinline__ Acc acc0() { return {0.0}; }
    __device__ static __forceinline__ void mac(Acc& a, T x, T y) { a.v = fma(x, y, a.v); }
    __device__ static __forceinline__ void msub(Acc& a, T x, T y) { a.v = fma(-x, y, a.v); }
    __device__ static __forceinline__ T fin(Acc a) { return a.v; }

    __device__ static __forceinline__ T mul(T a, T b) { return a * b; }
    __device__ static __forceinline__ T rcp(T a) { return __drcp_rn(a); }
    __device__ static __forceinline__ T neg(T a) { return -a; }
    __device__ static __forceinline__ T zero() { return 0.0; }
    __device__ static __forceinline__ T one() { return 1.0; }
    __device__ static __forceinline__ unsigned long long key(T a) {
        return static_cast<unsigned long long>(__double_as_longlong(a)) & 0x7fffffffffffffffull;
    }
    __device__ static __forceinline__ T sel(unsigned s, T x, T y) { return dsel(s, x, y); }
    __device__ static __forceinline__ Acc asel(unsigned s, Acc x, Acc y) { return {dsel(s, x.v, y.v)}; }
    __device__ static __forceinline__ unsigned long long akey(Acc a) { return key(a.v); }
    __device__ static __forceinline__ bool is_zero(T a) { return key(a) == 0ull; }
    // FP64 carries the reference's own range: no output check.
    __device__ static __forceinline__ bool nonfinite(T) { return false; }
    __device__ static __forceinline__ unsigned mag(T) { return 0u; }
    static constexpr unsigned kTinyMag = 0u;
};

// ---------------------------------------------------------------------------
struct ff {
    float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // needs |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// Biased FP64 exponents of the magnitudes the float-float and FP32
// conversions accept: 2^-96 <= |x| < 2^96.
constexpr unsigned kFFExpLo = 1023u - 96u;
constexpr unsigned kFFExpHi = 1023u + 95u;

struct FF {
    using T = ff;
    struct Acc {
        float s, t;  // unnormalised: value = s + t, t collects rounding errors and low parts
    };
    static constexpr bool kConv = true;

    // FP64 -> (h, l) by bit manipulation: h = x truncated to 24 significant
    // bits, l = the next 23 bits, so |x - (h + l)| < 2^-46 |x|.  Only zero
    // and magnitudes in the window [2^-96, 2^96) convert (kFFExpLo..kFFExpHi):
    // there l is never below 2^-120, and a product of two such values stays
    // inside FP32's range.  Anything else -- a nonzero |x| < 2^-96 (FP64
    // subnormals read as zero), |x| >= 2^96, Inf, NaN -- becomes a NaN, which
    // every later operation carries into the solution, where the output check
    // (nonfinite) reports it: an input the arithmetic cannot carry gives a
    // reported failure, never a silently wrong number.
    __device__ static __forceinline__ T split(double x) {
        const unsigned hi = static_cast<unsigned>(__double2hiint(x));
        const unsigned lo = static_cast<unsigned>(__double2loint(x));
        const unsigned e = (hi >> 20) & 0x7ffu;
        const unsigned sign = hi & 0x80000000u;
        // h: rebias the exponent (1023 -> 127) and keep 23 mantissa bits.
        const unsigned hb = __funnelshift_l(lo, (hi & 0x7fffffffu) - (896u << 20), 3) | sign;
        // l: the 23 bits below h's mantissa as a float with an explicit leading
        // one, minus that one (exact).
        const unsigned eb = (e - 919u) << 23;
        const float lf = __fsub_rn(__uint_as_float(eb | ((lo >> 6) & 0x7fffffu)), __uint_as_float(eb));
        const unsigned lb = __float_as_uint(lf) | sign;
        const bool in = (e - kFFExpLo) <= (kFFExpHi - kFFExpLo);
        const unsigned out = (e != 0u) ? 0x7fc00000u : 0u;  // outside the window: NaN; zero: 0
        return {__uint_as_float(in ? hb : out), __uint_as_float(in ? lb : 0u)};
    }
    // The same conversion without the window, for right-hand sides and the
    // library's own intermediates (the reduced rows of a segmented plan after
    // an FP64 sub-solve, a refinement residual): |x| < 2^-126 gives 0,
    // 2^-126 <= |x| < 2^-103 keeps h only, |x| >= 2^128 and Inf/NaN give NaN.
    // Entries that small are negligible next to the rest of a right-hand side
    // (the solve is linear in it), next to the reduced system's identity
    // diagonal blocks, or as the correction of a converged iterate; a whole
    // solution that small is caught by the output check, and an overflow is a
    // NaN in the solution.
    __device__ static __forceinline__ T split_wide(double x) {
        const unsigned hi = static_cast<unsigned>(__double2hiint(x));
        const unsigned lo = static_cast<unsigned>(__double2loint(x));
        const unsigned e = (hi >> 20) & 0x7ffu;
        const unsigned sign = hi & 0x80000000u;
        const unsigned hb = __funnelshift_l(lo, (hi & 0x7fffffffu) - (896u << 20), 3) | sign;
        const unsigned eb = (e - 919u) << 23;
        const float lf = __fsub_rn(__uint_as_float(eb | ((lo >> 6) & 0x7fffffu)), __uint_as_float(eb));
        const unsigned lb = __float_as_uint(lf) | sign;
        const unsigned h = (e > 1150u) ? 0x7fc00000u : (e > 896u ? hb : 0u);
        return {__uint_as_float(h), __uint_as_float((e >= 920u && e <= 1150u) ? lb : 0u)};
    }

    // float -> double by bit manipulation: normal floats exactly, Inf and NaN
    // to FP64 Inf and NaN, zero and subnormals to signed zero.
    __device__ static __forceinline__ double widen(float f) {
        const unsigned u = __float_as_uint(f);
        const unsigned a = u & 0x7fffffffu;
        const unsigned s = u & 0x80000000u;
        unsigned hiw = (a >= 0x00800000u) ? (s | ((a >> 3) + (896u << 20))) : s;
        hiw = (a >= 0x7f800000u) ? (s | 0x7ff00000u | ((a >> 3) & 0x000fffffu)) : hiw;
        const unsigned low = (a >= 0x00800000u) ? (a << 29) : 0u;
        return __hiloint2double(static_cast<int>(hiw), static_cast<int>(low));
    }
    __device__ static __forceinline__ double join(T v) { return widen(v.h) + widen(v.l); }
    // Whether a value is Inf or NaN (its high part decides).
    __device__ static __forceinline__ bool nonfinite(T v) { return (__float_as_uint(v.h) & 0x7fffffffu) >= 0x7f800000u; }
    // |v| as an ordered integer (high part), Inf/NaN above every finite value.
    __device__ static __forceinline__ unsigned mag(T v) { return __float_as_uint(v.h) & 0x7fffffffu; }
    // A solution whose largest |x| is below 2^-100 has subnormal low words:
    // the pairs no longer carry 47 bits.
    static constexpr unsigned kTinyMag = (127u - 100u) << 23;

    __device__ static __forceinline__ T in(const double* p) { return split(*p); }
    __device__ static __forceinline__ T in_ro(const double* p) { return split(__ldg(p)); }
    __device__ static __forceinline__ T in_rhs(const double* p) { return split_wide(*p); }
    __device__ static __forceinline__ void out(double* p, T v) { *p = join(v); }
    __device__ static __forceinline__ double f64(T v) { return join(v); }
    __device__ static __forceinline__ T lds(const double* p) {
        const float2 f = *reinterpret_cast<const float2*>(p);
        return {f.x, f.y};
    }
    __device__ static __forceinline__ void sts(double* p, T v) { *reinterpret_cast<float2*>(p) = make_float2(v.h, v.l); }
    __device__ static __forceinline__ T from_raw(double v) {
        return {__int_as_float(__double2loint(v)), __int_as_float(__double2hiint(v))};
    }

    __device__ static __forceinline__ Acc acc(T x) { return {x.h, x.l}; }
    __device__ static __forceinline__ Acc acc0() { return {0.f, 0.f}; }
    // a += x*y: exact product of the high parts, the two cross terms folded
    // into its error, the high sum by TwoSum, all errors into a.t.
    __device__ static __forceinline__ void mac(Acc& a, T x, T y) {
        const float p = __fmul_rn(x.h, y.h);
        float e = __fmaf_rn(x.h, y.h, -p);
        e = __fmaf_rn(x.h, y.l, e);
        e = __fmaf_rn(x.l, y.h, e);
        const ff s = two_sum(a.s, p);
        a.s = s.h;
        a.t = __fadd_rn(a.t, __fadd_rn(s.l, e));
    }
    __device__ static __forceinline__ void msub(Acc& a, T x, T y) { mac(a, {-x.h, -x.l}, y); }
    __device__ static __forceinline__ T fin(Acc a) { return two_sum(a.s, a.t); }

    __device__ static __forceinline__ T mul(T a, T b) {
        const float p = __fmul_rn(a.h, b.h);
        float e = __fmaf_rn(a.h, b.h, -p);
        e = __fmaf_rn(a.h, b.l, e);
        e = __fmaf_rn(a.l, b.h, e);
        return fast_two_sum(p, e);
    }
    // 1/a: r0 = rcp(a.h); one Newton step r0 + r0*(1 - a*r0), where
    // 1 - a.h*r0 is exact in one FMA.
    __device__ static __forceinline__ T rcp(T a) {
        const float r0 = __frcp_rn(a.h);
        float e = __fmaf_rn(-a.h, r0, 1.0f);
        e = __fmaf_rn(-a.l, r0, e);
        return fast_two_sum(r0, __fmul_rn(r0, e));
    }
    __device__ static __forceinline__ T neg(T a) { return {-a.h, -a.l}; }
    __device__ static __forceinline__ T zero() { return {0.f, 0.f}; }
    __device__ static __forceinline__ T one() { return {1.f, 0.f}; }
    __device__ static __forceinline__ unsigned key(T a) { return __float_as_uint(a.h) & 0x7fffffffu; }
    __device__ static __forceinline__ T sel(unsigned s, T x, T y) { return {fsel(s, x.h, y.h), fsel(s, x.l, y.l)}; }
    __device__ static __forceinline__ Acc asel(unsigned s, Acc x, Acc y) { return {fsel(s, x.s, y.s), fsel(s, x.t, y.t)}; }
    // Pivot key of an accumulator: its high part decides.
    __device__ static __forceinline__ unsigned akey(Acc a) { return __float_as_uint(a.s) & 0x7fffffffu; }
    __device__ static __forceinline__ bool is_zero(T a) { return key(a) == 0u; }
};

// ---------------------------------------------------------------------------
// F32: plain IEEE float, for the FP32 factorisation of the refined solve.
// Inputs are truncated to float on load; raw workspace slots (8 bytes) hold
// the float in their first 4 bytes.
struct F32 {
    using T = float;
    struct Acc {
        float v;
    };
    static constexpr bool kConv = true;

    // Conversions by bit manipulation (the high part of FF::split /
    // FF::split_wide truncates to 24 bits; FF::widen is exact): GB300 runs F2F
    // conversions with a double operand at the FP64 rate, which would cost
    // more than the solve itself.  Matrix entries take float-float's window
    // (a row scaled out of it cannot be refined: its residuals fall below
    // FP32's range); right-hand sides and residuals convert without it.
    __device__ static __forceinline__ T in(const double* p) { return FF::split(*p).h; }
    __device__ static __forceinline__ T in_ro(const double* p) { return FF::split(__ldg(p)).h; }
    __device__ static __forceinline__ T in_rhs(const double* p) { return FF::split_wide(*p).h; }
    __device__ static __forceinline__ void out(double* p, T v) { *p = FF::widen(v); }
    __device__ static __forceinline__ double f64(T v) { return FF::widen(v); }
    // Raw slots are written whole (the float and a zero pad), so every 32-byte
    // sector of a warp's store is complete and L2 never has to fetch the rest.
    __device__ static __forceinline__ T lds(const double* p) { return reinterpret_cast<const float2*>(p)->x; }
    __device__ static __forceinline__ void sts(double* p, T v) { *reinterpret_cast<float2*>(p) = make_float2(v, 0.f); }
    __device__ static __forceinline__ T from_raw(double v) { return __int_as_float(__double2loint(v)); }

    __device__ static __forceinline__ Acc acc(T x) { return {x}; }
    __device__ static __forceinline__ Acc acc0() { return {0.f}; }
    __device__ static __forceinline__ void mac(Acc& a, T x, T y) { a.v = __fmaf_rn(x, y, a.v); }
    __device__ static __forceinline__ void msub(Acc& a, T x, T y) { a.v = __fmaf_rn(-x, y, a.v); }
    __device__ static __forceinline__ T fin(Acc a) { return a.v; }

    __device__ static __forceinline__ T mul(T a, T b) { return __fmul_rn(a, b); }
    __device__ static __forceinline__ T rcp(T a) { return __frcp_rn(a); }
    __device__ static __forceinline__ T neg(T a) { return -a; }
    __device__ static __forceinline__ T zero() { return 0.f; }
    __device__ static __forceinline__ T one() { return 1.f; }
    __device__ static __forceinline__ unsigned key(T a) { return __float_as_uint(a) & 0x7fffffffu; }
    __device__ static __forceinline__ T sel(unsigned s, T x, T y) { return fsel(s, x, y); }
    __device__ static __forceinline__ Acc asel(unsigned s, Acc x, Acc y) { return {fsel(s, x.v, y.v)}; }
    __device__ static __forceinline__ unsigned akey(Acc a) { return key(a.v); }
    __device__ static __forceinline__ bool is_zero(T a) { return key(a) == 0u; }
    __device__ static __forceinline__ bool nonfinite(T v) { return (__float_as_uint(v) & 0x7fffffffu) >= 0x7f800000u; }
    __device__ static __forceinline__ unsigned mag(T v) { return __float_as_uint(v) & 0x7fffffffu; }
    // The FP32 pass checks Inf/NaN only; the refinement checks the size of
    // its FP64 solution (k_accumulate, k_refine_step, k_refine_staged).
    static constexpr unsigned kTinyMag = 0u;
};

// Per-thread outcome bits of a solve, reported into the plan's status word at
// the end of a kernel (report_status).
constexpr unsigned kBadPivot = 1u;  // a zero pivot was met
constexpr unsigned kBadRange = 2u;  // the solution left the float-float / FP32 range

// The range check of a thread's solution (float-float and FP32; nothing for
// FP64).  `amax` is the largest Num::mag of the values the thread wrote.
// kBadRange if a value came out Inf/NaN -- an input outside the conversion
// window, or an overflow on the way -- or, with `whole` (the values are a
// whole system's solution) in float-float, if the largest |x| is nonzero and
// below Num::kTinyMag.
template <class Num>
__device__ __forceinline__ unsigned range_bits(unsigned amax, bool whole) {
    if constexpr (!Num::kConv) {
        return 0u;
    } else {
        const bool tiny = whole && amax != 0u && amax < Num::kTinyMag;
        return (amax >= 0x7f800000u || tiny) ? kBadRange : 0u;
    }
}
// A thread's outcome into a status word (layout in pbt_internal.h).
__device__ __forceinline__ void report_status(unsigned long long* status, unsigned bad) {
    if (bad & kBadPivot) atomicAdd(status, 1ull);
    if (bad & kBadRange) atomicOr(status, kRangeMark);
}

}  // namespace pbt
