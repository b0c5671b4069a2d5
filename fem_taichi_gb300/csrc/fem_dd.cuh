// Double-float ("dd") arithmetic on the FP32 pipes.
//
// A value is an unevaluated pair hi + lo of floats with |lo| <= ulp(hi) / 2 (about 48
// significant bits).  GB300 executes FP32 instructions ~64x faster than FP64 ones, so the
// element integrals run in this format and only the final values are formed in FP64.
// The error-free transformations (Knuth's two-sum, Dekker's fast-two-sum, the FMA-based
// exact product) use the __f*_rn intrinsics so that the compiler can neither contract a
// multiply-add into an FMA nor reorder the operations they rely on.
#pragma once

#include <stdint.h>

namespace fem {

struct dd {
    float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ dd fast_two_sum(float a, float b) {  // requires |a| >= |b| (or a == 0)
    const float s = __fadd_rn(a, b);
    return dd{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dd dd_from_float(float a) { return dd{a, 0.f}; }

// Exact split of an FP64 value (used only for inputs: coordinates, material constants).
__device__ __forceinline__ dd dd_from_double(double x) {
    const float hi = __double2float_rn(x);
    return dd{hi, __double2float_rn(x - double(hi))};
}

__device__ __forceinline__ dd dd_add(dd a, dd b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s, e);
}

__device__ __forceinline__ dd dd_neg(dd a) { return dd{-a.hi, -a.lo}; }
__device__ __forceinline__ dd dd_sub(dd a, dd b) { return dd_add(a, dd_neg(b)); }

__device__ __forceinline__ dd dd_mul(dd a, dd b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

// a * b for a float b (exact constants)
__device__ __forceinline__ dd dd_mul_f(dd a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return fast_two_sum(p, e);
}

// 1 / a by one Newton step from the float reciprocal
__device__ __forceinline__ dd dd_rcp(dd a) {
    const float r = __frcp_rn(a.hi);
    // residual 1 - a r computed in dd
    const dd ar = dd_mul(a, dd_from_float(r));
    const dd res = dd_sub(dd_from_float(1.f), ar);
    return dd_add(dd_from_float(r), dd_mul_f(res, r));
}

__device__ __forceinline__ dd dd_div(dd a, dd b) { return dd_mul(a, dd_rcp(b)); }

__device__ __forceinline__ dd dd_abs(dd a) { return a.hi < 0.f ? dd_neg(a) : a; }

// sqrt by one Newton step from the float square root (a >= 0)
__device__ __forceinline__ dd dd_sqrt(dd a) {
    if (!(a.hi > 0.f)) return dd{0.f, 0.f};
    const float s = __fsqrt_rn(a.hi);
    const float ps = __fmul_rn(s, s);
    const float pe = __fmaf_rn(s, s, -ps);  // s*s = ps + pe exactly
    const dd res = dd_sub(a, dd{ps, pe});
    return dd_add(dd_from_float(s), dd_mul_f(res, __fdividef(0.5f, s)));
}

__device__ __forceinline__ bool dd_lt(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

// Unnormalised accumulator for sums of products: value = s + c.
struct dd_acc {
    float s, c;
};

__device__ __forceinline__ dd_acc acc_zero() { return dd_acc{0.f, 0.f}; }

__device__ __forceinline__ void acc_fma(dd_acc& acc, dd a, dd b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    float s, t;
    two_sum(acc.s, p, s, t);
    acc.s = s;
    acc.c = __fadd_rn(acc.c, __fadd_rn(t, e));
}

__device__ __forceinline__ void acc_add(dd_acc& acc, dd a) {
    float s, t;
    two_sum(acc.s, a.hi, s, t);
    acc.s = s;
    acc.c = __fadd_rn(acc.c, __fadd_rn(t, a.lo));
}

__device__ __forceinline__ dd acc_value(dd_acc acc) {
    float s, e;
    two_sum(acc.s, acc.c, s, e);
    return dd{s, e};
}

// Nearest-below double of hi + lo built with integer operations only (no FP64 pipe).
// The result is within 2^-52 relative of hi + lo; NaN/Inf/zero/denormal hi are handled.
__device__ __forceinline__ double dd_to_double(dd v) {
    const uint32_t bh = __float_as_uint(v.hi), bl = __float_as_uint(v.lo);
    const uint32_t eh = (bh >> 23) & 0xffu;
    const uint64_t sign = uint64_t(bh >> 31) << 63;
    if (eh == 0xffu) {  // Inf / NaN
        const uint64_t man = uint64_t(bh & 0x7fffffu) << 29;
        return __longlong_as_double(int64_t(sign | (uint64_t(0x7ff) << 52) | man));
    }
    if (eh == 0u) {  // zero or denormal hi: |value| < 2^-126, return lo (or 0)
        const uint32_t el = (bl >> 23) & 0xffu;
        if (el == 0u) return 0.0;
        const uint64_t sl = uint64_t(bl >> 31) << 63;
        return __longlong_as_double(int64_t(sl | (uint64_t(el - 127 + 1023) << 52) | (uint64_t(bl & 0x7fffffu) << 29)));
    }
    int64_t T = int64_t(uint64_t((bh & 0x7fffffu) | 0x800000u) << 29);  // 53-bit significand of hi
    int e = int(eh) - 127 + 1023;
    const uint32_t el = (bl >> 23) & 0xffu;
    if (el != 0u && el != 0xffu) {
        const uint64_t ml = uint64_t((bl & 0x7fffffu) | 0x800000u);
        const int sh = int(eh) - int(el) - 29;  // lo in units of hi's 2^-52 ulp: ml * 2^-sh
        int64_t L = 0;
        if (sh >= 0) L = sh < 63 ? int64_t(ml >> sh) : 0;
        else L = int64_t(ml << (-sh));
        if ((bh >> 31) == (bl >> 31)) T += L;
        else T -= L;
    }
    if (T >= (int64_t(1) << 53)) {
        T >>= 1;
        e += 1;
    } else if (T < (int64_t(1) << 52)) {
        T <<= 1;
        e -= 1;
    }
    return __longlong_as_double(int64_t(sign | (uint64_t(e) << 52) | (uint64_t(T) & ((uint64_t(1) << 52) - 1))));
}

}  // namespace fem
