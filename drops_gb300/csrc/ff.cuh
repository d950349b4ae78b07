// Float-float ("pair") arithmetic for FP64-accurate work on the FP32 pipe.
//
// GB300 retires FP64 at 1/64 of its FP32 rate, so FP64-bound kernels run a
// number as an unevaluated pair hi + lo of floats (|lo| <= ulp(hi) / 2 after
// normalisation, ~48 significant bits).  Products use the exact FMA residual
// (Dekker's TwoProduct with FMA), sums Knuth's TwoSum on the high parts with
// the low parts added (the "sloppy" pair sum: error ~2^-44 of the operands'
// magnitudes, also under cancellation).  Every operation names its rounding
// through the _rn intrinsics, so the compiler neither contracts nor
// reorders them.  Exponent range: that of FP32 normals for the high part;
// the splits below fall back to conversions outside it.
#pragma once

#include <cuda_runtime.h>

namespace tf {

struct ff {
    float h, l;
};

__device__ __forceinline__ ff ff_of(float h) { return ff{h, 0.f}; }

// s + e == a + b exactly (TwoSum, no magnitude condition)
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return ff{s, e};
}

// s + e == a + b exactly when |a| >= |b| or a == 0 (Fast2Sum)
__device__ __forceinline__ ff ff_fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return ff{s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = ff_two_sum(a.h, b.h);
    return ff_fast_two_sum(s.h, __fadd_rn(__fadd_rn(a.l, b.l), s.l));
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.h, -a.l}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return ff_fast_two_sum(p, e);
}

// a * b for a float b
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
    const float p = __fmul_rn(a.h, b);
    float e = __fmaf_rn(a.h, b, -p);
    e = __fmaf_rn(a.l, b, e);
    return ff_fast_two_sum(p, e);
}

// scaling by a power of two (exact; any other factor needs ff_mul_f)
__device__ __forceinline__ ff ff_scale(ff a, float pow2) { return ff{__fmul_rn(a.h, pow2), __fmul_rn(a.l, pow2)}; }

// a + b for a float b
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    const ff s = ff_two_sum(a.h, b);
    return ff_fast_two_sum(s.h, __fadd_rn(a.l, s.l));
}

// a * b + c
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }

// Accumulator (sh, sl) += a * b, left unnormalised (the low part collects the
// product residuals and the TwoSum errors; read it once, at the end).
struct ffacc {
    float h = 0.f, l = 0.f;
    __device__ __forceinline__ void add_prod(ff a, ff b) {
        const float p = __fmul_rn(a.h, b.h);
        const float pe = __fmaf_rn(a.h, b.h, -p);
        const float t = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, pe));
        const ff s = ff_two_sum(h, p);
        h = s.h;
        l = __fadd_rn(l, __fadd_rn(s.l, t));
    }
    __device__ __forceinline__ void add(ff a) {
        const ff s = ff_two_sum(h, a.h);
        h = s.h;
        l = __fadd_rn(l, __fadd_rn(s.l, a.l));
    }
    __device__ __forceinline__ ff value() const { return ff_fast_two_sum(h, l); }
};

// 1/sqrt(s) for s > 0 in the FP32 normal range: the FP32 estimate and two
// Newton steps y <- y + y (1 - s y^2) / 2 with the residual formed in pair
// arithmetic (the first step leaves ~1.5 e0^2 <= 2^-43, the second ~2^-47).
__device__ __forceinline__ ff ff_rsqrt(ff s) {
    const float y0 = rsqrtf(s.h);
    // r0 = 1 - s y0^2; y0^2 exactly as a pair
    const float q = __fmul_rn(y0, y0);
    const ff sq = ff_mul(s, ff{q, __fmaf_rn(y0, y0, -q)});
    const float r0 = __fsub_rn(__fsub_rn(1.0f, sq.h), sq.l);
    ff y = ff_fast_two_sum(y0, __fmul_rn(__fmul_rn(0.5f, y0), r0));
    const ff sy2 = ff_mul(s, ff_mul(y, y));
    const float r1 = __fsub_rn(__fsub_rn(1.0f, sy2.h), sy2.l);
    return ff_add_f(y, __fmul_rn(__fmul_rn(0.5f, y.h), r1));
}

// sqrt(s); s below 2^-100 (and s <= 0) gives 0, keeping every step in the
// FP32 normal range (the result is then below 2^-50)
__device__ __forceinline__ ff ff_sqrt(ff s) { return s.h > 7.8886091e-31f ? ff_mul(s, ff_rsqrt(s)) : ff_of(0.f); }

// double -> pair.  Integer path (no conversion, which GB300 runs on its
// narrow FP64 pipe): hi = the top 24 significand bits (truncated), lo = the
// remaining 29 bits normalised and truncated to 24, |x - hi - lo| <= 2^-47 |x|;
// valid while lo is a normal float (|x| in [2^-74, 2^100]).  Outside that
// range (and for non-finite x) the conversions of the FP64 pipe.
__device__ __forceinline__ ff ff_split(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    if ((b << 1) == 0ull) return ff{0.f, 0.f};
    const unsigned e = (unsigned)(b >> 52) & 0x7ffu, sgn = (unsigned)(b >> 63) << 31;
    if (e < 949u || e > 1123u) {
        const float h = __double2float_rn(x);
        return ff{h, __double2float_rn(x - (double)h)};
    }
    const unsigned long long mant = b & 0xfffffffffffffull;
    const unsigned hb = sgn | ((e - 896u) << 23) | (unsigned)(mant >> 29);
    const unsigned rem = (unsigned)(mant & 0x1fffffffu);
    unsigned lb = 0u;
    if (rem) {
        const int lz = __clz((int)rem);          // >= 3
        const unsigned p = 31u - (unsigned)lz;   // leading bit of rem
        const unsigned m23 = (unsigned)((((unsigned long long)rem << (lz + 1)) & 0xffffffffull) >> 9);
        lb = sgn | ((p + e - 948u) << 23) | m23;  // rem * 2^(e - 1075)
    }
    return ff{__int_as_float((int)hb), __int_as_float((int)lb)};
}

// pair -> double (two conversions and an add on the FP64 pipe)
__device__ __forceinline__ double ff_to_double(ff a) { return __dadd_rn((double)a.h, (double)a.l); }

}  // namespace tf
