// df64.cuh -- double-float arithmetic: a value is an unevaluated sum hi + lo of two FP32 numbers
// (|lo| <= ulp(hi)/2), about 48 significant bits.
//
// GB300 issues FP32 at 64x its FP64 rate, so long FP64 dot products run faster as FP32 pairs.
// The building blocks are the error-free transformations of Knuth (two-sum: a + b = s + e
// exactly) and Dekker (two-product, here with one FMA: a * b = p + e exactly), the double-word
// arithmetic of Dekker (1971) and of Hida, Li & Bailey's quad-double papers (2001).
// The error-free steps must not be contracted into FMAs or re-associated: they use the
// round-to-nearest intrinsics (__fadd_rn, __fsub_rn, __fmul_rn), which the compiler never fuses,
// and the exact product error is an explicit fmaf.
// Range: FP32 pairs underflow below ~1e-38 and lose their low word below ~1e-31; callers keep
// vanishingly small operands on an FP64 path.
#pragma once

#include <cuda_runtime.h>

namespace klsa {

struct df2 {
    float h, l;
};

__device__ __forceinline__ df2 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// requires |a| >= |b| (or a == 0)
__device__ __forceinline__ df2 df_quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// GB300 runs conversions between FP64 and FP32 on its FP64 pipe, at the FP64 rate.  The split of
// a double into a pair and the widening of a pair's halves are therefore done with integer
// operations on the IEEE-754 fields (sign, biased exponent, mantissa), which run on the integer
// pipes; only the final FP64 addition of a widening is FP64 work.

// x = h + l: h = x truncated to 24 significant bits, l = the remaining 29 mantissa bits rounded
// to 24; |x - h - l| <= 2^-47 |x| + 1.2e-38 once both halves are widened again (l can fall below
// the normal float range when |x| < 2^-74).  |x| < 2^-126 gives (0, 0); |x| >= 2^128,
// infinities and NaN take the hardware conversion (they propagate).
__device__ __forceinline__ df2 df_split(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned hw = static_cast<unsigned>(b >> 32);
    const int e = static_cast<int>((hw >> 20) & 0x7ffu);   // biased exponent (bias 1023)
    if (e >= 1151) return {__double2float_rn(x), 0.f};
    if (e < 897) return {0.f, 0.f};
    const unsigned sign = hw & 0x80000000u;
    const unsigned long long mant = b & 0x000FFFFFFFFFFFFFull;
    const float h = __uint_as_float(sign | (static_cast<unsigned>(e - 896) << 23) | static_cast<unsigned>(mant >> 29));
    // l = r 2^(E - 52) with E = e - 1023 and r the low 29 bits; the power of two is applied in
    // two factors when it lies below the normal float range
    const unsigned r = static_cast<unsigned>(mant) & 0x1FFFFFFFu;
    const int E = e - 1023;
    const bool deep = E < -74;
    const float scale = __uint_as_float(static_cast<unsigned>(E - 52 + (deep ? 64 : 0) + 127) << 23);
    float l = __uint2float_rn(r) * scale;
    if (deep) l *= 5.42101086242752217e-20f;   // 2^-64
    return {h, __uint_as_float(__float_as_uint(l) | sign)};
}

// exact widening of a normal float; zero and subnormals give a signed zero (absolute error below
// 1.2e-38), infinities and NaN are kept
__device__ __forceinline__ double df_widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long s = static_cast<unsigned long long>(u & 0x80000000u) << 32;
    const unsigned long long de = e == 0 ? 0ull : (e == 255 ? 2047ull : e + 896ull);
    const unsigned long long m = e == 0 ? 0ull : static_cast<unsigned long long>(u & 0x7fffffu) << 29;
    return __longlong_as_double(static_cast<long long>(s | (de << 52) | m));
}

__device__ __forceinline__ double df_to_double(df2 a) { return df_widen(a.h) + df_widen(a.l); }

// a * b, both operands double-float
__device__ __forceinline__ df2 df_mul(df2 a, df2 b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    return df_quick_two_sum(p, e);
}

// acc += a * b
__device__ __forceinline__ void df_fma(df2& acc, df2 a, df2 b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    df2 s = df_two_sum(acc.h, p);
    s.l = __fadd_rn(s.l, __fadd_rn(e, acc.l));
    acc = df_quick_two_sum(s.h, s.l);
}

// acc -= a * b
__device__ __forceinline__ void df_fms(df2& acc, df2 a, df2 b) { df_fma(acc, {-a.h, -a.l}, b); }

}  // namespace klsa
