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

__device__ __forceinline__ df2 df_split(double x) {
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double df_to_double(df2 a) { return (double)a.h + (double)a.l; }

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
