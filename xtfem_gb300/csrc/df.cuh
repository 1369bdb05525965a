// df.cuh -- double-float arithmetic: a value held as hi + lo in two FP32
// numbers with |lo| <= ulp(hi)/2 (about 48 significant bits).  GB300 runs
// FP32 at 64 times its FP64 rate, so FP64-accurate sums and products that
// sit on a hot path are formed this way.  Knuth's two-sum keeps the rounding
// error of every addition and an fma recovers the error of every leading
// product; explicit _rn intrinsics keep the compiler from fusing or
// reordering the error-free steps.
#pragma once

#include <cuda_runtime.h>

namespace xt {

// (hi, lo) += x
__device__ __forceinline__ void df_add(float& hi, float& lo, float x)
{
    const float s = __fadd_rn(hi, x);
    const float bb = __fsub_rn(s, hi);
    const float t = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb));
    hi = s;
    lo = __fadd_rn(lo, t);
}

// (hi, lo) += (xh + xl)
__device__ __forceinline__ void df_add_df(float& hi, float& lo, float xh, float xl)
{
    df_add(hi, lo, xh);
    lo = __fadd_rn(lo, xl);
}

// (hi, lo) += (ah + al)(bh + bl): the leading product exactly (fma), the
// cross terms in FP32 (their rounding is below the format's precision).
__device__ __forceinline__ void df_mul_acc(float& hi, float& lo, float ah, float al, float bh,
                                           float bl)
{
    const float p = __fmul_rn(ah, bh);
    const float e = fmaf(ah, bh, -p);
    df_add(hi, lo, p);
    lo = __fadd_rn(lo, __fadd_rn(e, fmaf(ah, bl, __fmul_rn(al, bh))));
}

// Two double-float accumulators side by side, (h.x + l.x, h.y + l.y) +=
// (vh + vl) (x.x, x.y) for FP32 x: the steps of an FP32-input axpy (leading
// product exact by fma, two-sum of the sum, the low part's products in
// FP32) on packed two-wide FP32 instructions, each element rounded exactly
// as the scalar sequence would round it.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ void df2_axpy(float2& h, float2& l, float vh, float vl, float2 x)
{
    const float2 v = make_float2(vh, vh);
    const float2 p = __fmul2_rn(v, x);
    const float2 e = __ffma2_rn(v, x, neg2(p));
    const float2 s = __fadd2_rn(h, p);
    const float2 bb = __fadd2_rn(s, neg2(h));
    const float2 t = __fadd2_rn(__fadd2_rn(h, neg2(__fadd2_rn(s, neg2(bb)))), __fadd2_rn(p, neg2(bb)));
    h = s;
    l = __fadd2_rn(l, t);
    l = __fadd2_rn(l, __ffma2_rn(make_float2(vl, vl), x, e));
}

// Renormalise (hi, lo) so that hi carries the rounded value.
__device__ __forceinline__ float2 df_norm(float hi, float lo)
{
    const float s = __fadd_rn(hi, lo);
    return make_float2(s, __fsub_rn(lo, __fsub_rn(s, hi)));
}

}  // namespace xt
