// double_float.cuh — pairs of floats as extended-precision values on the
// FP32 pipe (GB300 issues FP64 at 1/64 of the FP32 rate).
#pragma once

#include <cuda_runtime.h>

namespace nufi_gb300 {

// Double-float arithmetic: a value as a pair of floats (hi, lo), hi + lo
// its value to about 2^-48 relative, with Dekker's fast two-sum, Knuth's
// two-sum and the two-product by one FMA (T. J. Dekker, "A floating-point
// technique for extending the available precision", Numer. Math. 18,
// 1971).  Every operation goes through the _rn intrinsics, which the
// compiler never contracts into an FMA: the error-free transformations need
// each rounding as written.
struct ff {
    float hi, lo;
};
__device__ __forceinline__ ff ff_of(double x)
{
    const float h = __double2float_rn(x);
    return {h, __double2float_rn(x - double(h))};
}
__device__ __forceinline__ double ff_value(ff a) { return double(a.hi) + double(a.lo); }
// hi + lo renormalised, |s| >= |e| (Dekker's fast two-sum)
__device__ __forceinline__ ff ff_norm(float s, float e)
{
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
// a + b: Knuth's two-sum of the high parts, the low parts added to its error
__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return ff_norm(s, e);
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
// a b: the exact product of the high parts (its error by one FMA) plus the
// cross terms (a.lo b.lo, below 2^-48 of the product, dropped)
__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return ff_norm(p, e);
}
// a b + c
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float pe = __fmaf_rn(a.hi, b.hi, -p);
    pe = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, pe));
    const float s = __fadd_rn(p, c.hi);
    const float bb = __fsub_rn(s, p);
    float e = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(c.hi, bb));
    e = __fadd_rn(e, __fadd_rn(pe, c.lo));
    return ff_norm(s, e);
}
// a times a power of two (exact)
__device__ __forceinline__ ff ff_scale2(ff a, float s) { return {__fmul_rn(a.hi, s), __fmul_rn(a.lo, s)}; }

}  // namespace nufi_gb300
