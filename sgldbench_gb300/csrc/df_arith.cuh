// Double-float arithmetic: a value is an unevaluated sum hi + lo of two FP32
// numbers (48 significant bits).  Sums use Knuth's TwoSum on the high parts
// followed by a fast renormalisation; products use the FMA form of Dekker's
// exact product.  GB300 issues FP32 at about 64 times its FP64 rate, so these
// ~7-11 FP32 operations per add or multiply are cheaper than one FP64
// operation in issue-bound kernels.
#pragma once

namespace sgld {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_from(double v) {
    const float h = __double2float_rn(v);
    return {h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

// The error-free transforms must not be contracted or reassociated, so every
// operation is an explicitly rounded intrinsic (nvcc never fuses those).
__device__ __forceinline__ df quick_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df a, df b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return quick_two_sum(s, e);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_mul(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return quick_two_sum(p, e);
}

__device__ __forceinline__ df df_shfl(df v, int src, int width = 32) {
    return {__shfl_sync(0xffffffffu, v.hi, src, width), __shfl_sync(0xffffffffu, v.lo, src, width)};
}

// Compensated double-float dot-product accumulator (the Dot2 scheme of Ogita,
// Rump and Oishi, 2005, with the low parts of the operands folded into the
// error term): s + e carries the running sum.
struct dacc {
    float s = 0.f, e = 0.f;
    __device__ __forceinline__ void add(float2 a, float2 b) {
        const float p = __fmul_rn(a.x, b.x);
        float pe = __fmaf_rn(a.x, b.x, -p);
        pe = __fmaf_rn(a.x, b.y, pe);
        pe = __fmaf_rn(a.y, b.x, pe);
        const float t = __fadd_rn(s, p);
        const float bb = __fsub_rn(t, s);
        const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
        s = t;
        e = __fadd_rn(e, __fadd_rn(err, pe));
    }
    __device__ __forceinline__ df value() const { return quick_two_sum(s, e); }
};

}  // namespace sgld
