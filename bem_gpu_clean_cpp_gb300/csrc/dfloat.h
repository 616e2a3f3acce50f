// Double-float arithmetic on the FP32 pipe (FP64-class accuracy where the
// FP64 pipe is the bottleneck).
#pragma once

#include <cuda_runtime.h>

namespace bem {

// ---- double-float accumulation for the FP64 refinement residuals ----
// The entries of a c64 matrix are exact floats.  A product a*xh (xh the float
// head of an FP64 value) is split exactly into p + e by TwoProduct (FMA), p is
// added to the running head with TwoSum (Knuth), and all the low-order parts
// go into a float tail; x's own tail xl contributes a*xl to the tail.  The
// result (head + tail, summed in FP64 at the end) is accurate to ~1e-13
// relative while the kernel runs on the FP32 pipe, so the FP64-accurate
// residual costs one HBM pass over A instead of FP64 FMA throughput.  _rn
// intrinsics keep the compiler from contracting the error-free transforms.
__device__ __forceinline__ void df_mac(float &hi, float &lo, float a, float xh, float xl) {
    const float p = __fmul_rn(a, xh);
    const float e = fmaf(a, xh, -p);
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = fmaf(a, xl, __fadd_rn(lo, __fadd_rn(err, e)));
}

// hi + lo += v: v added to the head by TwoSum, the rounding error into the
// tail (a sum of n floats accurate to ~n u^2 of the sum of magnitudes).
__device__ __forceinline__ void df_add(float &hi, float &lo, float v) {
    const float s = __fadd_rn(hi, v);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(v, bb));
    hi = s;
    lo = __fadd_rn(lo, err);
}
// (hi, lo) += (hi2, lo2); the same result with the operands swapped (TwoSum's
// error term is exact, the tails' sum commutative).
__device__ __forceinline__ void df_add2(float &hi, float &lo, float hi2, float lo2) {
    const float s = __fadd_rn(hi, hi2);
    const float bb = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(hi2, bb));
    hi = s;
    lo = __fadd_rn(__fadd_rn(lo, lo2), err);
}

// ---- double-float values (head, tail) as float2 ----
// a + b, with the result renormalised by TwoSum (no magnitude assumption).
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    float e1, e2;
    const float s = __fadd_rn(a.x, b.x);
    {
        const float bb = __fsub_rn(s, a.x);
        e1 = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    }
    const float t = __fadd_rn(e1, __fadd_rn(a.y, b.y));
    const float u = __fadd_rn(s, t);
    {
        const float bb = __fsub_rn(u, s);
        e2 = __fadd_rn(__fsub_rn(s, __fsub_rn(u, bb)), __fsub_rn(t, bb));
    }
    return make_float2(u, e2);
}
__device__ __forceinline__ float2 ff_neg(float2 a) { return make_float2(-a.x, -a.y); }
// a b: the heads' product split exactly (FMA), the cross terms added to its
// error, renormalised by TwoSum.
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    const float e = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, __fmaf_rn(a.x, b.x, -p)));
    const float u = __fadd_rn(p, e);
    const float bb = __fsub_rn(u, p);
    return make_float2(u, __fadd_rn(__fsub_rn(p, __fsub_rn(u, bb)), __fsub_rn(e, bb)));
}

}  // namespace bem
