// Device helpers of the fp16 split operands (tc_gemm.cu and the QR's own
// packing kernels): power-of-two scales, the split into fp16 parts and the
// packed-plane stores.
#pragma once

#include <cuda_fp16.h>

namespace bem {

// The P fp16 parts of v (already scaled).
template <int P>
__device__ __forceinline__ void split_parts(float v, __half (&h)[3]) {
    h[0] = __float2half_rn(v);
    float r = v - __half2float(h[0]);
    h[1] = __float2half_rn(r);
    if (P == 3) {
        r -= __half2float(h[1]);
        h[2] = __float2half_rn(r);
    }
}

// v rounded to 11 significant bits (fp16's precision) by Dekker's splitting
// (c = (2^13 + 1) v, hi = c - (c - v)): three FP32 operations, exactly
// representable in fp16 for |hi| >= 2^-14; v - hi is exact.
__device__ __forceinline__ float dekker_hi11(float v) {
    const float c = __fmul_rn(v, 8193.0f);
    return __fsub_rn(c, __fsub_rn(c, v));
}

__device__ __forceinline__ uint32_t half2_bits(__half2 h) {
    return *reinterpret_cast<const uint32_t *>(&h);
}

// The P fp16 parts of the pair (a, b) (already scaled), each part packed as
// a half2: the same parts as split_parts in fp16's normal range, with one
// packed conversion per part instead of three scalar conversions per value
// (below 2^-14 the head is rounded once more into fp16's subnormals, an
// absolute error of at most 2^-25).
template <int P>
__device__ __forceinline__ void split_pair(float a, float b, uint32_t (&out)[3]) {
    const float ha = dekker_hi11(a), hb = dekker_hi11(b);
    out[0] = half2_bits(__floats2half2_rn(ha, hb));
    const float ra = __fsub_rn(a, ha), rb = __fsub_rn(b, hb);
    if (P == 2) {
        out[1] = half2_bits(__floats2half2_rn(ra, rb));
    } else {
        const float ma = dekker_hi11(ra), mb = dekker_hi11(rb);
        out[1] = half2_bits(__floats2half2_rn(ma, mb));
        out[2] = half2_bits(__floats2half2_rn(__fsub_rn(ra, ma), __fsub_rn(rb, mb)));
    }
}

// Power-of-two scale of a column from its largest magnitude.
__device__ __forceinline__ float pow2_scale(float amax) {
    if (!(amax > 0.f) || !isfinite(amax)) return 1.f;
    int ex;
    frexpf(amax, &ex);                         // amax = f 2^ex, f in [0.5, 1)
    ex = max(-100, min(100, ex));
    return ldexpf(1.f, 15 - ex);               // amax * scale in [2^14, 2^15)
}

// Largest of v over the CTA (all threads get it); red: 32 floats of shared memory.
__device__ __forceinline__ float block_max(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) red[0] = v;
    }
    __syncthreads();
    const float r = red[0];
    __syncthreads();
    return r;
}

// Stores the P parts of (a, b) at idx, idx + 1 of every plane.
template <int P>
__device__ __forceinline__ void put_parts(__half *planes, size_t plane_stride, size_t idx, float a, float b) {
    __half ha[3], hb[3];
    split_parts<P>(a, ha);
    split_parts<P>(b, hb);
#pragma unroll
    for (int p = 0; p < P; p++) {
        __half2 w;
        w.x = ha[p];
        w.y = hb[p];
        *reinterpret_cast<__half2 *>(planes + p * plane_stride + idx) = w;
    }
}

}  // namespace bem
