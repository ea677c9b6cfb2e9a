// Double-float arithmetic: a value held as the unevaluated sum hi + lo of two
// floats (about 48 bits), with the error-free transformations TwoSum (Knuth,
// TAOCP vol. 2, 4.2.2) and TwoProduct by fused multiply-add (Ogita, Rump &
// Oishi, "Accurate sum and dot product", 2005), all with round-to-nearest
// intrinsics so that nothing is contracted.  GB300's fp64 rate is a small
// fraction of its fp32 rate; the refinement's residual products run in these
// pairs instead of in double.
#pragma once

#include <cuda_runtime.h>

namespace mfem {

__device__ __forceinline__ float2 two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}

// |a| >= |b| (or a == 0)
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float2 s = two_sum(a.x, b.x);
    return fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}

__device__ __forceinline__ float2 df_add(float2 a, float b) {
    const float2 s = two_sum(a.x, b);
    return fast_two_sum(s.x, __fadd_rn(s.y, a.y));
}

// acc += h (x.hi + x.lo)
__device__ __forceinline__ void df_fma(float2 &acc, float h, float2 x) {
    const float p = __fmul_rn(h, x.x);
    float pe = __fmaf_rn(h, x.x, -p);  // h x.hi = p + pe exactly
    pe = __fmaf_rn(h, x.y, pe);
    const float2 s = two_sum(acc.x, p);
    acc = fast_two_sum(s.x, __fadd_rn(__fadd_rn(s.y, pe), acc.y));
}

__device__ __forceinline__ float2 df_shfl_xor(unsigned mask, float2 v, int off) {
    return make_float2(__shfl_xor_sync(mask, v.x, off), __shfl_xor_sync(mask, v.y, off));
}

// g - (acc.hi + acc.lo) in double
__device__ __forceinline__ double df_residual(float g, float2 acc) {
    const float2 r = df_add(two_sum(g, -acc.x), -acc.y);
    return (double)r.x + (double)r.y;
}

}  // namespace mfem
