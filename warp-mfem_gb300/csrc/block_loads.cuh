// Loads of one 3x3 block from global memory through the read-only path,
// shared by the PCG kernels.  Blocks are 36 bytes (fp32) or 20 bytes (BF16
// with one padding value), so block k starts on an 8-byte boundary for even
// k and 4 bytes past one for odd k (from a cudaMalloc'd base): four 8-byte
// loads and one 4-byte load instead of nine (fp32), two and one instead of
// five (BF16).
#pragma once

#include <cuda_bf16.h>

#include <cstdint>
#include <cstring>

namespace mfem {

__device__ __forceinline__ void load_block9(const float *values, long long k, float m[9]) {
    const bool odd = (k & 1) != 0;
    const float *h = values + 9 * k;
    const float2 *b2 = reinterpret_cast<const float2 *>(h + (odd ? 1 : 0));
    const float2 p0 = __ldg(b2), p1 = __ldg(b2 + 1), p2 = __ldg(b2 + 2), p3 = __ldg(b2 + 3);
    const float t = __ldg(odd ? h : h + 8);
    m[0] = odd ? t : p0.x;
    m[1] = odd ? p0.x : p0.y;
    m[2] = odd ? p0.y : p1.x;
    m[3] = odd ? p1.x : p1.y;
    m[4] = odd ? p1.y : p2.x;
    m[5] = odd ? p2.x : p2.y;
    m[6] = odd ? p2.y : p3.x;
    m[7] = odd ? p3.x : p3.y;
    m[8] = odd ? p3.y : t;
}

// The five words (BF16 pairs) of block k of a factor form.
__device__ __forceinline__ void load_bf16_words(const uint32_t *words, long long k, uint32_t u[5]) {
    const bool odd = (k & 1) != 0;
    const uint32_t *w = words + 5 * k;
    const uint2 *b2 = reinterpret_cast<const uint2 *>(w + (odd ? 1 : 0));
    const uint2 q0 = __ldg(b2), q1 = __ldg(b2 + 1);
    const uint32_t t = __ldg(odd ? w : w + 4);
    u[0] = odd ? t : q0.x;
    u[1] = odd ? q0.x : q0.y;
    u[2] = odd ? q0.y : q1.x;
    u[3] = odd ? q1.x : q1.y;
    u[4] = odd ? q1.y : t;
}

// Five words of BF16 pairs as the 3x3 block's nine floats.
__device__ __forceinline__ void bf16_words_to_block(const uint32_t u[5], float f[9]) {
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        __nv_bfloat162 b;
        memcpy(&b, &u[i], 4);
        const float2 t = __bfloat1622float2(b);
        f[2 * i] = t.x;
        if (2 * i + 1 < 9) f[2 * i + 1] = t.y;
    }
}

}  // namespace mfem
