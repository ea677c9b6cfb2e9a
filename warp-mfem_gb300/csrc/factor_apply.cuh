// One pass of a factor preconditioner, shared by the global-memory PCGs: out
// = F in over rows [lo, hi) for one form of the factor (row pointers,
// columns, row-major 3x3 blocks in BF16, kFactorLd values per block), `group`
// lanes per row.  `in` is read with __ldcg (other CTAs wrote it during this
// launch) unless LOCAL says this CTA's own stores, ordered by __syncthreads,
// are the only writers.
#pragma once

#include <cstring>

#include "block_loads.cuh"
#include "internal.h"

namespace mfem {

// the 3x3 block k of a BF16 factor form (kFactorLd values per block)
__device__ __forceinline__ void factor_block(const __nv_bfloat16 *val, int k, float f[9]) {
    uint32_t u[5];
    load_bf16_words(reinterpret_cast<const uint32_t *>(val), k, u);
    bf16_words_to_block(u, f);
}

template <bool LOCAL, int GROUP>
__device__ __forceinline__ void factor_pass(const int *rp, const int *col, const __nv_bfloat16 *val, const float *in,
                                            float *out, int lo, int hi) {
    const int g_lane = threadIdx.x & (GROUP - 1);
    const unsigned gmask = ((1u << GROUP) - 1u) << (threadIdx.x & (32 - GROUP));
    const int group = threadIdx.x / GROUP, ngroups = blockDim.x / GROUP;
    auto ld = [](const float *p) { return LOCAL ? *p : __ldcg(p); };
    for (int row = lo + group; row < hi; row += ngroups) {
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
        const int ke = __ldg(rp + row + 1);
        // two blocks per lane and trip: their loads are in flight together
        for (int k = __ldg(rp + row) + g_lane; k < ke; k += 2 * GROUP) {
            const int k2 = k + GROUP;
            const bool two = k2 < ke;
            const int c = __ldg(col + k), c2 = two ? __ldg(col + k2) : c;
            const float v0 = ld(in + 3 * c), v1 = ld(in + 3 * c + 1), v2 = ld(in + 3 * c + 2);
            float w0 = ld(in + 3 * c2), w1 = ld(in + 3 * c2 + 1), w2 = ld(in + 3 * c2 + 2);
            if (!two) w0 = w1 = w2 = 0.0f;
            float f[9], f2[9];
            factor_block(val, k, f);
            factor_block(val, two ? k2 : k, f2);
            a0 += f[0] * v0 + f[1] * v1 + f[2] * v2;
            a1 += f[3] * v0 + f[4] * v1 + f[5] * v2;
            a2 += f[6] * v0 + f[7] * v1 + f[8] * v2;
            a0 += f2[0] * w0 + f2[1] * w1 + f2[2] * w2;
            a1 += f2[3] * w0 + f2[4] * w1 + f2[5] * w2;
            a2 += f2[6] * w0 + f2[7] * w1 + f2[8] * w2;
        }
#pragma unroll
        for (int off = GROUP / 2; off > 0; off >>= 1) {
            a0 += __shfl_xor_sync(gmask, a0, off);
            a1 += __shfl_xor_sync(gmask, a1, off);
            a2 += __shfl_xor_sync(gmask, a2, off);
        }
        if (g_lane == 0) {
            out[3 * row] = a0;
            out[3 * row + 1] = a1;
            out[3 * row + 2] = a2;
        }
    }
}

// The two passes of M r for mode 2 (M = F^T F: lower form first) or mode 3
// (M = F F^T: upper form first), as (row pointers, columns, values) pairs.
struct FactorForms {
    const int *rp0, *c0, *rp1, *c1;
    const __nv_bfloat16 *v0, *v1;
};

__device__ __forceinline__ FactorForms factor_forms(const BatchViews &bw, int mode) {
    const bool lower_first = mode == 2;
    FactorForms f;
    f.rp0 = lower_first ? bw.lrow : bw.urow;
    f.c0 = lower_first ? bw.lcol : bw.ucol;
    f.v0 = lower_first ? bw.Lb : bw.Ub;
    f.rp1 = lower_first ? bw.urow : bw.lrow;
    f.c1 = lower_first ? bw.ucol : bw.lcol;
    f.v1 = lower_first ? bw.Ub : bw.Lb;
    return f;
}

}  // namespace mfem
