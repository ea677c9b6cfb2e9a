// The learned factor preconditioner's inference: a message-passing net on
// the vertex graph writes a lower block-triangular L on H's lower block
// pattern after every assembly; the PCG applies M = L L^T.  The host module
// mfem_gb300/factor_net.py defines the net, trains it and holds its float32
// reference.  Not a reference function: the reference's PCG is block-Jacobi.
//
// Stages (one launch each, all on the caller's stream):
//   scale   d_i = tr(H_ii) / 3, s_i = d_i^-1/2, log10 d_i
//   input   aggregation weights w_ij = ||(S H S)_ij||_F, the 16 inputs and
//           h = relu(W_in x + b_in) on the FP32 pipe
//   mp x3   a_i = sum_j w_ij h_j / sum_j w_ij; h += relu(W [h, a] + b)
//   node    P h + b_p, Q h and the diagonal blocks L_ii
//   edge    L_ij = s_i (W_o relu(P h_i + b_p + Q h_j + R e_ij) + b_o)
// The dense layers run on the tensor cores (mma.sync m16n8k16, BF16
// operands, FP32 accumulation): a warp owns a tile of 16 vertices or blocks,
// stages its BF16 operand rows in shared memory and multiplies them by the
// layer's weights, which every CTA keeps in shared memory.
#include <algorithm>
#include <cstring>

#include "internal.h"

namespace mfem {
namespace {

constexpr int kNetWarps = 4;
constexpr int kNetThreads = 32 * kNetWarps;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    uint32_t u;
    memcpy(&u, &v, 4);
    return u;
}

__device__ __forceinline__ float2 unpack_bf16(uint32_t u) {
    __nv_bfloat162 v;
    memcpy(&v, &u, 4);
    return __bfloat1622float2(v);
}

__device__ __forceinline__ uint32_t ld_u32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }
__device__ __forceinline__ void st_u32(__nv_bfloat16 *p, uint32_t v) { *reinterpret_cast<uint32_t *>(p) = v; }

// D += A B for one 16x8 tile: A 16x16 (row-major BF16), B 16x8 (column-major
// BF16), D FP32.  Fragment layouts per the PTX ISA for m16n8k16.
__device__ __forceinline__ void mma_16816(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// acc[nt] += A (16 x K, shared, row stride lda) W^T for NT n-tiles of 8
// output columns; W is [out][ldw] (row n holds output n's K weights).
template <int NT, int K>
__device__ __forceinline__ void warp_gemm(float (*acc)[4], const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *W,
                                          int ldw, int n0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int k0 = 0; k0 < K; k0 += 16) {
        uint32_t a[4];
        a[0] = ld_u32(A + g * lda + k0 + 2 * t);
        a[1] = ld_u32(A + (g + 8) * lda + k0 + 2 * t);
        a[2] = ld_u32(A + g * lda + k0 + 8 + 2 * t);
        a[3] = ld_u32(A + (g + 8) * lda + k0 + 8 + 2 * t);
#pragma unroll
        for (int nt = 0; nt < NT; ++nt) {
            const __nv_bfloat16 *wr = W + (size_t)(n0 + nt * 8 + g) * ldw + k0;
            uint32_t b[2];
            b[0] = ld_u32(wr + 2 * t);
            b[1] = ld_u32(wr + 8 + 2 * t);
            mma_16816(acc[nt], a, b);
        }
    }
}

template <class T>
__device__ __forceinline__ void copy_to_shared(T *dst, const T *src, int count) {
    // count * sizeof(T) is a multiple of 16 for every weight array here
    const int n16 = count * (int)sizeof(T) / 16;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (int i = threadIdx.x; i < n16; i += blockDim.x) d4[i] = s4[i];
}

__device__ __forceinline__ float softplus(float x) { return x > 20.0f ? x : log1pf(expf(x)); }

// d_i, s_i, log10 d_i from the diagonal block (the last block of the row's
// lower part)
__global__ void fn_scale_kernel(BsrViews bv, BatchViews bw, FactorNetViews fv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bv.n) return;
    const float *h = bv.values + (size_t)9 * fv.lslot[bw.lrow[i + 1] - 1];
    const float d = (h[0] + h[4] + h[8]) * (1.0f / 3.0f);
    const bool ok = d > 0.0f && isfinite(d);
    fv.s[i] = ok ? rsqrtf(d) : 1.0f;
    fv.ld[i] = ok ? log10f(d) : 0.0f;
}

// aggregation weights, the inputs and the first layer (K = 16, FP32 pipe)
__global__ void __launch_bounds__(kNetThreads) fn_input_kernel(BsrViews bv, FactorNetViews fv) {
    __shared__ float sw[kNetWidth * kNetIn];
    __shared__ float sb[kNetWidth];
    for (int t = threadIdx.x; t < kNetWidth * kNetIn; t += blockDim.x) sw[t] = fv.w_in[t];
    for (int t = threadIdx.x; t < kNetWidth; t += blockDim.x) sb[t] = fv.b_in[t];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bv.n) return;
    const float si = fv.s[i];
    float wsum = 0.0f, ldsum = 0.0f;
    int cnt = 0, dslot = -1;
    const int kb = bv.row_ptr[i], ke = bv.row_ptr[i + 1];
    for (int k = kb; k < ke; ++k) {
        const int c = bv.col_idx[k];
        if (c == i) {
            fv.w[k] = 0.0f;
            dslot = k;
            continue;
        }
        const float *hk = bv.values + (size_t)9 * k;
        float f = 0.0f;
#pragma unroll
        for (int q = 0; q < 9; ++q) f = fmaf(hk[q], hk[q], f);
        const float wk = sqrtf(f) * (si * fv.s[c]);
        fv.w[k] = wk;
        wsum += wk;
        ldsum += fv.ld[c];
        ++cnt;
    }
    fv.winv[i] = wsum > 0.0f ? 1.0f / wsum : 0.0f;
    float x[kNetIn];
    const float *hd = bv.values + (size_t)9 * dslot;
    const float s2 = si * si;
    x[0] = hd[0] * s2 - 1.0f;
    x[1] = hd[4] * s2 - 1.0f;
    x[2] = hd[8] * s2 - 1.0f;
    x[3] = hd[1] * s2;
    x[4] = hd[2] * s2;
    x[5] = hd[5] * s2;
    x[6] = cnt > 0 ? fv.ld[i] - ldsum / (float)cnt : 0.0f;
#pragma unroll
    for (int q = 0; q < 4; ++q) x[7 + q] = fv.vstatic[4 * (size_t)i + q];
    x[11] = (float)(ke - kb) * (1.0f / 15.0f);
#pragma unroll
    for (int q = 12; q < kNetIn; ++q) x[q] = 0.0f;
    float *hrow = fv.h + (size_t)kNetWidth * i;
    __nv_bfloat16 *brow = fv.hb[0] + (size_t)kNetWidth * i;
    for (int j = 0; j < kNetWidth; j += 2) {
        float v0 = sb[j], v1 = sb[j + 1];
#pragma unroll
        for (int q = 0; q < kNetIn; ++q) {
            v0 = fmaf(sw[j * kNetIn + q], x[q], v0);
            v1 = fmaf(sw[(j + 1) * kNetIn + q], x[q], v1);
        }
        v0 = fmaxf(v0, 0.0f);
        v1 = fmaxf(v1, 0.0f);
        *reinterpret_cast<float2 *>(hrow + j) = make_float2(v0, v1);
        st_u32(brow + j, pack_bf16(v0, v1));
    }
}

// one message-passing layer: reads hb[src], writes h and hb[src ^ 1]
__global__ void __launch_bounds__(kNetThreads) fn_mp_kernel(BsrViews bv, FactorNetViews fv, int layer, int src) {
    __shared__ __align__(16) __nv_bfloat16 sW[kNetWidth * kMpLd];
    __shared__ __align__(16) __nv_bfloat16 sA[kNetWarps][16 * kMpLd];
    __shared__ float sb[kNetWidth];
    copy_to_shared(sW, fv.w_mp[layer], kNetWidth * kMpLd);
    for (int t = threadIdx.x; t < kNetWidth; t += blockDim.x) sb[t] = fv.b_mp[layer][t];
    __syncthreads();
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const __nv_bfloat16 *hin = fv.hb[src];
    __nv_bfloat16 *hout = fv.hb[src ^ 1];
    __nv_bfloat16 *A = sA[wid];
    const int tiles = (bv.n + 15) / 16;
    for (int tile = blockIdx.x * kNetWarps + wid; tile < tiles; tile += gridDim.x * kNetWarps) {
        const int base = tile * 16;
        // rows [h_i, a_i] in BF16: a quarter-warp per vertex (four at a
        // time), a lane owns 8 channels and gathers them with 16-byte loads
        const int quarter = lane >> 3, ql = lane & 7;
        for (int r0 = 0; r0 < 16; r0 += 4) {
            const int r = r0 + quarter, i = base + r;
            uint4 hq = make_uint4(0u, 0u, 0u, 0u), aq = hq;
            if (i < bv.n) {
                hq = *reinterpret_cast<const uint4 *>(hin + (size_t)kNetWidth * i + 8 * ql);
                float a[8];
#pragma unroll
                for (int q = 0; q < 8; ++q) a[q] = 0.0f;
                const int kb = bv.row_ptr[i], ke = bv.row_ptr[i + 1];
                int k = kb;
                for (; k + 2 <= ke; k += 2) {
                    const int c0 = __ldg(bv.col_idx + k), c1 = __ldg(bv.col_idx + k + 1);
                    const float w0 = __ldg(fv.w + k), w1 = __ldg(fv.w + k + 1);
                    const uint4 v0 = *reinterpret_cast<const uint4 *>(hin + (size_t)kNetWidth * c0 + 8 * ql);
                    const uint4 v1 = *reinterpret_cast<const uint4 *>(hin + (size_t)kNetWidth * c1 + 8 * ql);
                    const uint32_t u0[4] = {v0.x, v0.y, v0.z, v0.w}, u1[4] = {v1.x, v1.y, v1.z, v1.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float2 f0 = unpack_bf16(u0[q]), f1 = unpack_bf16(u1[q]);
                        a[2 * q] = fmaf(w1, f1.x, fmaf(w0, f0.x, a[2 * q]));
                        a[2 * q + 1] = fmaf(w1, f1.y, fmaf(w0, f0.y, a[2 * q + 1]));
                    }
                }
                if (k < ke) {
                    const int c0 = __ldg(bv.col_idx + k);
                    const float w0 = __ldg(fv.w + k);
                    const uint4 v0 = *reinterpret_cast<const uint4 *>(hin + (size_t)kNetWidth * c0 + 8 * ql);
                    const uint32_t u0[4] = {v0.x, v0.y, v0.z, v0.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float2 f0 = unpack_bf16(u0[q]);
                        a[2 * q] = fmaf(w0, f0.x, a[2 * q]);
                        a[2 * q + 1] = fmaf(w0, f0.y, a[2 * q + 1]);
                    }
                }
                const float wi = fv.winv[i];
                aq = make_uint4(pack_bf16(a[0] * wi, a[1] * wi), pack_bf16(a[2] * wi, a[3] * wi),
                                pack_bf16(a[4] * wi, a[5] * wi), pack_bf16(a[6] * wi, a[7] * wi));
            }
            *reinterpret_cast<uint4 *>(A + r * kMpLd + 8 * ql) = hq;
            *reinterpret_cast<uint4 *>(A + r * kMpLd + kNetWidth + 8 * ql) = aq;
        }
        __syncwarp();
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[nt][q] = 0.0f;
        warp_gemm<8, 2 * kNetWidth>(acc, A, kMpLd, sW, kMpLd, 0);
        // h += relu(acc + b); rows g and g + 8, columns nt * 8 + 2t, + 1
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int i = base + g + 8 * half;
            if (i >= bv.n) continue;
            float *hrow = fv.h + (size_t)kNetWidth * i;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int n = nt * 8 + 2 * t;
                const float2 h0 = *reinterpret_cast<const float2 *>(hrow + n);
                const float v0 = h0.x + fmaxf(acc[nt][2 * half] + sb[n], 0.0f);
                const float v1 = h0.y + fmaxf(acc[nt][2 * half + 1] + sb[n + 1], 0.0f);
                *reinterpret_cast<float2 *>(hrow + n) = make_float2(v0, v1);
                st_u32(hout + (size_t)kNetWidth * i + n, pack_bf16(v0, v1));
            }
        }
        __syncwarp();  // A is rewritten by the next tile
    }
}

// P h + b_p, Q h (BF16) and the diagonal blocks L_ii = s_i L~_ii
__global__ void __launch_bounds__(kNetThreads) fn_node_kernel(BsrViews bv, BatchViews bw, FactorNetViews fv, int src) {
    __shared__ __align__(16) __nv_bfloat16 sW[kNodeOut * kNodeLd];
    __shared__ __align__(16) __nv_bfloat16 sA[kNetWarps][16 * kNodeLd];
    __shared__ float sb[kNodeOut];
    __shared__ float sD[kNetWarps][16][8];
    copy_to_shared(sW, fv.w_node, kNodeOut * kNodeLd);
    for (int t = threadIdx.x; t < kNodeOut; t += blockDim.x) sb[t] = fv.b_node[t];
    __syncthreads();
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const __nv_bfloat16 *hin = fv.hb[src];
    __nv_bfloat16 *A = sA[wid];
    const int tiles = (bv.n + 15) / 16;
    for (int tile = blockIdx.x * kNetWarps + wid; tile < tiles; tile += gridDim.x * kNetWarps) {
        const int base = tile * 16;
        for (int r = 0; r < 16; ++r) {
            const int i = base + r;
            st_u32(A + r * kNodeLd + 2 * lane, i < bv.n ? ld_u32(hin + (size_t)kNetWidth * i + 2 * lane) : 0u);
        }
        __syncwarp();
        float acc[kNodeOut / 8][4];
#pragma unroll
        for (int nt = 0; nt < kNodeOut / 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[nt][q] = 0.0f;
        warp_gemm<kNodeOut / 8, kNetWidth>(acc, A, kNodeLd, sW, kNodeLd, 0);
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int r = g + 8 * half, i = base + r;
#pragma unroll
            for (int nt = 0; nt < kNodeOut / 8; ++nt) {
                const int n = nt * 8 + 2 * t;
                const float v0 = acc[nt][2 * half] + sb[n], v1 = acc[nt][2 * half + 1] + sb[n + 1];
                if (nt < 16) {
                    if (i < bv.n) {
                        __nv_bfloat16 *dst = (nt < 8 ? fv.pb : fv.qb) + (size_t)kNetWidth * i + (n & (kNetWidth - 1));
                        st_u32(dst, pack_bf16(v0, v1));
                    }
                } else {
                    sD[wid][r][n - 2 * kNetWidth] = v0;
                    sD[wid][r][n - 2 * kNetWidth + 1] = v1;
                }
            }
        }
        __syncwarp();
        if (lane < 16 && base + lane < bv.n) {
            const int i = base + lane;
            const float *o = sD[wid][lane];
            const float si = fv.s[i];
            float *L = bw.Lval + (size_t)9 * (bw.lrow[i + 1] - 1);
            L[0] = si * softplus(o[0]);
            L[1] = 0.0f;
            L[2] = 0.0f;
            L[3] = si * o[3];
            L[4] = si * softplus(o[1]);
            L[5] = 0.0f;
            L[6] = si * o[4];
            L[7] = si * o[5];
            L[8] = si * softplus(o[2]);
        }
        __syncwarp();
    }
}

// off-diagonal lower blocks, 16 per warp tile
__global__ void __launch_bounds__(kNetThreads) fn_edge_kernel(BsrViews bv, BatchViews bw, FactorNetViews fv) {
    __shared__ __align__(16) __nv_bfloat16 sWr[kNetWidth * kRLd];
    __shared__ __align__(16) __nv_bfloat16 sWo[16 * kNodeLd];
    __shared__ float sbo[16];
    __shared__ __align__(16) __nv_bfloat16 sE[kNetWarps][16 * kRLd];
    __shared__ __align__(16) __nv_bfloat16 sZ[kNetWarps][16 * kNodeLd];
    __shared__ int sI[kNetWarps][16], sJ[kNetWarps][16], sL[kNetWarps][16];
    __shared__ float sS[kNetWarps][16];
    copy_to_shared(sWr, fv.w_r, kNetWidth * kRLd);
    copy_to_shared(sWo, fv.w_o, 16 * kNodeLd);
    for (int t = threadIdx.x; t < 16; t += blockDim.x) sbo[t] = fv.b_o[t];
    __syncthreads();
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    __nv_bfloat16 *E = sE[wid];
    __nv_bfloat16 *Z = sZ[wid];
    const int tiles = (fv.n_edges + 15) / 16;
    for (int tile = blockIdx.x * kNetWarps + wid; tile < tiles; tile += gridDim.x * kNetWarps) {
        const int e0 = tile * 16;
        if (lane < 16) {
            const int e = e0 + lane;
            int i = -1, j = 0, l = 0;
            float si = 0.0f;
            float ev[16];
#pragma unroll
            for (int q = 0; q < 16; ++q) ev[q] = 0.0f;
            if (e < fv.n_edges) {
                i = fv.erow[e];
                l = fv.elow[e];
                j = bw.lcol[l];
                si = fv.s[i];
                const float sc = si * fv.s[j];
                const float *hk = bv.values + (size_t)9 * fv.lslot[l];
#pragma unroll
                for (int q = 0; q < 9; ++q) ev[q] = hk[q] * sc;
            }
#pragma unroll
            for (int q = 0; q < 16; q += 2) st_u32(E + lane * kRLd + q, pack_bf16(ev[q], ev[q + 1]));
            sI[wid][lane] = i;
            sJ[wid][lane] = j;
            sL[wid][lane] = l;
            sS[wid][lane] = si;
        }
        __syncwarp();
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[nt][q] = 0.0f;
        warp_gemm<8, 16>(acc, E, kRLd, sWr, kRLd, 0);
        // z = relu(P h_i + b_p + Q h_j + R e) in BF16
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int r = g + 8 * half;
            const int i = sI[wid][r], j = sJ[wid][r];
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int n = nt * 8 + 2 * t;
                uint32_t zp = 0u;
                if (i >= 0) {
                    const float2 p = unpack_bf16(ld_u32(fv.pb + (size_t)kNetWidth * i + n));
                    const float2 q = unpack_bf16(ld_u32(fv.qb + (size_t)kNetWidth * j + n));
                    zp = pack_bf16(fmaxf(p.x + q.x + acc[nt][2 * half], 0.0f),
                                   fmaxf(p.y + q.y + acc[nt][2 * half + 1], 0.0f));
                }
                st_u32(Z + r * kNodeLd + n, zp);
            }
        }
        __syncwarp();
        float out[2][4];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) out[nt][q] = 0.0f;
        warp_gemm<2, kNetWidth>(out, Z, kNodeLd, sWo, kNodeLd, 0);
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            const int r = g + 8 * half;
            if (sI[wid][r] < 0) continue;
            float *L = bw.Lval + (size_t)9 * sL[wid][r];
            const float si = sS[wid][r];
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int n = nt * 8 + 2 * t + u;
                    if (n < 9) L[n] = si * (out[nt][2 * half + u] + sbo[n]);
                }
        }
        __syncwarp();
    }
}

// CTAs for `tiles` warp tiles: the kernels stride over tiles, so the grid
// is only bounded (a few waves of the GPU's resident CTAs)
int grid_for(int tiles, int per_cta) {
    const int ctas = (tiles + per_cta - 1) / per_cta;
    return std::max(1, std::min(ctas, 1 << 14));
}

}  // namespace

cudaError_t launch_factor_net(const BsrViews &bv, const BatchViews &bw, const FactorNetViews &fv, cudaStream_t s) {
    if (bv.n == 0) return cudaSuccess;
    const int n = bv.n;
    fn_scale_kernel<<<(n + 255) / 256, 256, 0, s>>>(bv, bw, fv);
    fn_input_kernel<<<(n + kNetThreads - 1) / kNetThreads, kNetThreads, 0, s>>>(bv, fv);
    const int node_tiles = (n + 15) / 16;
    int src = 0;
    for (int layer = 0; layer < 3; ++layer, src ^= 1)
        fn_mp_kernel<<<grid_for(node_tiles, kNetWarps), kNetThreads, 0, s>>>(bv, fv, layer, src);
    fn_node_kernel<<<grid_for(node_tiles, kNetWarps), kNetThreads, 0, s>>>(bv, bw, fv, src);
    count_launches(6);
    if (fv.n_edges > 0) {
        fn_edge_kernel<<<grid_for((fv.n_edges + 15) / 16, kNetWarps), kNetThreads, 0, s>>>(bv, bw, fv);
        count_launches(1);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_factor_transpose(bw, s);
    return e;
}

}  // namespace mfem
