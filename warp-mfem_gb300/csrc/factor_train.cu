// Training kernels of the learned factor preconditioner: the dense layers'
// forward and backward products as BF16 tensor-core GEMMs with FP32
// accumulation, and the Adam update.  The host trainer
// (mfem_gb300/factor_net.py, train) writes the net's backward pass by hand
// around these; no framework autograd or optimizer is involved.  No
// reference counterpart: the reference's PCG is block-Jacobi.
//
// gemm_bf16_kernel: C[M][N] = op(A)[M][K] op(B)[K][N] (or C += ...), with
// op(A) = A ([M][K] row-major) or A^T (A stored [K][M]), op(B) = B ([K][N])
// or B^T (B stored [N][K]).  The three products of a linear layer y = x W^T:
//   forward  Y  = X W^T     (A = X, B = W stored [N][K]: B transposed)
//   dX       dX = dY W      (A = dY, B = W stored [K][N])
//   dW       dW = dY^T X    (A = dY stored [K][M]: A transposed, B = X)
// Operands are read as FP32, rounded to BF16 where they are staged in shared
// memory (so every product is BF16-in / FP32-accumulate), and multiplied with
// mma.sync m16n8k16.  A CTA computes a 64 x 64 tile of C over a K range;
// long K (dW sums over every vertex or block) is split over grid.z into
// per-split partial tiles that gemm_reduce_kernel adds in split order, so the
// result does not depend on scheduling.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "internal.h"

namespace mfem {
namespace {

constexpr int kGm = 64, kGn = 64, kGk = 32;
constexpr int kGpad = 8;  // bf16 padding of a staged row: 80-byte rows keep the fragment loads conflict-free
constexpr int kGThreads = 128;

__device__ __forceinline__ void mma_bf16_16816(float d[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t lds_u32(const __nv_bfloat16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

struct GemmArgs {
    int M, N, K;
    const float *A;
    int lda;
    const float *B;
    int ldb;
    float *C;  // splits == 1: the output (ldc); else the partials [splits][M][N]
    int ldc;
    int accumulate;  // splits == 1: C += product
    int k_chunk;     // K range of one split (a multiple of kGk)
};

// Stages the [64 rows][32 k] tile starting at (r0, k0) of a logical
// row-major operand X[rows][K] into S[row][k] as BF16.  TRANS: X is stored
// [K][rows] with leading dimension ld; else [rows][K].
template <bool TRANS>
__device__ __forceinline__ void stage_tile(__nv_bfloat16 (*S)[kGk + kGpad], const float *__restrict__ X, int ld,
                                           int rows, int r0, int k0, int k_end) {
#pragma unroll
    for (int u = 0; u < (kGm * kGk) / kGThreads; ++u) {
        const int i = u * kGThreads + threadIdx.x;
        int r, k;
        if (TRANS) {  // consecutive threads along rows: contiguous in memory
            k = i / kGm;
            r = i - k * kGm;
        } else {      // consecutive threads along k
            r = i / kGk;
            k = i - r * kGk;
        }
        const int gr = r0 + r, gk = k0 + k;
        float v = 0.0f;
        if (gr < rows && gk < k_end) v = TRANS ? X[(size_t)gk * ld + gr] : X[(size_t)gr * ld + gk];
        S[r][k] = __float2bfloat16_rn(v);
    }
}

template <bool A_T, bool B_T>
__global__ void __launch_bounds__(kGThreads) gemm_bf16_kernel(GemmArgs g) {
    __shared__ __align__(16) __nv_bfloat16 As[kGm][kGk + kGpad];
    __shared__ __align__(16) __nv_bfloat16 Bs[kGn][kGk + kGpad];
    const int m0 = blockIdx.x * kGm, n0 = blockIdx.y * kGn;
    const int kb = blockIdx.z * g.k_chunk;
    const int ke = min(g.K, kb + g.k_chunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gq = lane >> 2, tq = lane & 3;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;  // the warp's 32 x 32 sub-tile
    float acc[2][4][4] = {};
    for (int k0 = kb; k0 < ke; k0 += kGk) {
        // op(A) rows are C's rows; op(B) is staged by output column n
        stage_tile<A_T>(As, g.A, g.lda, g.M, m0, k0, ke);
        stage_tile<!B_T>(Bs, g.B, g.ldb, g.N, n0, k0, ke);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kGk; kk += 16) {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt) {
                const int r = wm + mt * 16 + gq;
                a[mt][0] = lds_u32(&As[r][kk + 2 * tq]);
                a[mt][1] = lds_u32(&As[r + 8][kk + 2 * tq]);
                a[mt][2] = lds_u32(&As[r][kk + 8 + 2 * tq]);
                a[mt][3] = lds_u32(&As[r + 8][kk + 8 + 2 * tq]);
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int c = wn + nt * 8 + gq;
                b[nt][0] = lds_u32(&Bs[c][kk + 2 * tq]);
                b[nt][1] = lds_u32(&Bs[c][kk + 8 + 2 * tq]);
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) mma_bf16_16816(acc[mt][nt], a[mt], b[nt]);
        }
        __syncthreads();
    }
    const bool partial = gridDim.z > 1;
    float *out = partial ? g.C + (size_t)blockIdx.z * g.M * g.N : g.C;
    const int ld = partial ? g.N : g.ldc;
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = m0 + wm + mt * 16 + gq + 8 * h;
                if (r >= g.M) continue;
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    const int c = n0 + wn + nt * 8 + 2 * tq + j;
                    if (c >= g.N) continue;
                    float *dst = out + (size_t)r * ld + c;
                    const float v = acc[mt][nt][2 * h + j];
                    *dst = (!partial && g.accumulate) ? *dst + v : v;
                }
            }
}

// C (+)= sum of the split partials, in split order.
__global__ void gemm_reduce_kernel(const float *__restrict__ part, int splits, int M, int N, float *C, int ldc,
                                   int accumulate) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)M * N) return;
    const int r = (int)(i / N), c = (int)(i - (int64_t)r * N);
    float v = 0.0f;
    for (int z = 0; z < splits; ++z) v += part[(size_t)z * M * N + i];
    float *dst = C + (size_t)r * ldc + c;
    *dst = accumulate ? *dst + v : v;
}

// Adam (Kingma & Ba 2015): m = b1 m + (1 - b1) g, v = b2 v + (1 - b2) g^2,
// p -= lr m^ / (sqrt(v^) + eps) with the bias corrections of step t.
__global__ void adam_kernel(float *p, const float *__restrict__ grad, float *m, float *v, int64_t n, float lr,
                            float b1, float b2, float eps, float c1, float c2) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

thread_local std::string t_train_error;

int train_fail(int code, const std::string &msg) {
    t_train_error = msg;
    return code;
}

}  // namespace
}  // namespace mfem

using namespace mfem;

extern "C" {

int mfem_train_gemm(int32_t M, int32_t N, int32_t K, const float *d_A, int32_t lda, int32_t a_trans,
                    const float *d_B, int32_t ldb, int32_t b_trans, float *d_C, int32_t ldc, int32_t accumulate,
                    float *d_workspace, int64_t workspace_floats, mfem_stream stream) {
    if (M < 0 || N < 0 || K < 0) return train_fail(MFEM_BAD_ARG, "mfem_train_gemm: negative size");
    if (M == 0 || N == 0) return MFEM_OK;
    if (!d_A || !d_B || !d_C) return train_fail(MFEM_BAD_ARG, "mfem_train_gemm: NULL operand");
    if (lda < (a_trans ? M : K) || ldb < (b_trans ? K : N) || ldc < N)
        return train_fail(MFEM_BAD_ARG, "mfem_train_gemm: leading dimension too small");
    cudaStream_t s = (cudaStream_t)stream;
    const int gm = (M + kGm - 1) / kGm, gn = (N + kGn - 1) / kGn;
    // split K so that small outputs (dW) still fill the GPU; at most 256
    // splits, each a multiple of the K tile, partials in the workspace
    int splits = 1;
    if (K > 4 * kGk && gm * gn < 64) {
        splits = std::min<int64_t>(256, std::max<int64_t>(1, (int64_t)K / 512));
        const int64_t cap = d_workspace ? workspace_floats / ((int64_t)M * N) : 0;
        splits = (int)std::max<int64_t>(1, std::min<int64_t>(splits, cap));
    }
    int k_chunk = (K + splits - 1) / splits;
    k_chunk = std::max(kGk, (k_chunk + kGk - 1) / kGk * kGk);
    splits = std::max(1, (K + k_chunk - 1) / k_chunk);
    GemmArgs g{M, N, K, d_A, lda, d_B, ldb, splits > 1 ? d_workspace : d_C, ldc, accumulate, k_chunk};
    const dim3 grid(gm, gn, splits);
    if (K == 0) {
        // an empty sum: C = 0 (or unchanged)
        if (!accumulate) {
            for (int r = 0; r < M; ++r) {
                cudaError_t e = cudaMemsetAsync(d_C + (size_t)r * ldc, 0, (size_t)N * sizeof(float), s);
                if (e != cudaSuccess) return train_fail(MFEM_CUDA_ERROR, cudaGetErrorString(e));
            }
        }
        return MFEM_OK;
    }
    if (a_trans && b_trans) gemm_bf16_kernel<true, true><<<grid, kGThreads, 0, s>>>(g);
    else if (a_trans) gemm_bf16_kernel<true, false><<<grid, kGThreads, 0, s>>>(g);
    else if (b_trans) gemm_bf16_kernel<false, true><<<grid, kGThreads, 0, s>>>(g);
    else gemm_bf16_kernel<false, false><<<grid, kGThreads, 0, s>>>(g);
    count_launches(1);
    if (splits > 1) {
        const int64_t total = (int64_t)M * N;
        gemm_reduce_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(d_workspace, splits, M, N, d_C, ldc,
                                                                          accumulate);
        count_launches(1);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MFEM_OK : train_fail(MFEM_CUDA_ERROR, cudaGetErrorString(e));
}

int mfem_train_adam(float *d_params, const float *d_grads, float *d_m, float *d_v, int64_t n, float lr, float beta1,
                    float beta2, float eps, int32_t step, mfem_stream stream) {
    if (n < 0 || step < 1 || (n > 0 && (!d_params || !d_grads || !d_m || !d_v)))
        return train_fail(MFEM_BAD_ARG, "mfem_train_adam: bad arguments");
    if (n == 0) return MFEM_OK;
    const float c1 = 1.0f - powf(beta1, (float)step);
    const float c2 = 1.0f - powf(beta2, (float)step);
    adam_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(d_params, d_grads, d_m, d_v, n, lr,
                                                                              beta1, beta2, eps, c1, c2);
    count_launches(1);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MFEM_OK : train_fail(MFEM_CUDA_ERROR, cudaGetErrorString(e));
}

const char *mfem_train_last_error(void) { return t_train_error.c_str(); }

}  // extern "C"
