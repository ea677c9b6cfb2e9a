// Factorized sparse approximate inverse (FSAI) of the global system, in
// 3x3 blocks: a lower block-triangular G on the lower block pattern of H
// such that M = G^T G approximates H^-1 (Kolotilina & Yeremin, "Factorized
// sparse approximate inverse preconditionings I", SIAM J. Matrix Anal. Appl.
// 14, 1993).
//
// Block row i of G is computed on its own.  With P the block columns j <= i
// of row i of H (i last) and H[P, P] = L L^T (lower Cholesky), the FSAI row
// is G[i, P] = D E^T H[P, P]^-1 for E the last three unit columns and any D
// with D X_ii D^T = I, X_ii = E^T H[P, P]^-1 E.  Since E^T L^-T lives only in
// the last block, X_ii = (L_ii L_ii^T)^-1 and D = L_ii^T gives
//     G[i, P] = E^T L^-1,
// the last block row of L^-1, found by one back substitution L^T X = E.
// Every diagonal block of G H G^T is the identity.  (Another D changes G by
// a 3x3 orthogonal factor per row and leaves M unchanged.)  A row with more
// than kFsaiMaxCols lower blocks, or whose local matrix is not numerically
// positive definite in fp32, falls back to G_ii = chol(H_ii)^-1.
//
// One warp per block row; the dense local matrix sits in shared memory.
// Not a reference function: the reference's PCG is block-Jacobi.
#include <algorithm>

#include "internal.h"

namespace mfem {
namespace {

constexpr int kFsaiWarps = 4;
constexpr int kFsaiThreads = 32 * kFsaiWarps;

__device__ int find_slot(const int *row_ptr, const int *col_idx, int row, int col) {
    int lo = row_ptr[row], hi = row_ptr[row + 1] - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int c = col_idx[mid];
        if (c == col) return mid;
        if (c < col) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// 3x3 lower Cholesky factor of a symmetric 3x3 (row-major a); false if not
// positive definite.
__device__ __forceinline__ bool chol3(const float a[9], float l[9]) {
    for (int i = 0; i < 9; ++i) l[i] = 0.0f;
    const float d0 = a[0];
    if (!(d0 > 0.0f)) return false;
    l[0] = sqrtf(d0);
    l[3] = a[3] / l[0];
    l[6] = a[6] / l[0];
    const float d1 = a[4] - l[3] * l[3];
    if (!(d1 > 0.0f)) return false;
    l[4] = sqrtf(d1);
    l[7] = (a[7] - l[6] * l[3]) / l[4];
    const float d2 = a[8] - l[6] * l[6] - l[7] * l[7];
    if (!(d2 > 0.0f)) return false;
    l[8] = sqrtf(d2);
    return true;
}

// inverse of a 3x3 lower-triangular matrix
__device__ __forceinline__ void inv_lower3(const float l[9], float m[9]) {
    for (int i = 0; i < 9; ++i) m[i] = 0.0f;
    m[0] = 1.0f / l[0];
    m[4] = 1.0f / l[4];
    m[8] = 1.0f / l[8];
    m[3] = -l[3] * m[0] * m[4];
    m[7] = -l[7] * m[4] * m[8];
    m[6] = -(l[6] * m[0] + l[7] * m[3]) * m[8];
}

// Rows with at most kFsaiSmallCols lower blocks (every vertex of a Kuhn tet
// grid): one thread per row.  The local matrix, padded to kFsaiSmall with an
// identity block at its top left (which leaves the last block row of L^-1
// unchanged), is factored in place as a packed lower triangle in shared
// memory (row stride odd, so the threads of a warp hit distinct banks);
// every loop is unrolled, so addresses are constant offsets and row j of L
// sits in registers while column j is formed.  The last block row of L^-1
// comes from w L = E^T, solved column by column from the last.
constexpr int kFsaiSmallCols = 8;
constexpr int kFsaiSmall = 3 * kFsaiSmallCols;
constexpr int kFsaiPacked = kFsaiSmall * (kFsaiSmall + 1) / 2;
constexpr int kFsaiThreadStride = kFsaiPacked + 1;
constexpr int kFsaiRowThreads = 32;

__device__ __forceinline__ constexpr int pk(int r, int c) { return r * (r + 1) / 2 + c; }

__global__ void __launch_bounds__(kFsaiRowThreads) fsai_setup_small_kernel(BsrViews bv, BatchViews bw) {
    extern __shared__ float s_mat[];
    const int row = blockIdx.x * kFsaiRowThreads + threadIdx.x;
    if (row >= bv.n) return;
    const int lb = bw.lrow[row], m = bw.lrow[row + 1] - lb;
    if (m < 1 || m > kFsaiSmallCols) return;  // the shared-memory warp kernel's rows
    float *L = s_mat + threadIdx.x * kFsaiThreadStride;
    float *G = bw.Lval + (size_t)9 * lb;
    const int pad = kFsaiSmall - 3 * m;
    const int *pslot = bw.fsai_pairs + bw.fsai_pair_ptr[row];
#pragma unroll
    for (int r = 0; r < kFsaiSmall; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c) {
            float v;
            if (r < pad) {
                v = r == c ? 1.0f : 0.0f;
            } else if (c < pad) {
                v = 0.0f;
            } else {
                const int rr = r - pad, cc = c - pad, a = rr / 3, b = cc / 3;
                const int sl = pslot[a * (a + 1) / 2 + b];
                v = sl >= 0 ? bv.values[(size_t)9 * sl + 3 * (rr - 3 * a) + (cc - 3 * b)] : 0.0f;
            }
            L[pk(r, c)] = v;
        }
    bool ok = true;
#pragma unroll
    for (int j = 0; j < kFsaiSmall; ++j) {
        float lj[kFsaiSmall];
        float d = L[pk(j, j)];
#pragma unroll
        for (int k = 0; k < j; ++k) {
            lj[k] = L[pk(j, k)];
            d = fmaf(-lj[k], lj[k], d);
        }
        if (!(d > 0.0f) || !isfinite(d)) {
            ok = false;
            d = 1.0f;
        }
        const float ljj = sqrtf(d), inv = 1.0f / ljj;
        L[pk(j, j)] = ljj;
#pragma unroll
        for (int r = j + 1; r < kFsaiSmall; ++r) {
            float a0 = L[pk(r, j)], a1 = 0.0f;
#pragma unroll
            for (int k = 0; k + 1 < j; k += 2) {
                a0 = fmaf(-L[pk(r, k)], lj[k], a0);
                a1 = fmaf(-L[pk(r, k + 1)], lj[k + 1], a1);
            }
            if (j & 1) a0 = fmaf(-L[pk(r, j - 1)], lj[j - 1], a0);
            L[pk(r, j)] = (a0 + a1) * inv;
        }
    }
    if (ok) {
        // w L = E^T: w[t][c] = (E[t][c] - sum_{r > c} w[t][r] L[r][c]) / L[c][c]
        float w0[kFsaiSmall], w1[kFsaiSmall], w2[kFsaiSmall];
#pragma unroll
        for (int c = kFsaiSmall - 1; c >= 0; --c) {
            float a0 = c == kFsaiSmall - 3 ? 1.0f : 0.0f;
            float a1 = c == kFsaiSmall - 2 ? 1.0f : 0.0f;
            float a2 = c == kFsaiSmall - 1 ? 1.0f : 0.0f;
#pragma unroll
            for (int r = c + 1; r < kFsaiSmall; ++r) {
                const float l = L[pk(r, c)];
                a0 = fmaf(-w0[r], l, a0);
                a1 = fmaf(-w1[r], l, a1);
                a2 = fmaf(-w2[r], l, a2);
            }
            const float inv = 1.0f / L[pk(c, c)];
            w0[c] = a0 * inv;
            w1[c] = a1 * inv;
            w2[c] = a2 * inv;
        }
        // G[i, P] = w restricted to the real columns: block a, entry (p, q)
        // = w[p][pad + 3a + q]
#pragma unroll
        for (int c = 0; c < kFsaiSmall; ++c)
            if (c >= pad) {
                const int cc = c - pad, a = cc / 3, q = cc - 3 * a;
                float *g = G + 9 * a + q;
                g[0] = w0[c];
                g[3] = w1[c];
                g[6] = w2[c];
            }
        return;
    }
    // fallback: G_ii = chol(H_ii)^-1, the other blocks zero
    for (int t = 0; t < 9 * m; ++t) G[t] = 0.0f;
    const int sl = find_slot(bv.row_ptr, bv.col_idx, row, row);
    float h[9], l[9], li[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) h[q] = bv.values[(size_t)9 * sl + q];
    float *gd = G + 9 * (m - 1);
    if (chol3(h, l)) {
        inv_lower3(l, li);
#pragma unroll
        for (int q = 0; q < 9; ++q) gd[q] = li[q];
    } else {
#pragma unroll
        for (int q = 0; q < 9; ++q) gd[q] = (q % 4 == 0) ? 1.0f : 0.0f;
    }
}

// Rows with more lower blocks (kFsaiSmallCols < m <= kFsaiMaxCols, and the
// fallback of longer ones), one warp per listed row, the local matrix in
// shared memory.
__global__ void __launch_bounds__(kFsaiThreads) fsai_setup_kernel(BsrViews bv, BatchViews bw) {
    __shared__ float s_A[kFsaiWarps][kFsaiDim * (kFsaiDim + 1)];
    __shared__ float s_X[kFsaiWarps][kFsaiDim * 3];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int t_row = blockIdx.x * kFsaiWarps + wid;
    if (t_row >= bw.n_fsai_big) return;  // uniform per warp
    const int row = bw.fsai_big_rows[t_row];
    float *A = s_A[wid];
    float *X = s_X[wid];
    const int lb = bw.lrow[row], m = bw.lrow[row + 1] - lb;
    float *G = bw.Lval + (size_t)9 * lb;
    const int N = 3 * m;
    const int S = N | 1;  // odd row stride: the rows lanes own fall in distinct banks
    bool ok = m >= 1 && m <= kFsaiMaxCols;
    if (ok) {
        // A = H[P, P], lower block triangle; pair (a, b), b <= a, is entry
        // a (a + 1) / 2 + b of the row's precomputed slot list
        const int *pslot = bw.fsai_pairs + bw.fsai_pair_ptr[row];
        for (int t = lane; t < m * (m + 1) / 2; t += 32) {
            int a = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
            while (a * (a + 1) / 2 > t) --a;
            while ((a + 1) * (a + 2) / 2 <= t) ++a;
            const int b = t - a * (a + 1) / 2;
            const int s = pslot[t];
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    A[(3 * a + p) * S + 3 * b + q] = s >= 0 ? bv.values[(size_t)9 * s + 3 * p + q] : 0.0f;
        }
        __syncwarp();
        // in-place Cholesky A = L L^T, left-looking (Crout): for column j
        // the lane of row r >= j forms A[r][j] - sum_k<j L[r][k] L[j][k];
        // row j's value is the pivot
        bool pos = true;
        for (int j = 0; j < N; ++j) {
            const float *lj = A + j * S;
            float v0 = 0.0f, v1 = 0.0f;
            const int r0 = j + lane, r1 = j + 32 + lane;
            if (r0 < N) {
                const float *lr = A + r0 * S;
                float acc = lr[j], acc2 = 0.0f;
                int k = 0;
                for (; k + 2 <= j; k += 2) {
                    acc = fmaf(-lr[k], lj[k], acc);
                    acc2 = fmaf(-lr[k + 1], lj[k + 1], acc2);
                }
                if (k < j) acc = fmaf(-lr[k], lj[k], acc);
                v0 = acc + acc2;
            }
            if (r1 < N) {
                const float *lr = A + r1 * S;
                float acc = lr[j], acc2 = 0.0f;
                int k = 0;
                for (; k + 2 <= j; k += 2) {
                    acc = fmaf(-lr[k], lj[k], acc);
                    acc2 = fmaf(-lr[k + 1], lj[k + 1], acc2);
                }
                if (k < j) acc = fmaf(-lr[k], lj[k], acc);
                v1 = acc + acc2;
            }
            float d = __shfl_sync(0xffffffffu, v0, 0);
            if (!(d > 0.0f) || !isfinite(d)) {
                pos = false;
                d = 1.0f;
            }
            const float ljj = sqrtf(d);
            __syncwarp();  // every lane has read row j before it changes
            if (r0 < N) A[r0 * S + j] = r0 == j ? ljj : v0 / ljj;
            if (r1 < N) A[r1 * S + j] = v1 / ljj;
            __syncwarp();
        }
        ok = pos;
    }
    if (ok) {
        // L^T X = E by back substitution, column-oriented: once row r of X is
        // final, remove its contribution from the rows above it
        for (int t = lane; t < 3 * N; t += 32) X[t] = (t / 3 == N - 3 + t % 3) ? 1.0f : 0.0f;
        __syncwarp();
        for (int r = N - 1; r >= 0; --r) {
            if (lane < 3) X[3 * r + lane] /= A[r * S + r];
            __syncwarp();
            for (int t = lane; t < 3 * r; t += 32) X[t] -= A[r * S + t / 3] * X[3 * r + t % 3];
            __syncwarp();
        }
        // G[i, P] = X^T: block a, entry (p, q) = X[3a + q][p]
        for (int t = lane; t < 9 * m; t += 32) {
            const int a = t / 9, e = t - 9 * a;
            G[t] = X[3 * (3 * a + e % 3) + e / 3];
        }
        return;
    }
    // fallback: G_ii = chol(H_ii)^-1, the other blocks zero
    for (int t = lane; t < 9 * m; t += 32) G[t] = 0.0f;
    __syncwarp();
    if (lane == 0 && m >= 1) {
        const int s = find_slot(bv.row_ptr, bv.col_idx, row, row);
        float h[9], l[9], li[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) h[q] = bv.values[(size_t)9 * s + q];
        float *gd = G + 9 * (m - 1);
        if (chol3(h, l)) {
            inv_lower3(l, li);
#pragma unroll
            for (int q = 0; q < 9; ++q) gd[q] = li[q];
        } else {
#pragma unroll
            for (int q = 0; q < 9; ++q) gd[q] = (q % 4 == 0) ? 1.0f : 0.0f;
        }
    }
}

// F^T in upper-CSR order, Uval[u] = Lval[umap[u]]^T, and the BF16 copies
// of both forms
__global__ void factor_transpose_kernel(BatchViews bw) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= bw.nnzl) return;
    const float *src = bw.Lval + (size_t)9 * bw.umap[u];
    const float *own = bw.Lval + (size_t)9 * u;
    float *dst = bw.Uval + (size_t)9 * u;
    __nv_bfloat16 *ub = bw.Ub + (size_t)kFactorLd * u;
    __nv_bfloat16 *lb = bw.Lb + (size_t)kFactorLd * u;
    float v[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) v[q] = src[q];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            dst[3 * p + q] = v[3 * q + p];
            ub[3 * p + q] = __float2bfloat16_rn(v[3 * q + p]);
        }
#pragma unroll
    for (int q = 0; q < 9; ++q) lb[q] = __float2bfloat16_rn(own[q]);
    ub[9] = lb[9] = __float2bfloat16_rn(0.0f);
}

}  // namespace

cudaError_t launch_fsai_setup(const BsrViews &bv, const BatchViews &bw, cudaStream_t s) {
    if (bv.n == 0) return cudaSuccess;
    const size_t smem = (size_t)kFsaiRowThreads * kFsaiThreadStride * sizeof(float);
    fsai_setup_small_kernel<<<(bv.n + kFsaiRowThreads - 1) / kFsaiRowThreads, kFsaiRowThreads, smem, s>>>(bv, bw);
    count_launches(1);
    if (bw.n_fsai_big > 0) {
        fsai_setup_kernel<<<(bw.n_fsai_big + kFsaiWarps - 1) / kFsaiWarps, kFsaiThreads, 0, s>>>(bv, bw);
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_factor_transpose(const BatchViews &bw, cudaStream_t s) {
    if (bw.nnzl == 0) return cudaSuccess;
    factor_transpose_kernel<<<(bw.nnzl + 255) / 256, 256, 0, s>>>(bw);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace mfem
