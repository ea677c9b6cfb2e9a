// The persistent PCG with a factor preconditioner: M = F^T F (FSAI,
// use_precond 2) or M = F F^T (the learned factor, use_precond 3), F on H's
// lower block pattern.  One cooperative launch per solve, one CTA per SM.
//
// It is the standard two-barrier iteration of the persistent PCG (pcg.cu),
// with z = M r formed without a third and fourth grid barrier:
//
//   A: p = z + beta p over the CTA's column window, Ap = H p for its rows,
//      publish Ap, (p, Ap)                                  -> grid barrier
//   B: stage the published Ap over the row range R, r -= alpha Ap over R,
//      y = F0 r over the row range Y, z = F1 y for its rows, publish z,
//      (r, z), (r, r)                                       -> grid barrier
//
// F0 is the first pass's form (F for mode 2, F^T for mode 3) and F1 the
// second's.  Y holds the columns F1 reaches from the CTA's rows, R the
// columns F0 reaches from Y: two hops of H's pattern, about one column window
// on either side.  Each CTA keeps r over R in shared memory for the whole
// solve and updates it with the same instructions, from the same published
// Ap and the same alpha, as the rows' owners, so every copy of a row's r
// equals the owner's bit for bit; y over Y is recomputed by each CTA instead
// of exchanged.  The factor does not change during a solve: where shared
// memory allows, each CTA copies its rows of both forms (row pointers,
// columns, BF16 blocks) there once per launch, else only their row pointers,
// and reads the rest through the read-only path (L2).
//
// A factor solve that breaks down (non-finite values or p.Ap <= 0) is solved
// again from the same warm start with block-Jacobi inside the launch; every
// CTA takes that decision from the same totals.  Every wait is bounded.
//
// With `fused` it runs the whole mixed-precision refinement in one launch
// (the residual passes in double-float, the decisions, the inner solves;
// see the fused block of the kernel).  Without, it also serves as one inner
// solve of the refinement's launch sequence
// (pcg_mixed.cu): from e = 0 it solves Hq e = r / ||r||, reading the 16-bit
// blocks (20 bytes a block, widened and scaled by their row's scale as they
// are loaded) or H once the refinement has switched to it, reads
// and writes the refinement's state words, and returns e ||r||.  A
// block-Jacobi plan keeps a layout of this kernel, without factor rows, for
// that use only.
#include <algorithm>

#include "factor_apply.cuh"
#include "pcg_common.cuh"

namespace mfem {
namespace {

// Orders this thread's earlier generic-proxy accesses to shared memory
// before later bulk copies (async proxy) into the same bytes.
__device__ __forceinline__ void proxy_fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// How much of its factor rows a CTA keeps in shared memory: nothing, the row
// pointers (absolute block indices), or row pointers, columns and blocks.
constexpr int kFactorNone = 0, kFactorRows = 1, kFactorAll = 2;

// A 3x3 block from its five words of BF16 pairs (the tenth value is padding):
// from the shared-memory copy, or through L2 in three loads.
template <bool SHARED>
__device__ __forceinline__ void block_words(const uint32_t *words, long long k, float f[9]) {
    uint32_t u[5];
    if (SHARED) {
#pragma unroll
        for (int i = 0; i < 5; ++i) u[i] = words[5 * k + i];
    } else {
        load_bf16_words(words, k, u);
    }
    bf16_words_to_block(u, f);
}

// The factor rows a CTA applies (FC: kFactorNone, kFactorRows or
// kFactorAll in shared memory).  With kFactorAll the columns are relative to
// the input vector's first row and the row pointers to the first block.
struct FactorRows {
    const int *rp, *col;
    const uint32_t *words;  // kFactorLd BF16 values (five words) per block
    int row0;               // first row (global row pointers) or 0 (shared)
    int in_lo;              // subtracted from the columns (0 for kFactorAll)
};

// One row of a factor form times a shared-memory vector `in`, kGroup lanes a
// row, two blocks a lane and trip; the row's sum in every lane of the group.
template <int FC>
__device__ __forceinline__ void factor_row(const FactorRows &f, const float *in, int j, int g_lane, unsigned gmask,
                                           float (&y)[3]) {
    constexpr bool SH = FC == kFactorAll;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
    const int row = f.row0 + j;
    const int kb = FC != kFactorNone ? f.rp[row] : __ldg(f.rp + row);
    const int ke = FC != kFactorNone ? f.rp[row + 1] : __ldg(f.rp + row + 1);
    for (int k = kb + g_lane; k < ke; k += 2 * kGroup) {
        const int k2 = k + kGroup;
        const bool two = k2 < ke;
        const int kk2 = two ? k2 : k;
        const int c = (SH ? f.col[k] : __ldg(f.col + k)) - f.in_lo;
        const int c2 = (SH ? f.col[kk2] : __ldg(f.col + kk2)) - f.in_lo;
        const float v0 = in[3 * c], v1 = in[3 * c + 1], v2 = in[3 * c + 2];
        float w0 = in[3 * c2], w1 = in[3 * c2 + 1], w2 = in[3 * c2 + 2];
        if (!two) w0 = w1 = w2 = 0.0f;
        float m[9], m2[9];
        block_words<SH>(f.words, k, m);
        block_words<SH>(f.words, kk2, m2);
        a0 += m[0] * v0 + m[1] * v1 + m[2] * v2;
        a1 += m[3] * v0 + m[4] * v1 + m[5] * v2;
        a2 += m[6] * v0 + m[7] * v1 + m[8] * v2;
        a0 += m2[0] * w0 + m2[1] * w1 + m2[2] * w2;
        a1 += m2[3] * w0 + m2[4] * w1 + m2[5] * w2;
        a2 += m2[6] * w0 + m2[7] * w1 + m2[8] * w2;
    }
#pragma unroll
    for (int off = kGroup / 2; off > 0; off >>= 1) {
        a0 += __shfl_xor_sync(gmask, a0, off);
        a1 += __shfl_xor_sync(gmask, a1, off);
        a2 += __shfl_xor_sync(gmask, a2, off);
    }
    y[0] = a0;
    y[1] = a1;
    y[2] = a2;
}

// Rows ja and jb (if has_b) of a factor form times a shared-memory vector
// `in`, kGroup lanes a row pair: per lane and trip two blocks of each row,
// the four blocks' loads in flight at once; the rows' sums in every lane of
// the group.  For factor rows read through L2 (half the dependent-load
// trips); with the rows in shared memory the single-row form issues fewer
// instructions and runs faster.
template <int FC>
__device__ __forceinline__ void factor_row_pair(const FactorRows &f, const float *in, int ja, int jb, bool has_b,
                                                int g_lane, unsigned gmask, float (&ya)[3], float (&yb)[3]) {
    constexpr bool SH = FC == kFactorAll;
    const int ra = f.row0 + ja, rb = f.row0 + (has_b ? jb : ja);
    const int kba = FC != kFactorNone ? f.rp[ra] : __ldg(f.rp + ra);
    const int kea = FC != kFactorNone ? f.rp[ra + 1] : __ldg(f.rp + ra + 1);
    int kbb = FC != kFactorNone ? f.rp[rb] : __ldg(f.rp + rb);
    int keb = FC != kFactorNone ? f.rp[rb + 1] : __ldg(f.rp + rb + 1);
    if (!has_b) keb = kbb;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, b0 = 0.0f, b1 = 0.0f, b2 = 0.0f;
    for (int t = g_lane; kba + t < kea || kbb + t < keb; t += 2 * kGroup) {
        const int k[4] = {kba + t, kba + t + kGroup, kbb + t, kbb + t + kGroup};
        const bool ok[4] = {k[0] < kea, k[1] < kea, k[2] < keb, k[3] < keb};
        int c[4];
        float m[4][9];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int kk = ok[u] ? k[u] : kba;  // every row holds its diagonal block
            c[u] = (SH ? f.col[kk] : __ldg(f.col + kk)) - f.in_lo;
            block_words<SH>(f.words, kk, m[u]);
        }
        float v[4][3];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int q = 0; q < 3; ++q) v[u][q] = ok[u] ? in[3 * c[u] + q] : 0.0f;
        a0 += m[0][0] * v[0][0] + m[0][1] * v[0][1] + m[0][2] * v[0][2];
        a1 += m[0][3] * v[0][0] + m[0][4] * v[0][1] + m[0][5] * v[0][2];
        a2 += m[0][6] * v[0][0] + m[0][7] * v[0][1] + m[0][8] * v[0][2];
        a0 += m[1][0] * v[1][0] + m[1][1] * v[1][1] + m[1][2] * v[1][2];
        a1 += m[1][3] * v[1][0] + m[1][4] * v[1][1] + m[1][5] * v[1][2];
        a2 += m[1][6] * v[1][0] + m[1][7] * v[1][1] + m[1][8] * v[1][2];
        b0 += m[2][0] * v[2][0] + m[2][1] * v[2][1] + m[2][2] * v[2][2];
        b1 += m[2][3] * v[2][0] + m[2][4] * v[2][1] + m[2][5] * v[2][2];
        b2 += m[2][6] * v[2][0] + m[2][7] * v[2][1] + m[2][8] * v[2][2];
        b0 += m[3][0] * v[3][0] + m[3][1] * v[3][1] + m[3][2] * v[3][2];
        b1 += m[3][3] * v[3][0] + m[3][4] * v[3][1] + m[3][5] * v[3][2];
        b2 += m[3][6] * v[3][0] + m[3][7] * v[3][1] + m[3][8] * v[3][2];
    }
#pragma unroll
    for (int off = kGroup / 2; off > 0; off >>= 1) {
        a0 += __shfl_xor_sync(gmask, a0, off);
        a1 += __shfl_xor_sync(gmask, a1, off);
        a2 += __shfl_xor_sync(gmask, a2, off);
        b0 += __shfl_xor_sync(gmask, b0, off);
        b1 += __shfl_xor_sync(gmask, b1, off);
        b2 += __shfl_xor_sync(gmask, b2, off);
    }
    ya[0] = a0;
    ya[1] = a1;
    ya[2] = a2;
    yb[0] = b0;
    yb[1] = b1;
    yb[2] = b2;
}

// y[j] = (F0 r)_(y_lo + j) for j < ny, r over R in shared memory.
template <int FC>
__device__ __forceinline__ void first_pass(const FactorRows &f0, const float *sR, float *sY, int ny) {
    const int g_lane = threadIdx.x & (kGroup - 1);
    const unsigned gmask = ((1u << kGroup) - 1u) << (threadIdx.x & (32 - kGroup));
    const int group = threadIdx.x / kGroup, ngroups = blockDim.x / kGroup;
    if constexpr (FC == kFactorAll) {
        for (int j = group; j < ny; j += ngroups) {
            float y[3];
            factor_row<FC>(f0, sR, j, g_lane, gmask, y);
            if (g_lane == 0)
#pragma unroll
                for (int q = 0; q < 3; ++q) sY[3 * j + q] = y[q];
        }
    } else {
        for (int j = group; j < ny; j += 2 * ngroups) {  // rows j and j + ngroups together
            const int jb = j + ngroups;
            const bool has_b = jb < ny;
            float ya[3], yb[3];
            factor_row_pair<FC>(f0, sR, j, jb, has_b, g_lane, gmask, ya, yb);
            if (g_lane == 0) {
#pragma unroll
                for (int q = 0; q < 3; ++q) sY[3 * j + q] = ya[q];
                if (has_b)
#pragma unroll
                    for (int q = 0; q < 3; ++q) sY[3 * jb + q] = yb[q];
            }
        }
    }
}

// Row i's z: published, and (r, z), (r, r) added to acc.
__device__ __forceinline__ void emit_z(const float z[3], const float *sRown, int i, int row_lo, float *pubZ,
                                       float (&acc)[2]) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float r = sRown[3 * i + c];
        pubZ[(size_t)3 * (row_lo + i) + c] = z[c];
        acc[0] = __fmaf_rn(r, z[c], acc[0]);
        acc[1] = __fmaf_rn(r, r, acc[1]);
    }
}

// z = F1 y for the CTA's rows: published, and (r, z), (r, r) added to acc.
template <int FC>
__device__ __forceinline__ void second_pass(const FactorRows &f1, const float *sY, const float *sRown, int row_lo,
                                            int nrows, float *pubZ, float (&acc)[2]) {
    const int g_lane = threadIdx.x & (kGroup - 1);
    const unsigned gmask = ((1u << kGroup) - 1u) << (threadIdx.x & (32 - kGroup));
    const int group = threadIdx.x / kGroup, ngroups = blockDim.x / kGroup;
    if constexpr (FC == kFactorAll) {
        for (int i = group; i < nrows; i += ngroups) {
            float z[3];
            factor_row<FC>(f1, sY, i, g_lane, gmask, z);
            if (g_lane == 0) emit_z(z, sRown, i, row_lo, pubZ, acc);
        }
    } else {
        for (int i = group; i < nrows; i += 2 * ngroups) {  // rows i and i + ngroups together
            const int ib = i + ngroups;
            const bool has_b = ib < nrows;
            float za[3], zb[3];
            factor_row_pair<FC>(f1, sY, i, ib, has_b, g_lane, gmask, za, zb);
            if (g_lane == 0) {
                emit_z(za, sRown, i, row_lo, pubZ, acc);
                if (has_b) emit_z(zb, sRown, ib, row_lo, pubZ, acc);
            }
        }
    }
}

// Copies rows [r0, r0 + nrows) of a global factor form into shared memory:
// row offsets, columns minus col_lo, and the blocks' words.
__device__ __forceinline__ void stage_factor_rows(const int *rp, const int *col, const __nv_bfloat16 *val, int r0,
                                                  int nrows, int col_lo, int *s_rp, int *s_col, uint32_t *s_words) {
    const int kb = rp[r0], nb = rp[r0 + nrows] - kb;
    for (int j = threadIdx.x; j <= nrows; j += blockDim.x) s_rp[j] = rp[r0 + j] - kb;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) s_col[k] = col[kb + k] - col_lo;
    const uint32_t *w = reinterpret_cast<const uint32_t *>(val + (size_t)kFactorLd * kb);
    for (int t = threadIdx.x; t < 5 * nb; t += blockDim.x) s_words[t] = w[t];
}

// r = g - H x for the CTA's rows, with x over the CTA's column window as hi
// and lo planes and the fp32 H read through L2, the products summed in
// double-float; r (as float) to `res`, (r.r, g.g) in double added to acc.
__device__ __forceinline__ void residual_rows(const PcgArgs &a, const Common &cm, const int *rowoff,
                                              const float *whi, const float *wlo, float *res, double (&acc)[2]) {
    const int g_lane = threadIdx.x & (kGroup - 1);
    const int group = threadIdx.x / kGroup, ngroups = blockDim.x / kGroup;
    const unsigned gmask = ((1u << kGroup) - 1u) << (threadIdx.x & (32 - kGroup));
    for (int i = group; i < cm.nrows; i += ngroups) {
        float2 sum[3] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
        for (int k = rowoff[i] + g_lane; k < rowoff[i + 1]; k += kGroup) {
            float h[9];
            load_block9(a.values, (long long)cm.blk_lo + k, h);
            const int c = __ldg(a.col_idx + cm.blk_lo + k) - cm.win_lo;
            float2 x[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) x[q] = make_float2(whi[3 * c + q], wlo[3 * c + q]);
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int q = 0; q < 3; ++q) df_fma(sum[r], h[3 * r + q], x[q]);
        }
#pragma unroll
        for (int off = kGroup / 2; off > 0; off >>= 1)
#pragma unroll
            for (int r = 0; r < 3; ++r) sum[r] = df_add(sum[r], df_shfl_xor(gmask, sum[r], off));
        if (g_lane == 0) {
            const int row = cm.row_lo + i;
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const float gq = a.g[3 * row + r];
                const double rv = df_residual(gq, sum[r]);
                res[3 * row + r] = (float)rv;
                acc[0] += rv * rv;
                acc[1] += (double)gq * (double)gq;
            }
        }
    }
}

template <bool CACHE, int FC>
__global__ void __launch_bounds__(kPcgThreads, 1) pcg_factor_kernel(PcgArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    // As the refinement's inner solve: nothing to do once it has finished or
    // when it restarts from the warm start (its state words, as every CTA
    // reads them: the previous launch wrote them)
    const bool inner = a.ir_state != nullptr;
    const bool fused = inner && a.fused != 0;  // the whole refinement in this launch
    if (inner) {
        if (!fused && (ld_volatile(a.ir_state) != 0 || ld_volatile(a.ir_state + 7) != 0)) return;
        if (ld_volatile(a.error) != 0) {
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                a.ir_state[5] = MFEM_TIMEOUT;
                a.ir_state[0] = 1;
            }
            return;
        }
    }
    PCG_PROLOGUE
    __shared__ double s_redd[2][32];
    __shared__ double s_vald[2 * kMaxCtas];
    __shared__ double s_totd[2];
    __shared__ int s_dec[2];      // the fused refinement's decision: done, restart
    __shared__ float s_dscale[2];  // 1 / ||r|| and ||r||
    // the inner solve runs on the 16-bit blocks unless the refinement
    // switched to the fp32 H; its right-hand side is scaled to
    // unit norm and its solution scaled back
    bool full = !inner || ld_volatile(a.ir_state + 6) != 0;
    HBlocks hm = full ? HBlocks{a.values, nullptr, nullptr, 0}
                      : HBlocks{a.values, a.values_w, a.row_scale, a.lowp_kind};
    float bscale = inner && !fused ? a.ir_scale[0] : 1.0f;
    const int rows_max = a.rows_max, win_max = a.win_max;
    float *sX = reinterpret_cast<float *>(smem);
    float *sAp = sX + 3 * rows_max;
    float *winA = sAp + 3 * rows_max;
    float *winB = winA + 3 * win_max;  // the p window in A, Ap over R in B
    float *sR = winB + 3 * max(win_max, a.r_max);
    float *sY = sR + 3 * a.r_max;
    int *rowoff = reinterpret_cast<int *>(sY + 3 * a.y_max);
    float *sH = reinterpret_cast<float *>(rowoff + rows_max + 4);
    int *sCol = reinterpret_cast<int *>(sH + (CACHE ? 9 * a.blk_max : 0));
    int *f_rp0 = sCol + (CACHE ? a.blk_max : 0);  // the CTA's factor rows (FC)
    int *f_rp1 = f_rp0 + a.y_max + 4;
    int *f_c0 = f_rp1 + rows_max + 4;
    int *f_c1 = f_c0 + a.f0_max;
    uint32_t *f_w0 = reinterpret_cast<uint32_t *>(f_c1 + a.f1_max);
    uint32_t *f_w1 = f_w0 + 5 * a.f0_max;

    const int4 fi = a.fcta[blockIdx.x];
    const int y_lo = fi.x, y_hi = fi.y, r_lo = fi.z, nr = fi.w - fi.z;
    const size_t vec = (size_t)3 * a.n_pad;
    float *pubZ = a.pub;
    float *pubP[2] = {a.pub + vec, a.pub + 2 * vec};
    float *pubR = a.pub + 3 * vec;
    float *pubAp = a.pub + 4 * vec;
    const int own = cm.row_lo - cm.win_lo;  // the CTA's rows in the window
    float *sRown = sR + 3 * (cm.row_lo - r_lo);  // the CTA's rows in R
    const uint32_t wbytes = (uint32_t)cm.nwin * 12u, rbytes = (uint32_t)nr * 12u;

    load_matrix_slice(a, cm, rowoff, sH, sCol, CACHE, hm);
    FactorRows f0, f1;
    if (FC == kFactorAll) {
        stage_factor_rows(a.rp0, a.c0, a.v0, y_lo, y_hi - y_lo, r_lo, f_rp0, f_c0, f_w0);
        stage_factor_rows(a.rp1, a.c1, a.v1, cm.row_lo, cm.nrows, y_lo, f_rp1, f_c1, f_w1);
        f0 = FactorRows{f_rp0, f_c0, f_w0, 0, 0};
        f1 = FactorRows{f_rp1, f_c1, f_w1, 0, 0};
    } else if (FC == kFactorRows) {
        for (int j = threadIdx.x; j <= y_hi - y_lo; j += blockDim.x) f_rp0[j] = a.rp0[y_lo + j];
        for (int j = threadIdx.x; j <= cm.nrows; j += blockDim.x) f_rp1[j] = a.rp1[cm.row_lo + j];
        f0 = FactorRows{f_rp0, a.c0, reinterpret_cast<const uint32_t *>(a.v0), 0, r_lo};
        f1 = FactorRows{f_rp1, a.c1, reinterpret_cast<const uint32_t *>(a.v1), 0, y_lo};
    } else {
        f0 = FactorRows{a.rp0, a.c0, reinterpret_cast<const uint32_t *>(a.v0), y_lo, r_lo};
        f1 = FactorRows{a.rp1, a.c1, reinterpret_cast<const uint32_t *>(a.v1), cm.row_lo, y_lo};
    }
    int mode = a.use_precond;  // 2 or 3; 1 after a breakdown
    int it = 0, it_done = 0;
    bool pending = false;  // window copies in flight
    // One solve from x0 (the warm start, or 0 for an inner solve): sX holds
    // the solution and sc its outcome on return.
    auto solve = [&]() {
    mode = a.use_precond;
    it = 0;
    it_done = 0;
    pending = false;
    for (;;) {  // one attempt
        const bool factor = mode >= 2;
        it = 0;
        // ---- r = g - H x0 (x0: the warm start), z = M r
        proxy_fence_smem();
        __syncthreads();
        bool ok = true;
        if (!inner) {
            if (threadIdx.x == 0 && cm.nwin > 0) {
                tma_expect(&s_mbar, wbytes);
                tma_copy(winA, a.x + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
            }
            if (cm.nwin > 0) ok = tma_wait(&s_mbar, parity, a.error);
        }
        if (ok) {
            if (inner) {  // x0 = 0: r = b
                for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) sX[i] = sAp[i] = 0.0f;
            } else {
                for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) sX[i] = winA[3 * own + i];
                window_product<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.win_lo, cm.nrows, winA, sAp, hm, cm.row_lo);
            }
            __syncthreads();
            float acc[3] = {0.0f, 0.0f, 0.0f};
            for (int i = threadIdx.x; i < cm.nrows; i += blockDim.x) {
                const int row = cm.row_lo + i;
                float r[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const float bc = a.b[3 * row + c] * bscale;
                    r[c] = bc - sAp[3 * i + c];
                    acc[2] = __fmaf_rn(bc, bc, acc[2]);
                }
                if (factor) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) pubR[3 * row + c] = r[c];
                } else {
                    float z[3];
                    precond(a.Minv + (size_t)9 * row, r, z, 1);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        sRown[3 * i + c] = r[c];
                        pubZ[3 * row + c] = z[c];
                        acc[0] = __fmaf_rn(r[c], z[c], acc[0]);
                        acc[1] = __fmaf_rn(r[c], r[c], acc[1]);
                    }
                }
            }
            if (factor) {
                // every row's r is published; each CTA stages r over R
                float bb[1] = {acc[2]};
                ok = reduce_arrive<1>(bb, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok);
                if (ok) {
                    if (threadIdx.x == 0 && nr > 0) {
                        tma_expect(&s_mbar, rbytes);
                        tma_copy(sR, pubR + (size_t)3 * r_lo, rbytes, &s_mbar);
                    }
                    reduce_totals<1>(a.partials, bar, s_val, s_tot);
                    if (threadIdx.x == 0) sc.bb = s_tot[0];
                    if (nr > 0) ok = tma_wait(&s_mbar, parity, a.error);
                }
                ++bar;
                if (ok) {
                    first_pass<FC>(f0, sR, sY, y_hi - y_lo);
                    __syncthreads();
                    float rz[2] = {0.0f, 0.0f};
                    second_pass<FC>(f1, sY, sRown, cm.row_lo, cm.nrows, pubZ, rz);
                    proxy_fence_smem();
                    ok = reduce_arrive<2>(rz, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok);
                }
            } else {
                proxy_fence_smem();
                ok = reduce_arrive<3>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok);
            }
        }
        if (ok) {
            if (threadIdx.x == 0 && cm.nwin > 0) {
                tma_expect(&s_mbar, wbytes);
                tma_copy(winA, pubZ + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
            }
            if (factor) reduce_totals<2>(a.partials, bar, s_val, s_tot);
            else reduce_totals<3>(a.partials, bar, s_val, s_tot);
            if (threadIdx.x == 0) {
                if (!factor) sc.bb = s_tot[2];
                sc.gamma = s_tot[0];  // r.z
                sc.rr = s_tot[1];
                sc.thr2 = a.tol * a.tol * sc.bb;
                sc.beta = 0.0f;
                sc.status = (!isfinite(s_tot[0]) || !isfinite(s_tot[1]) || !isfinite(sc.bb)) ? MFEM_NONFINITE : MFEM_OK;
                sc.done = sc.status != MFEM_OK || s_tot[1] <= sc.thr2;
            }
            pending = cm.nwin > 0;
        } else if (threadIdx.x == 0) {
            sc.status = MFEM_TIMEOUT;
            sc.done = 1;
            sc.rr = 0.0f;
            sc.bb = 1.0f;
        }
        ++bar;
        __syncthreads();
        while (!sc.done) {
            if (it >= a.maxiter) {
                if (threadIdx.x == 0) sc.status = MFEM_MAXITER;
                break;
            }
            // ---- phase A: p = z + beta p over the window, Ap = H p, p.Ap
            float *p_new = pubP[it & 1];
            // each thread waits for the window copies itself; the verdicts
            // join the sync after the window update
            const bool landed = !pending || tma_wait_local(&s_mbar, parity);
            pending = false;
            const float fbeta = sc.beta;
            if (it > 0) {
                for (int j = threadIdx.x; j < 3 * cm.nwin; j += blockDim.x)
                    winA[j] = __fmaf_rn(fbeta, winB[j], winA[j]);
            }
            if (!__syncthreads_and(landed)) {
                if (threadIdx.x == 0) {
                    atomicExch(a.error, 1);
                    sc.status = MFEM_TIMEOUT;
                }
                break;
            }
            for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x)
                p_new[(size_t)3 * cm.row_lo + i] = winA[3 * own + i];
            window_product<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.win_lo, cm.nrows, winA, sAp, hm, cm.row_lo);
            __syncthreads();
            float pap[1] = {0.0f};
            for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) {
                pap[0] = __fmaf_rn(winA[3 * own + i], sAp[i], pap[0]);
                if (factor) pubAp[(size_t)3 * cm.row_lo + i] = sAp[i];
            }
            proxy_fence_smem();
            if (!reduce_arrive<1>(pap, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok)) {
                if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
                break;
            }
            // the copy from warp 1 while warp 0 fetches the totals
            const bool ap_pending = factor && nr > 0;
            if (ap_pending && threadIdx.x == 32) {
                tma_expect(&s_mbar, rbytes);
                tma_copy(winB, pubAp + (size_t)3 * r_lo, rbytes, &s_mbar);
            }
            reduce_totals_w0<1>(a.partials, bar, s_tot);
            ++bar;
            if (threadIdx.x == 0) {
                const float pAp = s_tot[0];
                if (!isfinite(pAp)) {
                    sc.status = MFEM_NONFINITE;
                    sc.done = 1;
                } else if (!(pAp > 0.0f)) {
                    sc.status = MFEM_STAGNATION;
                    sc.done = 1;
                } else {
                    sc.alpha = sc.gamma / pAp;
                }
            }
            __syncthreads();
            if (sc.done) {
                if (ap_pending) tma_wait(&s_mbar, parity, a.error);
                break;
            }
            const float alpha = sc.alpha;
            // the copy of Ap over R, waited for by each thread (joined below)
            const bool ap_landed = !ap_pending || tma_wait_local(&s_mbar, parity);
            // ---- phase B: r -= alpha Ap (over R with a factor), x += alpha p, z = M r
            if (factor) {
                for (int j = threadIdx.x; j < 3 * nr; j += blockDim.x) sR[j] = __fmaf_rn(-alpha, winB[j], sR[j]);
            } else {
                for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x)
                    sRown[i] = __fmaf_rn(-alpha, sAp[i], sRown[i]);
            }
            for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x)
                sX[i] = __fmaf_rn(alpha, winA[3 * own + i], sX[i]);
            if (!__syncthreads_and(ap_landed)) {
                if (threadIdx.x == 0) {
                    atomicExch(a.error, 1);
                    sc.status = MFEM_TIMEOUT;
                }
                break;
            }
            float acc[2] = {0.0f, 0.0f};
            if (factor) {
                first_pass<FC>(f0, sR, sY, y_hi - y_lo);
                __syncthreads();
                second_pass<FC>(f1, sY, sRown, cm.row_lo, cm.nrows, pubZ, acc);
            } else {
                for (int i = threadIdx.x; i < cm.nrows; i += blockDim.x) {
                    const int row = cm.row_lo + i;
                    float r[3], z[3];
#pragma unroll
                    for (int c = 0; c < 3; ++c) r[c] = sRown[3 * i + c];
                    precond(a.Minv + (size_t)9 * row, r, z, 1);
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        pubZ[3 * row + c] = z[c];
                        acc[0] = __fmaf_rn(r[c], z[c], acc[0]);
                        acc[1] = __fmaf_rn(r[c], r[c], acc[1]);
                    }
                }
            }
            proxy_fence_smem();
            if (!reduce_arrive<2>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok)) {
                if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
                break;
            }
            ++it;
            if (threadIdx.x == 32 && cm.nwin > 0) {
                tma_expect(&s_mbar, 2u * wbytes);
                tma_copy(winA, pubZ + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
                tma_copy(winB, p_new + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
            }
            pending = cm.nwin > 0;
            reduce_totals_w0<2>(a.partials, bar, s_tot);
            ++bar;
            if (threadIdx.x == 0) {
                sc.rr = s_tot[1];
                if (!isfinite(s_tot[0]) || !isfinite(s_tot[1])) {
                    sc.status = MFEM_NONFINITE;
                    sc.done = 1;
                } else {
                    sc.beta = s_tot[0] / sc.gamma;
                    sc.gamma = s_tot[0];
                    sc.done = s_tot[1] <= sc.thr2;
                }
            }
            __syncthreads();
        }
        if (pending) tma_wait(&s_mbar, parity, a.error);
        pending = false;
        __syncthreads();
        if (factor && (sc.status == MFEM_STAGNATION || sc.status == MFEM_NONFINITE)) {
            it_done += it;
            mode = 1;
            continue;
        }
        break;
    }
    __syncthreads();
    };
    if (fused) {
        // The refinement in one launch (the sequence of ir_residual_kernel
        // and inner launches, pcg_mixed.cu, without the launches): x starts
        // at the warm start; each pass publishes x, forms r = g - H x for the
        // CTA's rows in double-float, reduces ||r||, ||g|| in double, and
        // every CTA takes the same decision from the same totals: done, a
        // restart on the fp32 H (divergence on the 16-bit H), or an inner
        // solve of H e = r / ||r|| from 0 whose e ||r|| the next pass adds.
        const IrWork &w = a.irw;
        const int n3own = 3 * cm.nrows;
        const size_t off = (size_t)3 * cm.row_lo;
        float *xhi = w.xf_hi, *xlo = w.xf_lo;
        const uint32_t xbytes = (uint32_t)cm.nwin * 12u;
        // decision state, kept by thread 0 of every CTA
        double best = __longlong_as_double(0x7ff0000000000000ll);  // +inf
        int outer = 0, inner_its = 0, status = MFEM_OK, fp32_inner = full ? 1 : 0;
        bool restart = true, have_e = false;  // the first pass reads the warm start
        float es = 1.0f;
        for (;;) {
            if (restart || have_e) {
                for (int i = threadIdx.x; i < n3own; i += blockDim.x) {
                    if (restart) {
                        xhi[off + i] = w.dx_init[off + i];
                        xlo[off + i] = 0.0f;
                    } else {
                        const float2 x = df_add(make_float2(xhi[off + i], xlo[off + i]), __fmul_rn(sX[i], es));
                        xhi[off + i] = x.x;
                        xlo[off + i] = x.y;
                    }
                }
            }
            restart = false;
            have_e = false;
            // every row's x published: a barrier, then the CTA's window of it
            float none[1] = {0.0f};
            bool ok = reduce_arrive<1>(none, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok);
            ++bar;
            if (ok && cm.nwin > 0) {
                if (threadIdx.x == 0) {
                    tma_expect(&s_mbar, 2u * xbytes);
                    tma_copy(winA, xhi + (size_t)3 * cm.win_lo, xbytes, &s_mbar);
                    tma_copy(winB, xlo + (size_t)3 * cm.win_lo, xbytes, &s_mbar);
                }
                ok = tma_wait(&s_mbar, parity, a.error);
            }
            double acc[2] = {0.0, 0.0};
            if (ok) residual_rows(a, cm, rowoff, winA, winB, w.res, acc);
            ok = ok && reduce_arrive_d<2>(acc, w.partials, bar, a.counter, target, a.error, s_redd, &s_ok);
            if (ok) reduce_totals_d<2>(w.partials, bar, s_vald, s_totd);
            ++bar;
            if (threadIdx.x == 0) {
                int done = 0, rs = 0;
                double rel = 0.0;
                if (!ok) {
                    if (status == MFEM_OK) status = MFEM_TIMEOUT;
                    done = 1;
                } else {
                    const double rr = s_totd[0], gg = s_totd[1];
                    rel = gg > 0.0 ? sqrt(rr / gg) : sqrt(rr);
                    // the next inner right-hand side at unit norm: fp32 sums of
                    // products of a tiny residual's entries would underflow
                    const double rn = sqrt(rr);
                    const float inv = (float)(1.0 / rn);
                    const bool scaled = rn > 0.0 && isfinite(rn) && isfinite(inv);
                    s_dscale[0] = scaled ? inv : 1.0f;
                    s_dscale[1] = scaled ? (float)rn : 1.0f;
                    int st = MFEM_OK;
                    if (!fp32_inner && isfinite(best) && !(rel <= 4.0 * best) && outer < w.outer_max) {
                        fp32_inner = 1;  // diverging on the 16-bit H
                        rs = 1;
                    } else if (!isfinite(rel)) {
                        st = MFEM_NONFINITE;
                        done = 1;
                    } else if (rel <= w.outer_tol) {
                        done = 1;
                    } else if (outer >= w.outer_max) {
                        st = MFEM_MAXITER;
                        done = 1;
                    }
                    if (isfinite(rel) && rel < best && !rs) best = rel;
                    if (status == MFEM_OK) status = st;
                }
                if (blockIdx.x == 0) {
                    w.stats[a.slot] = IrStats{outer, inner_its, status, fp32_inner, rel};
                    a.stats[a.slot] = SolveStats{inner_its, status, (float)rel, 0.0f};
                }
                ++outer;
                s_dec[0] = done;
                s_dec[1] = rs;
            }
            __syncthreads();
            if (s_dec[0]) break;
            if (s_dec[1]) {  // restart from the warm start on the fp32 H
                full = true;
                hm = HBlocks{a.values, nullptr, nullptr, 0};
                if (CACHE) {
                    load_matrix_slice(a, cm, rowoff, sH, sCol, CACHE, hm);
                    __syncthreads();
                }
                restart = true;
                continue;
            }
            bscale = s_dscale[0];
            es = s_dscale[1];
            solve();
            if (threadIdx.x == 0) inner_its += it_done + it;
            if (sc.status == MFEM_NONFINITE && !full) {
                // the 16-bit H broke the inner solve: restart on the fp32 H
                if (threadIdx.x == 0) fp32_inner = 1;
                full = true;
                hm = HBlocks{a.values, nullptr, nullptr, 0};
                if (CACHE) {
                    load_matrix_slice(a, cm, rowoff, sH, sCol, CACHE, hm);
                    __syncthreads();
                }
                restart = true;
                continue;
            }
            if (sc.status == MFEM_TIMEOUT || sc.status == MFEM_NONFINITE) {
                if (threadIdx.x == 0) {
                    if (status == MFEM_OK) status = sc.status;
                    if (blockIdx.x == 0) {
                        w.stats[a.slot] = IrStats{outer, inner_its, status, fp32_inner, 0.0};
                        a.stats[a.slot] = SolveStats{inner_its, status, 0.0f, 0.0f};
                    }
                }
                break;
            }
            have_e = true;  // MAXITER and STAGNATION still hand over their iterate
        }
        // the solution: float for the local solve, double for the buffer
        for (int i = threadIdx.x; i < n3own; i += blockDim.x) {
            const float hi = xhi[off + i], lo = xlo[off + i];
            a.dx[off + i] = __fadd_rn(hi, lo);
            w.dx_out[off + i] = (double)hi + (double)lo;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) w.state[0] = 1;
        return;
    }
    solve();
    if (!inner) {
        finish(a, cm, sX, sc, it_done + it);
        return;
    }
    // the correction for the refinement, and its state: the outer loop adds
    // the correction at its next residual; a broken inner solve still hands
    // over its iterate, as the reference's CG does
    const float es = a.ir_scale[1];
    for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) a.x[(size_t)3 * cm.row_lo + i] = sX[i] * es;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ir_state[2] += it_done + it;
        a.ir_state[3] = 1;
        if (sc.status == MFEM_NONFINITE && !full) {
            // the 16-bit H broke the inner solve: restart on the fp32 H
            a.ir_state[3] = 0;
            a.ir_state[6] = 1;
            a.ir_state[7] = 1;
        } else if (sc.status == MFEM_TIMEOUT || sc.status == MFEM_NONFINITE) {
            a.ir_state[5] = sc.status;
            a.ir_state[0] = 1;
        }
    }
}

size_t smem_factor(const PcgLayout &L, bool cache, int fc) {
    const size_t floats = (size_t)L.rows_max * 6 + (size_t)L.win_max * 3 +
                          (size_t)std::max(L.win_max, L.r_max) * 3 + (size_t)L.r_max * 3 + (size_t)L.y_max * 3;
    size_t bytes = floats * 4 + (size_t)(L.rows_max + 4) * 4;
    if (cache) bytes += (size_t)L.blk_max * 40;
    if (fc != kFactorNone) bytes += (size_t)(L.y_max + 4 + L.rows_max + 4) * 4;
    if (fc == kFactorAll) bytes += (size_t)(L.f0_max + L.f1_max) * 24;
    return (bytes + 15) & ~(size_t)15;
}

typedef void (*FactorKernel)(PcgArgs);

FactorKernel pick_factor_kernel(const PcgLayout &L) {
    if (L.cache_matrix) {
        if (L.factor_cache == kFactorAll) return pcg_factor_kernel<true, kFactorAll>;
        if (L.factor_cache == kFactorRows) return pcg_factor_kernel<true, kFactorRows>;
        return pcg_factor_kernel<true, kFactorNone>;
    }
    if (L.factor_cache == kFactorAll) return pcg_factor_kernel<false, kFactorAll>;
    if (L.factor_cache == kFactorRows) return pcg_factor_kernel<false, kFactorRows>;
    return pcg_factor_kernel<false, kFactorNone>;
}

}  // namespace

cudaError_t pcg_factor_layout(int device, PcgLayout &L, const int32_t *row_ptr, const int32_t *col_idx, int n,
                              int ctas, int mode, std::vector<int4> &cta_info, std::vector<int4> &factor_info,
                              std::string &err, bool factor) {
    int optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e != cudaSuccess) return e;
    const size_t budget = (size_t)optin > kStaticSmem ? (size_t)optin - kStaticSmem : 0;
    if (ctas < 1 || ctas > kMaxCtas || (mode != 2 && mode != 3)) {
        err = "factor PCG layout: bad CTA count or mode";
        return cudaErrorInvalidValue;
    }
    // per row the smallest and largest column (the diagonal is in every row)
    std::vector<int> cmin(n), cmax(n);
    for (int j = 0; j < n; ++j) {
        int lo = j, hi = j;
        for (int64_t k = row_ptr[j]; k < row_ptr[j + 1]; ++k) {
            lo = std::min(lo, (int)col_idx[k]);
            hi = std::max(hi, (int)col_idx[k]);
        }
        cmin[j] = lo;
        cmax[j] = hi;
    }
    cta_info.assign(ctas, make_int4(0, 0, 0, 0));
    factor_info.assign(ctas, make_int4(0, 0, 0, 0));
    // blocks per row of the lower (columns <= row) and upper (>= row) forms
    std::vector<int64_t> lower_ptr(n + 1, 0), upper_ptr(n + 1, 0);
    for (int j = 0; j < n; ++j) {
        int nl = 0, nu = 0;
        for (int64_t k = row_ptr[j]; k < row_ptr[j + 1]; ++k) {
            nl += col_idx[k] <= j;
            nu += col_idx[k] >= j;
        }
        lower_ptr[j + 1] = lower_ptr[j] + nl;
        upper_ptr[j + 1] = upper_ptr[j] + nu;
    }
    const std::vector<int64_t> &first = mode == 2 ? lower_ptr : upper_ptr;
    const std::vector<int64_t> &second = mode == 2 ? upper_ptr : lower_ptr;
    int rows_max = 0, win_max = 0, blk_max = 0, y_max = 0, r_max = 0;
    int64_t f0_max = 0, f1_max = 0;
    for (int c = 0; c < ctas; ++c) {
        const int lo = (int)(((long long)n * c) / ctas);
        const int hi = (int)(((long long)n * (c + 1)) / ctas);
        int wlo = lo, whi = hi;
        for (int i = lo; i < hi; ++i) {
            wlo = std::min(wlo, cmin[i]);
            whi = std::max(whi, cmax[i] + 1);
        }
        // Y: the second pass's columns from [lo, hi); R: the first pass's from Y
        int ylo, yhi, rlo, rhi;
        if (mode == 2) {  // F^T (upper) second, F (lower) first
            ylo = lo;
            yhi = whi;
            rlo = ylo;
            for (int j = ylo; j < yhi; ++j) rlo = std::min(rlo, cmin[j]);
            rhi = yhi;
        } else {  // F (lower) second, F^T (upper) first
            ylo = wlo;
            yhi = hi;
            rlo = ylo;
            rhi = yhi;
            for (int j = ylo; j < yhi; ++j) rhi = std::max(rhi, cmax[j] + 1);
        }
        rlo = std::min(rlo, lo) & ~3;  // 48-byte aligned copies, whole groups of 4 rows
        rhi = (std::max(rhi, hi) + 3) & ~3;
        wlo &= ~3;
        whi = (whi + 3) & ~3;
        if (hi == lo) {
            wlo = whi = rlo = rhi = lo & ~3;
            ylo = yhi = lo;
        }
        cta_info[c] = make_int4(lo, hi, wlo, whi);
        factor_info[c] = make_int4(ylo, yhi, rlo, rhi);
        rows_max = std::max(rows_max, hi - lo);
        win_max = std::max(win_max, whi - wlo);
        blk_max = std::max(blk_max, (int)(row_ptr[hi] - row_ptr[lo]));
        y_max = std::max(y_max, yhi - ylo);
        r_max = std::max(r_max, rhi - rlo);
        f0_max = std::max(f0_max, first[yhi] - first[ylo]);
        f1_max = std::max(f1_max, second[hi] - second[lo]);
    }
    L.rows_max = (rows_max + 3) & ~3;
    L.win_max = (win_max + 3) & ~3;
    L.blk_max = (blk_max + 3) & ~3;
    L.y_max = (y_max + 3) & ~3;
    L.r_max = (r_max + 3) & ~3;
    L.f0_max = (int)((f0_max + 3) & ~(int64_t)3);
    L.f1_max = (int)((f1_max + 3) & ~(int64_t)3);
    L.variant = PcgLayout::kFactor;
    // shared-memory copies in order of worth: with few rows a CTA, the
    // factor passes (several trips of dependent loads) gain more than H's
    // product (one trip); the factor's row pointers (a few KB) take one
    // dependent load off every trip
    const int opts[5][2] = {{1, kFactorAll}, {0, kFactorAll}, {1, kFactorRows}, {0, kFactorRows}, {0, kFactorNone}};
    const int plain[2][2] = {{1, kFactorNone}, {0, kFactorNone}};  // block-Jacobi only: no factor rows
    for (const auto &o : opts) {
        if (!factor) break;
        const size_t bytes = smem_factor(L, o[0] != 0, o[1]);
        if (bytes <= budget) {
            L.cache_matrix = o[0];
            L.factor_cache = o[1];
            L.smem = bytes;
            return cudaFuncSetAttribute(pick_factor_kernel(L), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)L.smem);
        }
    }
    for (const auto &o : plain) {
        const size_t bytes = smem_factor(L, o[0] != 0, o[1]);
        if (factor || bytes > budget) continue;
        L.cache_matrix = o[0];
        L.factor_cache = o[1];
        L.smem = bytes;
        return cudaFuncSetAttribute(pick_factor_kernel(L), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
    }
    err = "mesh too large for the persistent factor PCG (shared memory per CTA exceeded)";
    return cudaErrorInvalidValue;
}

namespace {

cudaError_t launch_factor_args(const BsrViews &bv, const VertexViews &vv, const PcgWork &w, const BatchViews &bw,
                               const PcgLayout &L, int ctas, int slot, float tol, int maxiter, int mode,
                               const float *b, float *x, const IrWork *ir, cudaStream_t s, bool fused = false) {
    // 1 (block-Jacobi) only as an inner solve of a plan without a factor
    if (mode != 2 && mode != 3 && !(ir && mode == 1)) return cudaErrorInvalidValue;
    PcgArgs a = {};
    a.n = bv.n;
    a.row_ptr = bv.row_ptr;
    a.col_idx = bv.col_idx;
    a.values = bv.values;
    a.Minv = vv.Minv;
    a.b = b;
    a.x = x;
    a.pub = w.pub;
    a.n_pad = w.n_pad;
    a.cta = L.cta_info;
    a.rows_max = L.rows_max;
    a.blk_max = L.blk_max;
    a.win_max = L.win_max;
    a.partials = w.partials;
    a.counter = w.counter;
    a.error = w.error;
    // the one-body records, [slot][1]; an inner solve's record is the
    // refinement's, which its residual pass writes
    a.stats = ir ? w.stats : bw.stats;
    a.slot = slot;
    a.tol = tol;
    a.maxiter = maxiter;
    a.use_precond = mode;
    a.fcta = L.factor_info;
    const bool lower_first = mode == 2;
    a.rp0 = lower_first ? bw.lrow : bw.urow;
    a.c0 = lower_first ? bw.lcol : bw.ucol;
    a.v0 = lower_first ? bw.Lb : bw.Ub;
    a.rp1 = lower_first ? bw.urow : bw.lrow;
    a.c1 = lower_first ? bw.ucol : bw.lcol;
    a.v1 = lower_first ? bw.Ub : bw.Lb;
    a.y_max = L.y_max;
    a.r_max = L.r_max;
    a.f0_max = L.f0_max;
    a.f1_max = L.f1_max;
    if (ir) {
        a.ir_state = ir->state;
        a.ir_scale = ir->scale;
        a.values_w = ir->hq_words;
        a.row_scale = ir->row_scale;
        a.lowp_kind = ir->mode == kIrBf16 ? 1 : 2;
        if (fused) {
            a.fused = 1;
            a.g = vv.rhs;
            a.dx = vv.dx;
            a.irw = *ir;
        }
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(kPcgThreads);
    cfg.dynamicSmemBytes = L.smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t err = cudaLaunchKernelEx(&cfg, pick_factor_kernel(L), a);
    count_launches(1);
    return err;
}

}  // namespace

cudaError_t launch_pcg_factor(const BsrViews &bv, const VertexViews &vv, const PcgWork &w, const BatchViews &bw,
                              const PcgLayout &L, int ctas, int slot, float tol, int maxiter, int mode,
                              cudaStream_t s) {
    return launch_factor_args(bv, vv, w, bw, L, ctas, slot, tol, maxiter, mode, vv.rhs, vv.dx, nullptr, s);
}

cudaError_t launch_pcg_factor_inner(const BsrViews &bv, const VertexViews &vv, const IrWork &ir, const PcgWork &pw,
                                    const BatchViews &bw, const PcgLayout &L, int ctas, int slot, int maxiter,
                                    int mode, cudaStream_t s) {
    return launch_factor_args(bv, vv, pw, bw, L, ctas, slot, ir.inner_tol, maxiter, mode, ir.res, ir.e, &ir, s);
}

cudaError_t launch_pcg_factor_refine(const BsrViews &bv, const VertexViews &vv, const IrWork &ir,
                                     const PcgWork &pw, const BatchViews &bw, const PcgLayout &L, int ctas, int slot,
                                     int maxiter, int mode, cudaStream_t s) {
    return launch_factor_args(bv, vv, pw, bw, L, ctas, slot, ir.inner_tol, maxiter, mode, ir.res, ir.e, &ir, s,
                              true);
}

}  // namespace mfem
