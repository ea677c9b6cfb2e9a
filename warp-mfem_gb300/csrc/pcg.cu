// Block-Jacobi preconditioned CG on the 3x3-block BSR system H dx = g, as
// one persistent cooperative kernel per solve.
//
// The reference runs warp.optim.linear.cg (check_every=0, graph-captured,
// M = block-Jacobi inverse) (src/mfem/refinement/solver.py:220-235, 581-609).
// Here the whole solve loops on the device, with no host round trip.
//
// Data placement.  Each CTA owns a contiguous range of block rows, keeps that
// range's vectors in shared memory and -- when it fits -- its slice of H
// (values and window-local column indices), so H is read once per solve.
// Before each sparse product the CTA stages the contiguous "window" of rows
// that its columns reach (the mesh ordering keeps it narrow) from global into
// shared memory with bulk asynchronous copies (cp.async.bulk, completion on
// an mbarrier), issued as soon as the data is published.
//
// Two formulations of the same PCG iteration (equal iterates in exact
// arithmetic):
//
//  * single-reduction (Chronopoulos & Gear 1989, "s-step iterative methods
//    for symmetric linear systems"; the "CG-CG" of Ghysels & Vanroose 2014):
//        p = u + beta p;  s = w + beta s;  x += alpha p;  r -= alpha s;
//        u = M r;  w = H u;  gamma = (r, u), delta = (w, u), (r, r)
//        beta' = gamma' / gamma;  alpha' = gamma' / (delta' - beta' gamma' / alpha)
//    One grid barrier per iteration: the neighbours' u = M (r - alpha (w +
//    beta s)) is rebuilt by each CTA over its window from the (r, w, s) that
//    the owners published at the end of the previous iteration (double
//    buffered by iteration parity).  Every CTA computes its window rows with
//    the same instructions from the same published values, so owners and
//    neighbours agree bit for bit.
//  * standard (Hestenes-Stiefel, the reference's form), two barriers per
//    iteration: A: p = z + beta p over the window, Ap = H p, (p, Ap);
//    B: x += alpha p, r -= alpha Ap, z = M r, (r, z), (r, r).  Used when the
//    single-reduction windows do not fit in shared memory.
//  * gather: the standard form without windows, other rows gathered from L2;
//    for meshes whose vertex order is not banded.
//
// Grid synchronisation is a reduction: each CTA stores its partial sums
// (double buffered by barrier parity), then arrives on a 64-bit counter that
// is never reset -- the k-th barrier of a launch releases at base + k * CTAs
// -- with one thread per CTA polling it (release add, acquire loads:
// grid_sync.cuh).  Measured on GB300 with 152 CTAs, partials round trip
// included: 1.94 us per barrier.  Per-CTA flag words that every CTA polls
// took 4.6 us; per-CTA "published" words polled only by the CTAs whose
// windows they feed, to start the window copies before the whole grid has
// arrived, took 3.4 us packed eight to a cache line and 2.3 us one to a line,
// both slower than this barrier alone.  After the release every CTA reads
// all partials in one round trip while its thread 0 issues the next window
// copies, and sums them in the same fixed order, so all CTAs take the same
// decisions and the result is deterministic.  Dot products and the scalar
// recurrence are float32 like the reference's CG (GB300's float64 rate is
// low); the scalars are computed by one thread per CTA and broadcast.
// Stopping test ||r|| <= tol ||g|| on the recurrence residual, before the
// first iteration and after each one.
//
// Every wait (barrier, mbarrier) is bounded; after a timeout the kernel sets
// the sticky error flag, waits (bounded) for its own copies in flight and
// leaves, reporting MFEM_TIMEOUT.
#include "pcg_common.cuh"

namespace mfem {
namespace {

// ===========================================================================
// single-reduction (Chronopoulos-Gear) PCG
// ===========================================================================
// The single-reduction kernel keeps its cached slice of H as 48-byte blocks:
// the nine values, the column relative to the window as int bits, two zeros,
// read with three 16-byte loads instead of ten 4-byte ones (the sums in the
// order of window_product, so the iterates are the same bit for bit).
__device__ __forceinline__ void load_matrix_slice48(const PcgArgs &a, const Common &c, int *rowoff, float *sHB) {
    for (int i = threadIdx.x; i <= c.nrows; i += blockDim.x) rowoff[i] = a.row_ptr[c.row_lo + i] - c.blk_lo;
    for (int t = threadIdx.x; t < 12 * c.nblk; t += blockDim.x) {
        const int k = t / 12, e = t - 12 * k;
        float v = 0.0f;
        if (e < 9) v = a.values[(size_t)9 * (c.blk_lo + k) + e];
        else if (e == 9) v = __int_as_float(a.col_idx[c.blk_lo + k] - c.win_lo);
        sHB[t] = v;
    }
}

template <bool CACHE>
__device__ __forceinline__ void product48(const PcgArgs &a, const int *rowoff, const float *sH, const int *sCol,
                                          int blk_lo, int win_lo, int nrows, const float *win, float *out,
                                          const HBlocks &hm, int row_lo) {
    if constexpr (!CACHE) {
        window_product<false>(a, rowoff, sH, sCol, blk_lo, win_lo, nrows, win, out, hm, row_lo);
    } else {
        const int g_lane = threadIdx.x & (kGroup - 1);
        const int group = threadIdx.x / kGroup;
        const int ngroups = blockDim.x / kGroup;
        const unsigned gmask = ((1u << kGroup) - 1u) << (threadIdx.x & (32 - kGroup));
        const float4 *blocks = reinterpret_cast<const float4 *>(sH);
        for (int i = group; i < nrows; i += ngroups) {
            const int kb = rowoff[i], ke = rowoff[i + 1];
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
#pragma unroll 4
            for (int k = kb + g_lane; k < ke; k += kGroup) {
                const float4 h0 = blocks[3 * k], h1 = blocks[3 * k + 1], h2 = blocks[3 * k + 2];
                const int c = __float_as_int(h2.y);
                const float v0 = win[3 * c + 0], v1 = win[3 * c + 1], v2 = win[3 * c + 2];
                a0 += h0.x * v0 + h0.y * v1 + h0.z * v2;
                a1 += h0.w * v0 + h1.x * v1 + h1.y * v2;
                a2 += h1.z * v0 + h1.w * v1 + h2.x * v2;
            }
#pragma unroll
            for (int off = kGroup / 2; off > 0; off >>= 1) {
                a0 += __shfl_xor_sync(gmask, a0, off);
                a1 += __shfl_xor_sync(gmask, a1, off);
                a2 += __shfl_xor_sync(gmask, a2, off);
            }
            if (g_lane == 0) {
                out[3 * i + 0] = a0;
                out[3 * i + 1] = a1;
                out[3 * i + 2] = a2;
            }
        }
    }
}

template <bool CACHE>
__global__ void __launch_bounds__(kPcgThreads, 1) pcg_single_kernel(PcgArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    // As an inner solve of the mixed-precision refinement's launch sequence
    // (fp32 blocks, block-Jacobi): nothing to do once the refinement has
    // finished; otherwise a solve from 0 of the residual scaled to unit norm
    // (ir_scale[0]), the correction scaled back (ir_scale[1]) and the state
    // words updated as the factor kernel's inner solve does (pcg_factor.cu).
    const bool inner = a.ir_state != nullptr;
    if (inner) {
        if (ld_volatile(a.ir_state) != 0 || ld_volatile(a.ir_state + 7) != 0) return;
        if (ld_volatile(a.error) != 0) {
            if (blockIdx.x == 0 && threadIdx.x == 0) {
                a.ir_state[5] = MFEM_TIMEOUT;
                a.ir_state[0] = 1;
            }
            return;
        }
    }
    PCG_PROLOGUE
    const float bscale = inner ? a.ir_scale[0] : 1.0f;
    const HBlocks hf32{a.values, nullptr, nullptr, 0};
    const int rows_max = a.rows_max, win_max = a.win_max;
    // own rows
    float *sX = reinterpret_cast<float *>(smem);
    float *sU = sX + 3 * rows_max;
    float *sP = sU + 3 * rows_max;
    float *sW = sP + 3 * rows_max;
    // window rows
    float *wR = sW + 3 * rows_max;
    float *wW = wR + 3 * win_max;
    float *wS = wW + 3 * win_max;
    float *wM = wS + 3 * win_max;
    int *rowoff = reinterpret_cast<int *>(wM + 9 * win_max);
    float *sH = reinterpret_cast<float *>(rowoff + rows_max + 4);  // with CACHE: 48-byte blocks
    int *sCol = nullptr;

    const size_t vec = (size_t)3 * a.n_pad;
    float *pubR[2] = {a.pub, a.pub + vec};
    float *pubW[2] = {a.pub + 2 * vec, a.pub + 3 * vec};
    float *pubS[2] = {a.pub + 4 * vec, a.pub + 5 * vec};
    const int own = cm.row_lo - cm.win_lo;  // offset of the own rows inside the window
    const uint32_t wbytes = (uint32_t)cm.nwin * 12u;

    if (CACHE) load_matrix_slice48(a, cm, rowoff, sH);
    else load_matrix_slice(a, cm, rowoff, sH, sCol, false, hf32);
    // window of M^-1 blocks (kept for the whole solve) and of the warm start
    bool ok = true;
    if (threadIdx.x == 0 && cm.nwin > 0) {
        tma_expect(&s_mbar, wbytes * (inner ? 3u : 4u));
        tma_copy(wM, a.Minv + (size_t)9 * cm.win_lo, wbytes * 3u, &s_mbar);
        if (!inner) tma_copy(wR, a.x + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
    }
    if (cm.nwin > 0) ok = tma_wait(&s_mbar, parity, a.error);

    int it = 0;
    // ---- r0 = g - H x0 (x0 = 0 for an inner solve), published
    if (ok) {
        if (inner) {
            for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) sX[i] = sW[i] = 0.0f;
        } else {
            for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) sX[i] = wR[3 * own + i];
            product48<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.win_lo, cm.nrows, wR, sW, hf32, cm.row_lo);
        }
        __syncthreads();
        float acc[1] = {0.0f};
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) {
            const float bg = a.b[(size_t)3 * cm.row_lo + i] * bscale;
            pubR[0][(size_t)3 * cm.row_lo + i] = bg - sW[i];
            acc[0] = __fmaf_rn(bg, bg, acc[0]);
        }
        ok = reduce_arrive<1>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok);
        if (ok) {
            reduce_totals<1>(a.partials, bar, s_val, s_tot);
            if (threadIdx.x == 0) {
                sc.bb = s_tot[0];
                sc.thr2 = a.tol * a.tol * s_tot[0];
            }
        }
        ++bar;
    }
    // ---- u0 = M r0 over the window, w0 = H u0, gamma0, delta0, (r0, r0)
    if (ok) {
        if (threadIdx.x == 0 && cm.nwin > 0) {
            tma_expect(&s_mbar, wbytes);
            tma_copy(wR, pubR[0] + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
        }
        if (cm.nwin > 0) ok = tma_wait(&s_mbar, parity, a.error);
    }
    if (ok) {
        for (int j = threadIdx.x; j < cm.nwin; j += blockDim.x) {
            float u[3];
            precond(wM + 9 * j, wR + 3 * j, u, a.use_precond);
            wW[3 * j + 0] = u[0];
            wW[3 * j + 1] = u[1];
            wW[3 * j + 2] = u[2];
        }
        __syncthreads();
        product48<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.win_lo, cm.nrows, wW, sW, hf32, cm.row_lo);
        __syncthreads();
        float acc[3] = {0.0f, 0.0f, 0.0f};
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) {
            const float r = wR[3 * own + i], u = wW[3 * own + i], w = sW[i];
            sU[i] = u;
            pubW[0][(size_t)3 * cm.row_lo + i] = w;
            acc[0] = __fmaf_rn(r, u, acc[0]);
            acc[1] = __fmaf_rn(w, u, acc[1]);
            acc[2] = __fmaf_rn(r, r, acc[2]);
        }
        ok = reduce_arrive<3>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok);
    }
    bool pending = false;  // a staging copy is in flight
    if (ok) {
        if (threadIdx.x == 0 && cm.nwin > 0) {
            tma_expect(&s_mbar, 2u * wbytes);
            tma_copy(wR, pubR[0] + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
            tma_copy(wW, pubW[0] + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
        }
        pending = cm.nwin > 0;
        reduce_totals<3>(a.partials, bar, s_val, s_tot);
        if (threadIdx.x == 0) {
            const float gamma = s_tot[0], delta = s_tot[1], rr = s_tot[2];
            sc.gamma = gamma;
            sc.rr = rr;
            sc.beta = 0.0f;
            sc.status = MFEM_OK;
            if (!isfinite(gamma) || !isfinite(delta) || !isfinite(rr) || !isfinite(sc.bb))
                sc.status = MFEM_NONFINITE;
            else if (!(delta > 0.0f) && rr > 0.0f)
                sc.status = MFEM_STAGNATION;
            sc.alpha = delta > 0.0f ? gamma / delta : 0.0f;
            sc.done = sc.status != MFEM_OK || rr <= sc.thr2;
        }
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
        // state `it` of the window: r, w (and s of the previous iteration);
        // each thread waits for the copies itself and the verdicts join the
        // sync after the window update
        const bool landed = !pending || tma_wait_local(&s_mbar, parity);
        pending = false;
        const float fa = sc.alpha, fb = sc.beta;
        // s = w + beta s; r' = r - alpha s; u' = M r'   (every window row)
        for (int j = threadIdx.x; j < cm.nwin; j += blockDim.x) {
            float r[3], u[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float sv = it == 0 ? wW[3 * j + c] : __fmaf_rn(fb, wS[3 * j + c], wW[3 * j + c]);
                wS[3 * j + c] = sv;
                r[c] = __fmaf_rn(-fa, sv, wR[3 * j + c]);
                wR[3 * j + c] = r[c];
            }
            precond(wM + 9 * j, r, u, a.use_precond);
            wW[3 * j + 0] = u[0];
            wW[3 * j + 1] = u[1];
            wW[3 * j + 2] = u[2];
        }
        if (!__syncthreads_and(landed)) {
            if (threadIdx.x == 0) {
                atomicExch(a.error, 1);
                sc.status = MFEM_TIMEOUT;
            }
            break;
        }
        // own rows: p = u + beta p, x += alpha p; publish r', s
        float *pr = pubR[(it + 1) & 1];
        float *ps = pubS[(it + 1) & 1];
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) {
            const float pv = it == 0 ? sU[i] : __fmaf_rn(fb, sP[i], sU[i]);
            sP[i] = pv;
            sX[i] = __fmaf_rn(fa, pv, sX[i]);
            sU[i] = wW[3 * own + i];
            pr[(size_t)3 * cm.row_lo + i] = wR[3 * own + i];
            ps[(size_t)3 * cm.row_lo + i] = wS[3 * own + i];
        }
        // w' = H u'
        product48<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.win_lo, cm.nrows, wW, sW, hf32, cm.row_lo);
        __syncthreads();
        float *pw = pubW[(it + 1) & 1];
        float acc[3] = {0.0f, 0.0f, 0.0f};
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) {
            const float r = wR[3 * own + i], u = sU[i], w = sW[i];
            pw[(size_t)3 * cm.row_lo + i] = w;
            acc[0] = __fmaf_rn(r, u, acc[0]);
            acc[1] = __fmaf_rn(w, u, acc[1]);
            acc[2] = __fmaf_rn(r, r, acc[2]);
        }
        if (!reduce_arrive<3>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok)) {
            if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
            break;
        }
        ++it;
        // stage the next state from warp 1 while warp 0 fetches the totals
        if (threadIdx.x == 32 && cm.nwin > 0) {
            tma_expect(&s_mbar, 3u * wbytes);
            tma_copy(wR, pr + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
            tma_copy(wW, pw + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
            tma_copy(wS, ps + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
        }
        pending = cm.nwin > 0;
        reduce_totals_w0<3>(a.partials, bar, s_tot);
        ++bar;
        if (threadIdx.x == 0) {
            const float gamma_new = s_tot[0], delta = s_tot[1], rr = s_tot[2];
            sc.rr = rr;
            if (!isfinite(gamma_new) || !isfinite(delta) || !isfinite(rr)) {
                sc.status = MFEM_NONFINITE;
                sc.done = 1;
            } else if (rr <= sc.thr2) {
                sc.done = 1;
            } else {
                const float beta = gamma_new / sc.gamma;
                const float denom = delta - beta * gamma_new / sc.alpha;
                if (!(denom > 0.0f)) {
                    sc.status = MFEM_STAGNATION;
                    sc.done = 1;
                } else {
                    sc.beta = beta;
                    sc.alpha = gamma_new / denom;
                    sc.gamma = gamma_new;
                }
            }
        }
        __syncthreads();
    }
    if (pending) tma_wait(&s_mbar, parity, a.error);
    __syncthreads();
    if (!inner) {
        finish(a, cm, sX, sc, it);
        return;
    }
    // the correction for the refinement and its state (a solve that stopped
    // at the cap or stagnated still hands over its iterate)
    const float es = a.ir_scale[1];
    for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) a.x[(size_t)3 * cm.row_lo + i] = sX[i] * es;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ir_state[2] += it;
        a.ir_state[3] = 1;
        if (sc.status == MFEM_TIMEOUT || sc.status == MFEM_NONFINITE) {
            a.ir_state[5] = sc.status;
            a.ir_state[0] = 1;
        }
    }
}

// ===========================================================================
// standard (two-barrier) PCG
// ===========================================================================
template <bool CACHE>
__global__ void __launch_bounds__(kPcgThreads, 1) pcg_standard_kernel(PcgArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    PCG_PROLOGUE
    const HBlocks hf32{a.values, nullptr, nullptr, 0};
    const int rows_max = a.rows_max, win_max = a.win_max;
    float *sX = reinterpret_cast<float *>(smem);
    float *sR = sX + 3 * rows_max;
    float *sAp = sR + 3 * rows_max;
    float *sM = sAp + 3 * rows_max;
    float *winA = sM + 9 * rows_max;
    float *winB = winA + 3 * win_max;
    int *rowoff = reinterpret_cast<int *>(winB + 3 * win_max);
    float *sH = reinterpret_cast<float *>(rowoff + rows_max + 4);
    int *sCol = reinterpret_cast<int *>(sH + (CACHE ? 9 * a.blk_max : 0));

    const size_t vec = (size_t)3 * a.n_pad;
    float *pubZ = a.pub;
    float *pubP[2] = {a.pub + vec, a.pub + 2 * vec};
    const int own = cm.row_lo - cm.win_lo;
    const uint32_t wbytes = (uint32_t)cm.nwin * 12u;

    load_matrix_slice(a, cm, rowoff, sH, sCol, CACHE, HBlocks{a.values, nullptr, nullptr, 0});
    for (int i = threadIdx.x; i < 9 * cm.nrows; i += blockDim.x) sM[i] = a.Minv[(size_t)9 * cm.row_lo + i];
    bool ok = true;
    if (threadIdx.x == 0 && cm.nwin > 0) {
        tma_expect(&s_mbar, wbytes);
        tma_copy(winA, a.x + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
    }
    if (cm.nwin > 0) ok = tma_wait(&s_mbar, parity, a.error);

    int it = 0;
    if (ok) {
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) sX[i] = winA[3 * own + i];
        window_product<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.win_lo, cm.nrows, winA, sAp, hf32, cm.row_lo);
        __syncthreads();
        float acc[3] = {0.0f, 0.0f, 0.0f};
        for (int i = threadIdx.x; i < cm.nrows; i += blockDim.x) {
            const int row = cm.row_lo + i;
            float r[3], z[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float bc = a.b[3 * row + c];
                r[c] = bc - sAp[3 * i + c];
                sR[3 * i + c] = r[c];
                acc[2] = __fmaf_rn(bc, bc, acc[2]);
            }
            precond(sM + 9 * i, r, z, a.use_precond);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                pubZ[3 * row + c] = z[c];
                acc[0] = __fmaf_rn(r[c], z[c], acc[0]);
                acc[1] = __fmaf_rn(r[c], r[c], acc[1]);
            }
        }
        ok = reduce_arrive<3>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok);
    }
    bool pending = false;
    if (ok) {
        if (threadIdx.x == 0 && cm.nwin > 0) {
            tma_expect(&s_mbar, wbytes);
            tma_copy(winA, pubZ + (size_t)3 * cm.win_lo, wbytes, &s_mbar);
        }
        reduce_totals<3>(a.partials, bar, s_val, s_tot);
        if (threadIdx.x == 0) {
            sc.gamma = s_tot[0];  // r.z
            sc.rr = s_tot[1];
            sc.bb = s_tot[2];
            sc.thr2 = a.tol * a.tol * s_tot[2];
            sc.beta = 0.0f;
            sc.status = (!isfinite(s_tot[0]) || !isfinite(s_tot[1]) || !isfinite(s_tot[2])) ? MFEM_NONFINITE : MFEM_OK;
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
        // ---- phase A: p = z + beta p over the window, Ap = H p, partial p.Ap
        float *p_new = pubP[it & 1];
        if (pending && !tma_wait(&s_mbar, parity, a.error)) {
            pending = false;
            if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
            break;
        }
        pending = false;
        const float fbeta = sc.beta;
        if (it > 0) {
            for (int j = threadIdx.x; j < 3 * cm.nwin; j += blockDim.x) winA[j] = __fmaf_rn(fbeta, winB[j], winA[j]);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x)
            p_new[(size_t)3 * cm.row_lo + i] = winA[3 * own + i];
        window_product<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.win_lo, cm.nrows, winA, sAp, hf32, cm.row_lo);
        __syncthreads();
        float pap[1] = {0.0f};
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x)
            pap[0] = __fmaf_rn(winA[3 * own + i], sAp[i], pap[0]);
        if (!reduce_arrive<1>(pap, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok)) {
            if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
            break;
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
        if (sc.done) break;
        const float alpha = sc.alpha;
        // ---- phase B: x += alpha p, r -= alpha Ap, z = M r
        float acc[2] = {0.0f, 0.0f};
        for (int i = threadIdx.x; i < cm.nrows; i += blockDim.x) {
            const int row = cm.row_lo + i;
            const float *pp = winA + 3 * (own + i);
            float r[3], z[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sX[3 * i + c] = __fmaf_rn(alpha, pp[c], sX[3 * i + c]);
                r[c] = __fmaf_rn(-alpha, sAp[3 * i + c], sR[3 * i + c]);
                sR[3 * i + c] = r[c];
            }
            precond(sM + 9 * i, r, z, a.use_precond);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                pubZ[3 * row + c] = z[c];
                acc[0] = __fmaf_rn(r[c], z[c], acc[0]);
                acc[1] = __fmaf_rn(r[c], r[c], acc[1]);
            }
        }
        if (!reduce_arrive<2>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok)) {
            if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
            break;
        }
        ++it;
        // the copies from warp 1 while warp 0 fetches the totals
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
    __syncthreads();
    finish(a, cm, sX, sc, it);
}

// ===========================================================================
// gather variant: standard two-barrier PCG for any vertex order
// ===========================================================================
// When the column windows do not fit in shared memory (a mesh whose vertex
// order is not banded), each CTA keeps only its own rows in shared memory and
// gathers the other rows' published z and previous p straight from L2 in the
// product; p_j = z_j + beta p_j is formed on the fly, with the same
// instructions the owner uses, so every CTA sees the same p.
template <bool CACHE>
__device__ __forceinline__ void gather_product(const PcgArgs &a, const int *rowoff, const float *sH, const int *sCol,
                                               int blk_lo, int nrows, const float *z, const float *p_old, float beta,
                                               float *out) {
    const int g_lane = threadIdx.x & (kGroup - 1);
    const int group = threadIdx.x / kGroup;
    const int ngroups = blockDim.x / kGroup;
    const unsigned gmask = ((1u << kGroup) - 1u) << (threadIdx.x & (32 - kGroup));
    for (int i = group; i < nrows; i += ngroups) {
        const int kb = rowoff[i], ke = rowoff[i + 1];
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
        // kGatherDepth blocks per lane and trip: their L2 gathers are in
        // flight together
        for (int k = kb + g_lane; k < ke; k += kGatherDepth * kGroup) {
            int c[kGatherDepth], kk[kGatherDepth];
            bool ok[kGatherDepth];
#pragma unroll
            for (int u = 0; u < kGatherDepth; ++u) {
                ok[u] = k + u * kGroup < ke;
                kk[u] = ok[u] ? k + u * kGroup : k;
                c[u] = CACHE ? sCol[kk[u]] : __ldg(a.col_idx + blk_lo + kk[u]);
            }
            float v[kGatherDepth][3];
#pragma unroll
            for (int u = 0; u < kGatherDepth; ++u)
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const float zc = __ldcg(z + 3 * c[u] + q);
                    v[u][q] = p_old ? __fmaf_rn(beta, __ldcg(p_old + 3 * c[u] + q), zc) : zc;
                    if (!ok[u]) v[u][q] = 0.0f;
                }
#pragma unroll
            for (int u = 0; u < kGatherDepth; ++u) {
                const float *h = CACHE ? sH + (size_t)kk[u] * 9 : a.values + (size_t)(blk_lo + kk[u]) * 9;
                a0 += h[0] * v[u][0] + h[1] * v[u][1] + h[2] * v[u][2];
                a1 += h[3] * v[u][0] + h[4] * v[u][1] + h[5] * v[u][2];
                a2 += h[6] * v[u][0] + h[7] * v[u][1] + h[8] * v[u][2];
            }
        }
#pragma unroll
        for (int off = kGroup / 2; off > 0; off >>= 1) {
            a0 += __shfl_xor_sync(gmask, a0, off);
            a1 += __shfl_xor_sync(gmask, a1, off);
            a2 += __shfl_xor_sync(gmask, a2, off);
        }
        if (g_lane == 0) {
            out[3 * i + 0] = a0;
            out[3 * i + 1] = a1;
            out[3 * i + 2] = a2;
        }
    }
}

template <bool CACHE>
__global__ void __launch_bounds__(kPcgThreads, 1) pcg_gather_kernel(PcgArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    PCG_PROLOGUE
    const int rows_max = a.rows_max;
    float *sX = reinterpret_cast<float *>(smem);
    float *sR = sX + 3 * rows_max;
    float *sAp = sR + 3 * rows_max;
    float *sP = sAp + 3 * rows_max;
    float *sM = sP + 3 * rows_max;
    int *rowoff = reinterpret_cast<int *>(sM + 9 * rows_max);
    float *sH = reinterpret_cast<float *>(rowoff + rows_max + 4);
    int *sCol = reinterpret_cast<int *>(sH + (CACHE ? 9 * a.blk_max : 0));
    (void)parity;

    const size_t vec = (size_t)3 * a.n_pad;
    float *pubZ = a.pub;
    float *pubP[2] = {a.pub + vec, a.pub + 2 * vec};
    const size_t own3 = (size_t)3 * cm.row_lo;

    for (int i = threadIdx.x; i <= cm.nrows; i += blockDim.x) rowoff[i] = a.row_ptr[cm.row_lo + i] - cm.blk_lo;
    if (CACHE) {
        for (int k = threadIdx.x; k < 9 * cm.nblk; k += blockDim.x) sH[k] = a.values[(size_t)9 * cm.blk_lo + k];
        for (int k = threadIdx.x; k < cm.nblk; k += blockDim.x) sCol[k] = a.col_idx[cm.blk_lo + k];
    }
    for (int i = threadIdx.x; i < 9 * cm.nrows; i += blockDim.x) sM[i] = a.Minv[(size_t)9 * cm.row_lo + i];
    for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) sX[i] = a.x[own3 + i];
    __syncthreads();

    int it = 0;
    bool ok;
    {
        // r = g - H x0 (x0 was written before the launch), z = M r
        gather_product<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.nrows, a.x, nullptr, 0.0f, sAp);
        __syncthreads();
        float acc[3] = {0.0f, 0.0f, 0.0f};
        for (int i = threadIdx.x; i < cm.nrows; i += blockDim.x) {
            float r[3], z[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float bc = a.b[own3 + 3 * i + c];
                r[c] = bc - sAp[3 * i + c];
                sR[3 * i + c] = r[c];
                acc[2] = __fmaf_rn(bc, bc, acc[2]);
            }
            precond(sM + 9 * i, r, z, a.use_precond);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                pubZ[own3 + 3 * i + c] = z[c];
                acc[0] = __fmaf_rn(r[c], z[c], acc[0]);
                acc[1] = __fmaf_rn(r[c], r[c], acc[1]);
            }
        }
        ok = reduce_arrive<3>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok);
    }
    if (ok) {
        reduce_totals<3>(a.partials, bar, s_val, s_tot);
        if (threadIdx.x == 0) {
            sc.gamma = s_tot[0];
            sc.rr = s_tot[1];
            sc.bb = s_tot[2];
            sc.thr2 = a.tol * a.tol * s_tot[2];
            sc.beta = 0.0f;
            sc.status = (!isfinite(s_tot[0]) || !isfinite(s_tot[1]) || !isfinite(s_tot[2])) ? MFEM_NONFINITE : MFEM_OK;
            sc.done = sc.status != MFEM_OK || s_tot[1] <= sc.thr2;
        }
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
        // ---- phase A: p = z + beta p (formed on the fly), Ap = H p, p.Ap
        float *p_new = pubP[it & 1];
        const float *p_old = it == 0 ? nullptr : pubP[(it + 1) & 1];
        const float fbeta = sc.beta;
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) {
            const float zc = __ldcg(pubZ + own3 + i);
            const float pv = p_old ? __fmaf_rn(fbeta, __ldcg(p_old + own3 + i), zc) : zc;
            sP[i] = pv;
            p_new[own3 + i] = pv;
        }
        gather_product<CACHE>(a, rowoff, sH, sCol, cm.blk_lo, cm.nrows, pubZ, p_old, fbeta, sAp);
        __syncthreads();
        float pap[1] = {0.0f};
        for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) pap[0] = __fmaf_rn(sP[i], sAp[i], pap[0]);
        if (!reduce_arrive<1>(pap, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok)) {
            if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
            break;
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
        if (sc.done) break;
        const float alpha = sc.alpha;
        // ---- phase B: x += alpha p, r -= alpha Ap, z = M r
        float acc[2] = {0.0f, 0.0f};
        for (int i = threadIdx.x; i < cm.nrows; i += blockDim.x) {
            float r[3], z[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                sX[3 * i + c] = __fmaf_rn(alpha, sP[3 * i + c], sX[3 * i + c]);
                r[c] = __fmaf_rn(-alpha, sAp[3 * i + c], sR[3 * i + c]);
                sR[3 * i + c] = r[c];
            }
            precond(sM + 9 * i, r, z, a.use_precond);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                pubZ[own3 + 3 * i + c] = z[c];
                acc[0] = __fmaf_rn(r[c], z[c], acc[0]);
                acc[1] = __fmaf_rn(r[c], r[c], acc[1]);
            }
        }
        if (!reduce_arrive<2>(acc, a.partials, bar, a.counter, target, a.error, s_redf, &s_ok)) {
            if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
            break;
        }
        ++it;
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
    __syncthreads();
    finish(a, cm, sX, sc, it);
}

size_t smem_gather(int rows_max, int blk_max, bool cache) {
    size_t bytes = (size_t)rows_max * 21 * 4 + (size_t)(rows_max + 4) * 4;
    if (cache) bytes += (size_t)blk_max * 40;
    return (bytes + 15) & ~(size_t)15;
}

size_t smem_single(int rows_max, int win_max, int blk_max, bool cache) {
    size_t floats = (size_t)rows_max * 12 + (size_t)win_max * 18;
    size_t bytes = floats * 4 + (size_t)(rows_max + 4) * 4;
    if (cache) bytes += (size_t)blk_max * 48;  // load_matrix_slice48
    return (bytes + 15) & ~(size_t)15;
}

size_t smem_standard(int rows_max, int win_max, int blk_max, bool cache) {
    size_t floats = (size_t)rows_max * 18 + (size_t)win_max * 6;
    size_t bytes = floats * 4 + (size_t)(rows_max + 4) * 4;
    if (cache) bytes += (size_t)blk_max * 40;
    return (bytes + 15) & ~(size_t)15;
}

typedef void (*PcgKernel)(PcgArgs);

PcgKernel pick_kernel(const PcgLayout &L) {
    if (L.variant == PcgLayout::kSingleReduction)
        return L.cache_matrix ? pcg_single_kernel<true> : pcg_single_kernel<false>;
    if (L.variant == PcgLayout::kGather)
        return L.cache_matrix ? pcg_gather_kernel<true> : pcg_gather_kernel<false>;
    return L.cache_matrix ? pcg_standard_kernel<true> : pcg_standard_kernel<false>;
}

}  // namespace

cudaError_t pcg_max_ctas(int device, int *ctas) {
    int sms = 0;
    cudaError_t err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    *ctas = std::min(sms, kMaxCtas);
    return err;
}

cudaError_t pcg_plan_layout(int device, PcgLayout &L, const int32_t *row_ptr, const int32_t *col_idx, int n,
                            int ctas, int variant, std::vector<int4> &cta_info, std::string &err) {
    int optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (e != cudaSuccess) return e;
    const size_t budget = (size_t)optin > kStaticSmem ? (size_t)optin - kStaticSmem : 0;
    if (ctas > kMaxCtas) {
        err = "pcg_ctas above " + std::to_string(kMaxCtas);
        return cudaErrorInvalidValue;
    }
    cta_info.assign(ctas, make_int4(0, 0, 0, 0));
    int rows_max = 0, win_max = 0, blk_max = 0;
    for (int c = 0; c < ctas; ++c) {
        const int lo = (int)(((long long)n * c) / ctas);
        const int hi = (int)(((long long)n * (c + 1)) / ctas);
        int wlo = lo, whi = hi;
        for (int64_t k = row_ptr[lo]; k < row_ptr[hi]; ++k) {
            wlo = std::min(wlo, (int)col_idx[k]);
            whi = std::max(whi, (int)col_idx[k] + 1);
        }
        wlo &= ~3;             // 48-byte (3 x 16 B) aligned start
        whi = (whi + 3) & ~3;  // length a multiple of 4 rows
        if (hi == lo) wlo = whi = lo & ~3;
        cta_info[c] = make_int4(lo, hi, wlo, whi);
        rows_max = std::max(rows_max, hi - lo);
        win_max = std::max(win_max, whi - wlo);
        blk_max = std::max(blk_max, (int)(row_ptr[hi] - row_ptr[lo]));
    }
    L.rows_max = (rows_max + 3) & ~3;
    L.win_max = (win_max + 3) & ~3;
    L.blk_max = (blk_max + 3) & ~3;
    struct Option {
        int variant;
        bool cache;
        size_t bytes;
    } opts[6] = {
        {PcgLayout::kSingleReduction, true, smem_single(L.rows_max, L.win_max, L.blk_max, true)},
        {PcgLayout::kStandard, true, smem_standard(L.rows_max, L.win_max, L.blk_max, true)},
        {PcgLayout::kSingleReduction, false, smem_single(L.rows_max, L.win_max, L.blk_max, false)},
        {PcgLayout::kStandard, false, smem_standard(L.rows_max, L.win_max, L.blk_max, false)},
        {PcgLayout::kGather, true, smem_gather(L.rows_max, L.blk_max, true)},
        {PcgLayout::kGather, false, smem_gather(L.rows_max, L.blk_max, false)},
    };
    bool found = false;
    for (const auto &o : opts) {
        if (variant != PcgLayout::kAuto && o.variant != variant) continue;
        if (o.bytes <= budget) {
            L.variant = o.variant;
            L.cache_matrix = o.cache ? 1 : 0;
            L.smem = o.bytes;
            found = true;
            break;
        }
    }
    if (!found) {
        err = "mesh too large for the persistent PCG (shared memory per CTA exceeded)";
        return cudaErrorInvalidValue;
    }
    PcgKernel k = pick_kernel(L);
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
}

namespace {

// The launch arguments of the plan's PCG from its views and workspace.
PcgArgs pcg_args(const BsrViews &bv, const VertexViews &vv, const PcgWork &w, const PcgLayout &L, int slot, float tol,
                 int maxiter, int use_precond) {
    PcgArgs a = {};
    a.n = bv.n;
    a.row_ptr = bv.row_ptr;
    a.col_idx = bv.col_idx;
    a.values = bv.values;
    a.Minv = vv.Minv;
    a.b = vv.rhs;
    a.x = vv.dx;
    a.pub = w.pub;
    a.n_pad = w.n_pad;
    a.cta = L.cta_info;
    a.rows_max = L.rows_max;
    a.blk_max = L.blk_max;
    a.win_max = L.win_max;
    a.partials = w.partials;
    a.counter = w.counter;
    a.error = w.error;
    a.stats = w.stats;
    a.slot = slot;
    a.tol = tol;
    a.maxiter = maxiter;
    a.use_precond = use_precond;
    return a;
}

// One cooperative launch of the layout's kernel.
cudaError_t launch_cooperative(const PcgArgs &a, const PcgLayout &L, int ctas, cudaStream_t s) {
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
    cudaError_t err = cudaLaunchKernelEx(&cfg, pick_kernel(L), a);
    count_launches(1);
    return err;
}

}  // namespace

cudaError_t launch_pcg(const BsrViews &bv, const VertexViews &vv, const PcgWork &w, const PcgLayout &L, int ctas,
                       int slot, float tol, int maxiter, int use_precond, cudaStream_t s) {
    return launch_cooperative(pcg_args(bv, vv, w, L, slot, tol, maxiter, use_precond), L, ctas, s);
}

// The single-reduction PCG as one inner solve of the refinement's launch
// sequence (block-Jacobi, fp32 blocks): rhs ir.res, correction to ir.e.
cudaError_t launch_pcg_inner(const BsrViews &bv, const VertexViews &vv, const IrWork &ir, const PcgWork &w,
                             const PcgLayout &L, int ctas, int slot, int maxiter, cudaStream_t s) {
    if (L.variant != PcgLayout::kSingleReduction) return cudaErrorInvalidValue;
    PcgArgs a = pcg_args(bv, vv, w, L, slot, ir.inner_tol, maxiter, 1);
    a.b = ir.res;
    a.x = ir.e;
    a.ir_state = ir.state;
    a.ir_scale = ir.scale;
    return launch_cooperative(a, L, ctas, s);
}

}  // namespace mfem
