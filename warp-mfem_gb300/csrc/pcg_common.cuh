// Building blocks of the persistent PCG kernels (pcg.cu, pcg_factor.cu): the
// launch arguments, the grid barrier that doubles as the reduction, the
// fixed-order totals, the bulk window copies with their bounded mbarrier
// waits, and the shared-memory window product.  Header-only: each kernel file
// instantiates its own copy.
#pragma once

#include "block_loads.cuh"
#include "double_float.cuh"
#include "grid_sync.cuh"
#include "internal.h"

namespace mfem {
namespace {
constexpr int kPcgThreads = 512;
constexpr int kGroup = 4;                         // lanes per block row in the product
constexpr int kGatherDepth = 4;                   // blocks per lane and trip in the gather product
constexpr int kMaxCtas = 256;
constexpr long long kWaitCycles = 8000000000ll;   // ~4 s at 2 GHz per wait
constexpr size_t kStaticSmem = 12 * 1024;         // static shared memory reserve

struct PcgArgs {
    int n;
    const int *row_ptr;
    const int *col_idx;
    const float *values;
    const float *Minv;   // [n_pad][9]
    const float *b;
    float *x;            // [n_pad][3] warm start in, solution out
    float *pub;          // published vectors, 6 x [n_pad][3]
    int n_pad;
    const int4 *cta;     // [ctas] (row_lo, row_hi, win_lo, win_hi)
    int rows_max, blk_max, win_max;
    float *partials;            // [2][kMaxCtas][4] per-CTA partial sums
    unsigned long long *counter;  // grid barrier arrivals (never reset)
    int *error;
    SolveStats *stats;
    int slot;
    float tol;
    int maxiter;
    int use_precond;
    // the factor preconditioner (pcg_factor.cu): per CTA the row ranges
    // (y_lo, y_hi, r_lo, r_hi); the first and second pass's forms (row
    // pointers, columns, BF16 blocks of kFactorLd values)
    const int4 *fcta;
    const int *rp0, *c0, *rp1, *c1;
    const __nv_bfloat16 *v0, *v1;
    int y_max, r_max;
    int f0_max, f1_max;  // most first- / second-pass blocks of a CTA (factor kept in shared memory)
    // the inner solve of the mixed-precision refinement (pcg_factor.cu): its
    // state words, the right-hand side's scale, H's blocks rounded to 16 bits
    int *ir_state;
    const float *ir_scale;
    // H's blocks rounded to 16 bits (kind 1 BF16, 2 FP16), nine values and a
    // zero in five words a block, with per-row scales: the inner solve's
    // matrix until the refinement switches to the fp32 H
    const uint32_t *values_w;
    const float *row_scale;
    int lowp_kind;
    // the whole refinement in this launch (pcg_factor.cu): every correction's
    // residual, decision and inner solve
    int fused;
    const float *g;      // [n][3] the system's right-hand side
    float *dx;           // [n][3] the solution as float for the local solve
    IrWork irw;
};

// The matrix a product reads: fp32 blocks, or 16-bit blocks (five words of
// pairs a block) times their row's scale.
struct HBlocks {
    const float *f32;
    const uint32_t *w16;  // null: fp32
    const float *scale;   // [n] row scales of the 16-bit blocks
    int kind;             // 1 BF16, 2 FP16
};

// One 16-bit block as nine floats, each the widened value times the row
// scale s: the numbers an fp32 copy of the scaled 16-bit blocks would hold.
__device__ __forceinline__ void load_block16(const HBlocks &h, long long k, float s, float m[9]) {
    uint32_t u[5];
    load_bf16_words(h.w16, k, u);
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        float2 t;
        if (h.kind == 1) {
            __nv_bfloat162 b;
            memcpy(&b, &u[i], 4);
            t = __bfloat1622float2(b);
        } else {
            __half2 b;
            memcpy(&b, &u[i], 4);
            t = __half22float2(b);
        }
        m[2 * i] = t.x * s;
        if (2 * i + 1 < 9) m[2 * i + 1] = t.y * s;
    }
}

// Value j (0..8) of 16-bit block k times s.
__device__ __forceinline__ float block16_value(const HBlocks &h, long long k, int j, float s) {
    const uint32_t w = __ldg(h.w16 + 5 * k + (j >> 1));
    const unsigned short bits = (unsigned short)((j & 1) ? (w >> 16) : (w & 0xffffu));
    const float v = h.kind == 1 ? __uint_as_float((uint32_t)bits << 16) : __half2float(__ushort_as_half(bits));
    return v * s;
}

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_volatile(const int *p) { return *(const volatile int *)p; }

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ---- reduction barrier --------------------------------------------------------
// Block-reduces NV per-thread float partials, stores the CTA's sums for
// barrier `k` (parity buffer) and waits at the grid barrier.  Returns false
// if the wait gave up.  CTA-uniform.
template <int NV>
__device__ bool reduce_arrive(float (&v)[NV], float *partials, unsigned k, unsigned long long *counter,
                              unsigned long long &target, int *error, float (*s_redf)[32], int *s_ok) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) s_redf[i][wid] = v[i];
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        float part[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            part[i] = lane < nw ? s_redf[i][lane] : 0.0f;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) part[i] += __shfl_down_sync(0xffffffffu, part[i], off);
        }
        if (lane == 0) {
            float *buf = partials + (size_t)(k & 1u) * kMaxCtas * 4 + (size_t)blockIdx.x * 4;
#pragma unroll
            for (int i = 0; i < NV; ++i) buf[i] = part[i];
            // arrive: every earlier store of this CTA (published vectors,
            // partials) is released before the counter moves
            target += gridDim.x;
            grid_arrive(counter);
            int ok = 1;
            const long long t0 = clock64();
            unsigned spins = 0;
            while (grid_count(counter) < target) {
                if ((++spins & 1023u) == 0 && (ld_volatile(error) != 0 || clock64() - t0 > kWaitCycles)) {
                    atomicExch(error, 1);
                    ok = 0;
                    break;
                }
            }
            *s_ok = ok;
        }
    }
    __syncthreads();
    return *s_ok != 0;
}

// Sums the partials of barrier `k` over all CTAs (after reduce_arrive):
// threads 0..nb*NV-1 fetch one each (one round trip), warp 0 adds them in a
// fixed order.  tot[] is valid for every thread on return.
template <int NV>
__device__ void reduce_totals(const float *partials, unsigned k, float *s_val, float *tot) {
    const int nb = gridDim.x;
    const float *buf = partials + (size_t)(k & 1u) * kMaxCtas * 4;
    for (int t = threadIdx.x; t < nb * NV; t += blockDim.x) {
        const int b = t / NV, i = t - b * NV;
        s_val[b * 4 + i] = __ldcg(buf + (size_t)b * 4 + i);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        float acc[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) acc[i] = 0.0f;
        for (int b = lane; b < nb; b += 32) {
#pragma unroll
            for (int i = 0; i < NV; ++i) acc[i] += s_val[b * 4 + i];
        }
#pragma unroll
        for (int i = 0; i < NV; ++i) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], off);
        }
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < NV; ++i) tot[i] = acc[i];
        }
    }
    __syncthreads();
}

// reduce_totals in warp 0 alone, for callers whose totals only thread 0
// reads: each lane loads its CTAs' partials into registers first (all in
// flight at once), then the warp adds them in reduce_totals' order, so the
// totals are the same bit for bit.  No shared-memory staging and no CTA-wide
// sync; tot[] is valid in thread 0 on return, and warps 1.. return at once
// (a window copy issued from warp 1 then leaves while warp 0 loads).
template <int NV>
__device__ __forceinline__ void reduce_totals_w0(const float *partials, unsigned k, float *tot) {
    if (threadIdx.x >= 32) return;
    const int nb = gridDim.x, lane = threadIdx.x;
    const float *buf = partials + (size_t)(k & 1u) * kMaxCtas * 4;
    float v[kMaxCtas / 32][NV];
#pragma unroll
    for (int j = 0; j < kMaxCtas / 32; ++j) {
        const int b = lane + 32 * j;
#pragma unroll
        for (int i = 0; i < NV; ++i) v[j][i] = b < nb ? __ldcg(buf + (size_t)b * 4 + i) : 0.0f;
    }
    float acc[NV];
#pragma unroll
    for (int i = 0; i < NV; ++i) acc[i] = 0.0f;
#pragma unroll
    for (int j = 0; j < kMaxCtas / 32; ++j) {
        if (lane + 32 * j < nb) {
#pragma unroll
            for (int i = 0; i < NV; ++i) acc[i] += v[j][i];
        }
    }
#pragma unroll
    for (int i = 0; i < NV; ++i) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], off);
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) tot[i] = acc[i];
    }
}

// reduce_arrive and reduce_totals in double, on a double partials buffer of
// the same [2][kMaxCtas][4] shape and the same barrier counter and parity.
template <int NV>
__device__ bool reduce_arrive_d(double (&v)[NV], double *partials, unsigned k, unsigned long long *counter,
                                unsigned long long &target, int *error, double (*s_redd)[32], int *s_ok) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) s_redd[i][wid] = v[i];
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        double part[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            part[i] = lane < nw ? s_redd[i][lane] : 0.0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) part[i] += __shfl_down_sync(0xffffffffu, part[i], off);
        }
        if (lane == 0) {
            double *buf = partials + (size_t)(k & 1u) * kMaxCtas * 4 + (size_t)blockIdx.x * 4;
#pragma unroll
            for (int i = 0; i < NV; ++i) buf[i] = part[i];
            target += gridDim.x;
            grid_arrive(counter);
            int ok = 1;
            const long long t0 = clock64();
            unsigned spins = 0;
            while (grid_count(counter) < target) {
                if ((++spins & 1023u) == 0 && (ld_volatile(error) != 0 || clock64() - t0 > kWaitCycles)) {
                    atomicExch(error, 1);
                    ok = 0;
                    break;
                }
            }
            *s_ok = ok;
        }
    }
    __syncthreads();
    return *s_ok != 0;
}

template <int NV>
__device__ void reduce_totals_d(const double *partials, unsigned k, double *s_vald, double *tot) {
    const int nb = gridDim.x;
    const double *buf = partials + (size_t)(k & 1u) * kMaxCtas * 4;
    for (int t = threadIdx.x; t < nb * NV; t += blockDim.x) {
        const int b = t / NV, i = t - b * NV;
        s_vald[b * NV + i] = __ldcg(buf + (size_t)b * 4 + i);
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double acc[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) acc[i] = 0.0;
        for (int b = lane; b < nb; b += 32) {
#pragma unroll
            for (int i = 0; i < NV; ++i) acc[i] += s_vald[b * NV + i];
        }
#pragma unroll
        for (int i = 0; i < NV; ++i) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], off);
        }
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < NV; ++i) tot[i] = acc[i];
        }
    }
    __syncthreads();
}

// Scalars of the iteration, decided by thread 0 and broadcast.
struct Scalars {
    float alpha, beta, gamma, rr, bb, thr2;
    int status, done;
};

// ---- bulk copies -----------------------------------------------------------
// Issued by thread 0 after a __syncthreads that ended every read of the
// destinations and after the reduction that published the sources.
__device__ __forceinline__ void tma_expect(uint64_t *mbar, uint32_t bytes) {
    asm volatile("fence.proxy.async.global;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void tma_copy(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(mbar))
                 : "memory");
}

// tma_wait without the CTA sync: each thread waits for the phase itself
// (bounded, the same second wait after a timeout), and the caller joins the
// verdicts at its next __syncthreads_and (setting the error flag if one gave
// up).  Per thread, not CTA-uniform.
__device__ __forceinline__ bool tma_wait_local(uint64_t *mbar, uint32_t &parity) {
    const uint32_t mb = smem_addr(mbar);
    bool ok = true;
    for (int attempt = 0; attempt < 2; ++attempt) {
        uint32_t done = 0;
        const long long t0 = clock64();
        unsigned spins = 0;
        while (!done) {
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(mb), "r"(parity)
                : "memory");
            if (!done && (++spins & 255u) == 0 && clock64() - t0 > kWaitCycles / 2) break;
        }
        if (done) break;
        ok = false;
    }
    parity ^= 1u;
    return ok;
}

// Waits for the mbarrier phase `parity` (bounded; a second bounded wait after
// a timeout so no copy is still writing when the CTA leaves).  CTA-uniform.
__device__ bool tma_wait(uint64_t *mbar, uint32_t &parity, int *error) {
    const uint32_t mb = smem_addr(mbar);
    bool ok = true;
    for (int attempt = 0; attempt < 2; ++attempt) {
        uint32_t done = 0;
        const long long t0 = clock64();
        unsigned spins = 0;
        while (!done) {
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(mb), "r"(parity)
                : "memory");
            if (!done && (++spins & 255u) == 0 && clock64() - t0 > kWaitCycles / 2) break;
        }
        if (done) break;
        ok = false;
    }
    ok = __syncthreads_and(ok) != 0;
    if (!ok && threadIdx.x == 0) atomicExch(error, 1);
    parity ^= 1u;
    return ok;
}

// out[i] = sum_k H[k] win[col_k] over the CTA's rows, kGroup lanes per row;
// H's blocks from the shared-memory slice (CACHE) or from `values`.
template <bool CACHE>
__device__ __forceinline__ void window_product(const PcgArgs &a, const int *rowoff, const float *sH, const int *sCol,
                                               int blk_lo, int win_lo, int nrows, const float *win, float *out,
                                               const HBlocks &hm, int row_lo) {
    const int g_lane = threadIdx.x & (kGroup - 1);
    const int group = threadIdx.x / kGroup;
    const int ngroups = blockDim.x / kGroup;
    const unsigned gmask = ((1u << kGroup) - 1u) << (threadIdx.x & (32 - kGroup));
    if constexpr (!CACHE) {
        // H through L2: a group takes rows i and i + ngroups together, so
        // each lane has both rows' loads in flight; each row's sum runs in
        // the single-row order
        for (int i = group; i < nrows; i += 2 * ngroups) {
            const int ib = i + ngroups;
            const bool has_b = ib < nrows;
            const int kba = rowoff[i], kea = rowoff[i + 1];
            const int kbb = has_b ? rowoff[ib] : kba, keb = has_b ? rowoff[ib + 1] : kba;
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, b0 = 0.0f, b1 = 0.0f, b2 = 0.0f;
            const bool q16 = hm.w16 != nullptr;
            const float sa = q16 ? __ldg(hm.scale + row_lo + i) : 1.0f;
            const float sb = q16 ? __ldg(hm.scale + row_lo + (has_b ? ib : i)) : 1.0f;
#pragma unroll 2
            for (int t = g_lane; kba + t < kea || kbb + t < keb; t += kGroup) {
                const bool oka = kba + t < kea, okb = kbb + t < keb;
                const int ka = oka ? kba + t : kba, kq = okb ? kbb + t : kba;  // in-range stand-ins
                float ha[9], hb[9];
                if (q16) {
                    load_block16(hm, (long long)blk_lo + ka, sa, ha);
                    load_block16(hm, (long long)blk_lo + kq, sb, hb);
                } else {
                    load_block9(hm.f32, (long long)blk_lo + ka, ha);
                    load_block9(hm.f32, (long long)blk_lo + kq, hb);
                }
                const int ca = __ldg(a.col_idx + blk_lo + ka) - win_lo;
                const int cb = __ldg(a.col_idx + blk_lo + kq) - win_lo;
                const float u0 = oka ? win[3 * ca] : 0.0f, u1 = oka ? win[3 * ca + 1] : 0.0f,
                            u2 = oka ? win[3 * ca + 2] : 0.0f;
                const float w0 = okb ? win[3 * cb] : 0.0f, w1 = okb ? win[3 * cb + 1] : 0.0f,
                            w2 = okb ? win[3 * cb + 2] : 0.0f;
                a0 += ha[0] * u0 + ha[1] * u1 + ha[2] * u2;
                a1 += ha[3] * u0 + ha[4] * u1 + ha[5] * u2;
                a2 += ha[6] * u0 + ha[7] * u1 + ha[8] * u2;
                b0 += hb[0] * w0 + hb[1] * w1 + hb[2] * w2;
                b1 += hb[3] * w0 + hb[4] * w1 + hb[5] * w2;
                b2 += hb[6] * w0 + hb[7] * w1 + hb[8] * w2;
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
            if (g_lane == 0) {
                out[3 * i + 0] = a0;
                out[3 * i + 1] = a1;
                out[3 * i + 2] = a2;
                if (has_b) {
                    out[3 * ib + 0] = b0;
                    out[3 * ib + 1] = b1;
                    out[3 * ib + 2] = b2;
                }
            }
        }
    } else {
        for (int i = group; i < nrows; i += ngroups) {
            const int kb = rowoff[i], ke = rowoff[i + 1];
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
#pragma unroll 4
            for (int k = kb + g_lane; k < ke; k += kGroup) {
                const float *h = sH + (size_t)k * 9;
                const int c = sCol[k];
                const float v0 = win[3 * c + 0], v1 = win[3 * c + 1], v2 = win[3 * c + 2];
                a0 += h[0] * v0 + h[1] * v1 + h[2] * v2;
                a1 += h[3] * v0 + h[4] * v1 + h[5] * v2;
                a2 += h[6] * v0 + h[7] * v1 + h[8] * v2;
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

__device__ __forceinline__ void precond(const float *m, const float r[3], float z[3], int use) {
    if (!use) {
        z[0] = r[0];
        z[1] = r[1];
        z[2] = r[2];
        return;
    }
    z[0] = m[0] * r[0] + m[1] * r[1] + m[2] * r[2];
    z[1] = m[3] * r[0] + m[4] * r[1] + m[5] * r[2];
    z[2] = m[6] * r[0] + m[7] * r[1] + m[8] * r[2];
}

struct Common {
    int row_lo, nrows, win_lo, nwin, blk_lo, nblk;
};

__device__ __forceinline__ Common setup_common(const PcgArgs &a) {
    const int4 info = a.cta[blockIdx.x];
    Common c;
    c.row_lo = info.x;
    c.nrows = info.y - info.x;
    c.win_lo = info.z;
    c.nwin = info.w - info.z;
    c.blk_lo = a.row_ptr[c.row_lo];
    c.nblk = a.row_ptr[info.y] - c.blk_lo;
    return c;
}

__device__ __forceinline__ void load_matrix_slice(const PcgArgs &a, const Common &c, int *rowoff, float *sH,
                                                  int *sCol, bool cache, const HBlocks &hm) {
    for (int i = threadIdx.x; i <= c.nrows; i += blockDim.x) rowoff[i] = a.row_ptr[c.row_lo + i] - c.blk_lo;
    if (cache) {
        if (hm.w16 == nullptr) {
            for (int k = threadIdx.x; k < 9 * c.nblk; k += blockDim.x) sH[k] = hm.f32[(size_t)9 * c.blk_lo + k];
        } else {
            // a warp per row: its blocks' values times the row's scale
            __syncthreads();  // rowoff
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
            for (int i = warp; i < c.nrows; i += nwarps) {
                const float s = __ldg(hm.scale + c.row_lo + i);
                const int k0 = rowoff[i], nv = 9 * (rowoff[i + 1] - k0);
                for (int e = lane; e < nv; e += 32) {
                    const int k = k0 + e / 9, j = e - 9 * (e / 9);
                    sH[(size_t)9 * k + j] = block16_value(hm, (long long)c.blk_lo + k, j, s);
                }
            }
        }
        for (int k = threadIdx.x; k < c.nblk; k += blockDim.x) sCol[k] = a.col_idx[c.blk_lo + k] - c.win_lo;
    }
}

// Final bookkeeping: solution rows and stats.
__device__ __forceinline__ void finish(const PcgArgs &a, const Common &cm, const float *sX, const Scalars &sc,
                                       int it) {
    for (int i = threadIdx.x; i < 3 * cm.nrows; i += blockDim.x) a.x[(size_t)3 * cm.row_lo + i] = sX[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const float rel = sc.bb > 0.0f ? sqrtf(sc.rr / sc.bb) : sqrtf(sc.rr);
        a.stats[a.slot] = SolveStats{it, sc.status, rel, 0.0f};
    }
}

#define PCG_PROLOGUE                                                                        \
    __shared__ float s_redf[4][32];                                                         \
    __shared__ float s_val[4 * kMaxCtas];                                                   \
    __shared__ float s_tot[4];                                                              \
    __shared__ Scalars sc;                                                                  \
    __shared__ int s_ok;                                                                    \
    __shared__ unsigned long long s_base;                                                   \
    __shared__ __align__(8) uint64_t s_mbar;                                                \
    const Common cm = setup_common(a);                                                      \
    if (threadIdx.x == 0) {                                                                 \
        s_base = (ld_relaxed(a.counter) / gridDim.x) * (unsigned long long)gridDim.x;     \
        s_ok = ld_volatile(a.error) == 0;                                                   \
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&s_mbar)) : "memory"); \
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");                  \
    }                                                                                       \
    __syncthreads();                                                                        \
    unsigned long long target = s_base;                                                     \
    unsigned bar = 0;                                                                       \
    uint32_t parity = 0;                                                                    \
    if (!s_ok) {                                                                            \
        if (blockIdx.x == 0 && threadIdx.x == 0) a.stats[a.slot] = SolveStats{0, MFEM_TIMEOUT, 0.0f, 0.0f}; \
        return;                                                                             \
    }

}  // namespace
}  // namespace mfem
