// Mixed-precision global solve: iterative refinement with an FP64 residual
// around a block-Jacobi PCG on 16-bit blocks.
//
//   Hq = BSR blocks of H stored as bf16 or fp16, each block row scaled by its
//        largest |entry| (one fp32 scale per row), so every stored value is
//        in [-1, 1]; products accumulate in fp32.
//   dx (hi + lo pairs of floats, about 48 bits) starts at the reference's
//   warm start x~ - x; each outer iteration forms r = g - H dx from the fp32
//   H with the products summed in those pairs, stops when
//   ||r|| <= outer_tol ||g||, else solves Hq e = r to inner_tol with the PCG
//   (fp32 vectors, the fp32 block-Jacobi inverse) and sets dx += e.
//   If the refinement diverges (the relative residual rises above 4x its
//   best, or turns non-finite), the 16-bit H is too coarse for this system:
//   the solve restarts from the warm start with the fp32 H in the inner PCG.
//
// This is a mixed-precision variant of the global solve (the reference
// solves H dx = g with one float32 PCG, src/mfem/refinement/
// solver.py:581-609).  Every launch is unconditional so the sequence can be
// captured: a device flag written by the residual kernel turns the later
// kernels of a converged solve into no-ops.
//
// Kernels:
//   ir_convert_kernel   Hq and the row scales from H (one warp per row)
//   ir_begin_kernel     dx = warm start, state reset
//   ir_residual_kernel  dx += e (double-buffered, so rows read a consistent dx),
//                       r = g - H dx with dx and the sums of products held as
//                       pairs of floats (about 48 bits; GB300's fp64 pipe is
//                       narrow), its norm in fp64, partial sums; the last block
//                       to finish adds the partials in a fixed order and
//                       decides (converged / outer cap)
//   ir_pcg_kernel<T>    persistent cooperative PCG on Hq e = r, e0 = 0
//
// Precision FP32 (kIrFp32) keeps the fp32 H in the inner PCG from the start
// and converts nothing: the plain fp32 PCG inside the same fp64 refinement,
// for a solution whose fp64 residual reaches the outer tolerance.
//
// A plan on the persistent factor PCG (pcg_factor.cu) runs the inner solves
// there instead: ir_convert_kernel also writes Hq padded to 20-byte blocks
// (which that kernel widens and scales by the row scale as it loads them), and
// the residual kernel hands over r / ||r|| (so the fp32 sums of products
// cannot underflow) with ||r|| to scale the correction back.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>

#include "double_float.cuh"
#include "factor_apply.cuh"
#include "grid_sync.cuh"
#include "internal.h"

namespace mfem {
namespace {

constexpr int kIrThreads = 512;
constexpr int kIrGroup = 4;  // lanes per block row in the product
constexpr int kIrDepth = 4;  // blocks per lane and loop trip in the product
constexpr int kResThreads = 256;
constexpr long long kIrWaitCycles = 8000000000ll;

template <class T>
__device__ __forceinline__ T to_lowp(float v);
template <>
__device__ __forceinline__ __nv_bfloat16 to_lowp<__nv_bfloat16>(float v) {
    return __float2bfloat16_rn(v);
}
template <>
__device__ __forceinline__ __half to_lowp<__half>(float v) {
    return __float2half_rn(v);
}
__device__ __forceinline__ float from_lowp(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float from_lowp(__half v) { return __half2float(v); }

template <class T>
__global__ void ir_convert_kernel(BsrViews bv, IrWork w) {
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= bv.n) return;
    const int kb = bv.row_ptr[row], ke = bv.row_ptr[row + 1];
    float m = 0.0f;
    for (int k = kb + lane; k < ke; k += 32)
#pragma unroll
        for (int i = 0; i < 9; ++i) m = fmaxf(m, fabsf(bv.values[(size_t)9 * k + i]));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    const float s = (m > 0.0f && isfinite(m)) ? m : 1.0f;
    if (lane == 0) w.row_scale[row] = s;
    const float inv = 1.0f / s;
    T *q = reinterpret_cast<T *>(w.lowp);
    for (int k = kb + lane; k < ke; k += 32) {
        unsigned short bits[10];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const T v = to_lowp<T>(bv.values[(size_t)9 * k + i] * inv);
            q[(size_t)9 * k + i] = v;
            memcpy(&bits[i], &v, 2);
        }
        bits[9] = 0;
        if (w.hq_words)  // the persistent factor PCG's copy: five words a block
#pragma unroll
            for (int i = 0; i < 5; ++i)
                w.hq_words[(size_t)5 * k + i] = (uint32_t)bits[2 * i] | ((uint32_t)bits[2 * i + 1] << 16);
    }
}

__global__ void ir_begin_kernel(VertexViews vv, IrWork w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 3 * vv.n) {
        w.dx_pair[i] = make_float2(vv.dx[i], 0.0f);
        w.dx_init[i] = vv.dx[i];
    }
    if (i == 0) {
        w.state[6] = w.mode == kIrFp32 ? 1 : 0;  // inner PCG on the fp32 H
        w.state[7] = 0;  // restart from the warm start at the next residual
        *w.best = __longlong_as_double(0x7ff0000000000000ll);  // +inf
        w.state[0] = 0;  // done
        w.state[1] = 0;  // outer iterations
        w.state[2] = 0;  // inner iterations
        w.state[3] = 0;  // an inner correction is pending
        w.state[4] = 0;  // dx buffer parity
        w.state[5] = MFEM_OK;
    }
}

__global__ void __launch_bounds__(kResThreads)
    ir_residual_kernel(BsrViews bv, VertexViews vv, IrWork w, PcgWork pw, int slot) {
    __shared__ double s_red[2][kResThreads / 32];
    __shared__ int s_last;
    if (*(volatile int *)&w.state[0]) return;  // converged or capped
    const int par = w.state[4];
    const bool restart = w.state[7] != 0;
    const bool pending = !restart && w.state[3] != 0;
    const size_t vec = (size_t)3 * vv.n;
    const float2 *xo = w.dx_pair + (size_t)par * vec;
    float2 *xn = w.dx_pair + (size_t)(par ^ 1) * vec;
    const int g_lane = threadIdx.x & (kIrGroup - 1);
    const unsigned gmask = ((1u << kIrGroup) - 1u) << (threadIdx.x & (32 - kIrGroup));
    const int row = (blockIdx.x * blockDim.x + threadIdx.x) / kIrGroup;
    // the iterate of row c: the warm start after a restart, else the last
    // iterate plus the pending inner correction
    auto iterate = [&](int c, int q) -> float2 {
        if (restart) return make_float2(w.dx_init[3 * c + q], 0.0f);
        const float2 x = xo[3 * c + q];
        return pending ? df_add(x, w.e[3 * c + q]) : x;
    };
    double rr = 0.0, gg = 0.0;
    if (row < vv.n) {
        float2 acc[3] = {make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f), make_float2(0.0f, 0.0f)};
        for (int k = bv.row_ptr[row] + g_lane; k < bv.row_ptr[row + 1]; k += kIrGroup) {
            const int c = bv.col_idx[k];
            float2 xc[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) xc[q] = iterate(c, q);
            const float *h = bv.values + (size_t)9 * k;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int q = 0; q < 3; ++q) df_fma(acc[a], h[3 * a + q], xc[q]);
        }
#pragma unroll
        for (int off = kIrGroup / 2; off > 0; off >>= 1)
#pragma unroll
            for (int a = 0; a < 3; ++a) acc[a] = df_add(acc[a], df_shfl_xor(gmask, acc[a], off));
        if (g_lane == 0) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float2 xr = iterate(row, a);
                xn[3 * row + a] = xr;
                w.dx_out[3 * row + a] = (double)xr.x + (double)xr.y;
                vv.dx[3 * row + a] = __fadd_rn(xr.x, xr.y);
                // r = g - (acc.hi + acc.lo), as a pair, then its double value
                const float gq = vv.rhs[3 * row + a];
                const double r = df_residual(gq, acc[a]);
                w.res[3 * row + a] = (float)r;
                rr += r * r;
                gg += (double)gq * (double)gq;
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rr += __shfl_down_sync(0xffffffffu, rr, off);
        gg += __shfl_down_sync(0xffffffffu, gg, off);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        s_red[0][wid] = rr;
        s_red[1][wid] = gg;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a0 = 0.0, a1 = 0.0;
        for (int k = 0; k < kResThreads / 32; ++k) {
            a0 += s_red[0][k];
            a1 += s_red[1][k];
        }
        w.res_partials[2 * blockIdx.x + 0] = a0;
        w.res_partials[2 * blockIdx.x + 1] = a1;
        __threadfence();
        s_last = atomicAdd(w.ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last) return;
    // the last block: fixed-order totals and the decision
    if (threadIdx.x == 0) {
        __threadfence();
        double trr = 0.0, tgg = 0.0;
        for (int b = 0; b < (int)gridDim.x; ++b) {
            trr += __ldcg(w.res_partials + 2 * b);
            tgg += __ldcg(w.res_partials + 2 * b + 1);
        }
        const double rel = tgg > 0.0 ? sqrt(trr / tgg) : sqrt(trr);
        // the scale of the next inner right-hand side (unit norm: fp32 sums
        // of products of a tiny residual's entries would underflow)
        const double rn = sqrt(trr);
        const float inv = (float)(1.0 / rn);
        const bool scaled = rn > 0.0 && isfinite(rn) && isfinite(inv);
        w.scale[0] = scaled ? inv : 1.0f;
        w.scale[1] = scaled ? (float)rn : 1.0f;
        const int outer = w.state[1];
        int status = MFEM_OK;
        int done = 0;
        const double best = *w.best;
        w.state[7] = 0;
        if (w.state[6] == 0 && isfinite(best) && !(rel <= 4.0 * best) && outer < w.outer_max) {
            // diverging on the 16-bit H: restart from the warm start with
            // the fp32 H (the next inner PCG is skipped; the next residual
            // pass reads the warm start)
            w.state[6] = 1;
            w.state[7] = 1;
        } else if (!isfinite(rel)) {
            status = MFEM_NONFINITE;
            done = 1;
        } else if (rel <= w.outer_tol) {
            done = 1;
        } else if (outer >= w.outer_max) {
            status = MFEM_MAXITER;
            done = 1;
        }
        if (isfinite(rel) && rel < best && w.state[7] == 0) *w.best = rel;
        w.state[1] = outer + 1;
        w.state[3] = 0;
        w.state[4] = par ^ 1;
        w.state[0] = done;
        if (w.state[5] == MFEM_OK) w.state[5] = status;
        w.stats[slot] = IrStats{outer, w.state[2], w.state[5], w.state[6], rel};
        pw.stats[slot] = SolveStats{w.state[2], w.state[5], (float)rel, 0.0f};
        *w.ticket = 0u;
    }
}

__device__ __forceinline__ unsigned long long ir_ld_relaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Block-reduce NV partials, store them for barrier k, wait at the grid
// barrier, sum all CTAs' partials in a fixed order into tot[].  In fp64:
// the inner right-hand side is a residual that can be tiny, and fp32
// products of its entries would underflow (0/0 in the recurrence).
template <int NV>
__device__ bool ir_reduce(double (&v)[NV], const IrWork &w, int *error, unsigned k, unsigned long long &target,
                          double *tot, double (*s_redf)[32], double *s_val, int *s_ok) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nb = gridDim.x;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) s_redf[i][wid] = v[i];
    __syncthreads();
    double *buf = w.partials + (size_t)(k & 1u) * 256 * 4;
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        double part[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            part[i] = lane < nw ? s_redf[i][lane] : 0.0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) part[i] += __shfl_down_sync(0xffffffffu, part[i], off);
        }
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < NV; ++i) buf[(size_t)blockIdx.x * 4 + i] = part[i];
            target += nb;
            grid_arrive(w.counter);
            int ok = 1;
            const long long t0 = clock64();
            unsigned spins = 0;
            while (grid_count(w.counter) < target) {
                if ((++spins & 1023u) == 0 && (*(const volatile int *)error != 0 || clock64() - t0 > kIrWaitCycles)) {
                    atomicExch(error, 1);
                    ok = 0;
                    break;
                }
            }
            *s_ok = ok;
        }
    }
    __syncthreads();
    if (!*s_ok) return false;
    for (int t = threadIdx.x; t < nb * NV; t += blockDim.x) {
        const int b = t / NV, i = t - b * NV;
        s_val[b * 4 + i] = __ldcg(buf + (size_t)b * 4 + i);
    }
    __syncthreads();
    if (wid == 0) {
        double acc[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) acc[i] = 0.0;
        for (int b = lane; b < nb; b += 32)
#pragma unroll
            for (int i = 0; i < NV; ++i) acc[i] += s_val[b * 4 + i];
#pragma unroll
        for (int i = 0; i < NV; ++i)
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], off);
        if (lane == 0)
#pragma unroll
            for (int i = 0; i < NV; ++i) tot[i] = acc[i];
    }
    __syncthreads();
    return true;
}

__device__ __forceinline__ void ir_precond(const float *Minv, int use, int row, const float r[3], float z[3]) {
    if (!use) {
        z[0] = r[0];
        z[1] = r[1];
        z[2] = r[2];
        return;
    }
    const float *m = Minv + (size_t)9 * row;
    z[0] = m[0] * r[0] + m[1] * r[1] + m[2] * r[2];
    z[1] = m[3] * r[0] + m[4] * r[1] + m[5] * r[2];
    z[2] = m[6] * r[0] + m[7] * r[1] + m[8] * r[2];
}

// z = M r over this CTA's rows with the plan's factor (every row's r is in
// place on entry): the first pass into fb.y, a grid barrier, the second into
// w.z; z of the CTA's own rows on return.
__device__ __forceinline__ bool ir_apply_factor(const BatchViews &fb, int mode, const IrWork &w, int *error,
                                                unsigned &k, unsigned long long &target, double *s_tot,
                                                double (*s_redf)[32], double *s_val, int *s_ok, int lo, int hi) {
    const FactorForms f = factor_forms(fb, mode);
    factor_pass<false, kIrGroup>(f.rp0, f.c0, f.v0, w.r, fb.y, lo, hi);
    double d[1] = {0.0};
    if (!ir_reduce<1>(d, w, error, k++, target, s_tot, s_redf, s_val, s_ok)) return false;
    factor_pass<false, kIrGroup>(f.rp1, f.c1, f.v1, fb.y, w.z, lo, hi);
    __syncthreads();
    return true;
}

// y_row = s_row sum_k Hq[k] (z[col] + beta p_old[col]), fp32 accumulation;
// with `full`, the fp32 H instead (after a restart).
template <class T>
__device__ __forceinline__ void ir_row_product(const BsrViews &bv, const IrWork &w, int row, const float *z,
                                               const float *p_old, float beta, bool full, float y[3]) {
    const int g_lane = threadIdx.x & (kIrGroup - 1);
    const unsigned gmask = ((1u << kIrGroup) - 1u) << (threadIdx.x & (32 - kIrGroup));
    const int kb = bv.row_ptr[row], ke = bv.row_ptr[row + 1];
    const T *q = reinterpret_cast<const T *>(w.lowp);
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
    // kIrDepth blocks per lane and trip: their loads are in flight together
    for (int k = kb + g_lane; k < ke; k += kIrDepth * kIrGroup) {
        int kk[kIrDepth], cc[kIrDepth];
        bool ok[kIrDepth];
#pragma unroll
        for (int u = 0; u < kIrDepth; ++u) {
            ok[u] = k + u * kIrGroup < ke;
            kk[u] = ok[u] ? k + u * kIrGroup : k;
            cc[u] = __ldg(bv.col_idx + kk[u]);
        }
        float v[kIrDepth][3];
#pragma unroll
        for (int u = 0; u < kIrDepth; ++u)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float zc = __ldcg(z + 3 * cc[u] + i);
                v[u][i] = p_old ? __fmaf_rn(beta, __ldcg(p_old + 3 * cc[u] + i), zc) : zc;
                if (!ok[u]) v[u][i] = 0.0f;
            }
#pragma unroll
        for (int u = 0; u < kIrDepth; ++u) {
            if (full) {
                const float *h = bv.values + (size_t)9 * kk[u];
                a0 += __ldg(h + 0) * v[u][0] + __ldg(h + 1) * v[u][1] + __ldg(h + 2) * v[u][2];
                a1 += __ldg(h + 3) * v[u][0] + __ldg(h + 4) * v[u][1] + __ldg(h + 5) * v[u][2];
                a2 += __ldg(h + 6) * v[u][0] + __ldg(h + 7) * v[u][1] + __ldg(h + 8) * v[u][2];
            } else {
                const T *h = q + (size_t)9 * kk[u];
                a0 += from_lowp(h[0]) * v[u][0] + from_lowp(h[1]) * v[u][1] + from_lowp(h[2]) * v[u][2];
                a1 += from_lowp(h[3]) * v[u][0] + from_lowp(h[4]) * v[u][1] + from_lowp(h[5]) * v[u][2];
                a2 += from_lowp(h[6]) * v[u][0] + from_lowp(h[7]) * v[u][1] + from_lowp(h[8]) * v[u][2];
            }
        }
    }
#pragma unroll
    for (int off = kIrGroup / 2; off > 0; off >>= 1) {
        a0 += __shfl_xor_sync(gmask, a0, off);
        a1 += __shfl_xor_sync(gmask, a1, off);
        a2 += __shfl_xor_sync(gmask, a2, off);
    }
    const float s = full ? 1.0f : w.row_scale[row];
    y[0] = s * a0;
    y[1] = s * a1;
    y[2] = s * a2;
}

struct IrScalars {
    double alpha, beta, rz, thr2;
    int status, done;
};

// FACTOR: the instantiation for the factor preconditioners (use_precond 2
// or 3: M r = F^T (F r) or F (F^T r) from the plan's factor fb, two more grid
// barriers per iteration; an inner solve that breaks down is restarted from
// e = 0 with block-Jacobi).
template <class T, bool FACTOR>
__global__ void __launch_bounds__(kIrThreads, 1)
    ir_pcg_kernel(BsrViews bv, VertexViews vv, IrWork w, BatchViews fb, int *error, int maxiter, int use_precond) {
    __shared__ double s_redf[3][32];
    __shared__ double s_val[4 * 256];
    __shared__ double s_tot[3];
    __shared__ IrScalars sc;
    __shared__ int s_ok;
    __shared__ unsigned long long s_base;
    if (*(volatile int *)&w.state[0]) return;  // the outer loop has finished
    if (*(volatile int *)&w.state[7]) return;  // a restart: no correction this round
    const bool full = *(volatile int *)&w.state[6] != 0;  // the fp32 H
    const int n = vv.n, nb = gridDim.x, cta = blockIdx.x;
    const int lo = (int)(((long long)n * cta) / nb), hi = (int)(((long long)n * (cta + 1)) / nb);
    const int group = threadIdx.x / kIrGroup, ngroups = blockDim.x / kIrGroup;
    const bool g_lead = (threadIdx.x & (kIrGroup - 1)) == 0;
    if (threadIdx.x == 0) {
        s_base = (ir_ld_relaxed(w.counter) / nb) * (unsigned long long)nb;
        s_ok = *(const volatile int *)error == 0;
    }
    __syncthreads();
    if (!s_ok) {
        if (cta == 0 && threadIdx.x == 0) {
            w.state[5] = MFEM_TIMEOUT;
            w.state[0] = 1;
        }
        return;
    }
    unsigned long long target = s_base;
    unsigned k = 0;
    int it = 0;
    int mode = use_precond, it_done = 0;
    bool timed_out = false;
    for (;;) {  // one attempt; a factor solve that breaks down restarts with block-Jacobi
        const bool factor = FACTOR && mode >= 2;
        it = 0;
        // e0 = 0: r = rhs, z = M r
        double acc3[3] = {0.0, 0.0, 0.0};
        for (int row = lo + threadIdx.x; row < hi; row += blockDim.x) {
            float r[3], z[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                r[q] = w.res[3 * row + q];
                w.e[3 * row + q] = 0.0f;
                w.r[3 * row + q] = r[q];
            }
            if (factor) continue;  // z comes from the factor passes below
            ir_precond(vv.Minv, mode, row, r, z);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                w.z[3 * row + q] = z[q];
                acc3[0] = fma((double)r[q], (double)z[q], acc3[0]);
                acc3[1] = fma((double)r[q], (double)r[q], acc3[1]);
            }
        }
        if (factor) {
            // every row's r in place, then z = M r, then (r, z) and (r, r)
            double d[1] = {0.0};
            if (!ir_reduce<1>(d, w, error, k++, target, s_tot, s_redf, s_val, &s_ok) ||
                !ir_apply_factor(fb, mode, w, error, k, target, s_tot, s_redf, s_val, &s_ok, lo, hi)) {
                timed_out = true;
                break;
            }
            for (int row = lo + threadIdx.x; row < hi; row += blockDim.x)
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const float rq = w.r[3 * row + q], zq = w.z[3 * row + q];
                    acc3[0] = fma((double)rq, (double)zq, acc3[0]);
                    acc3[1] = fma((double)rq, (double)rq, acc3[1]);
                }
        }
        acc3[2] = acc3[1];  // ||rhs||^2 = ||r0||^2
        bool ok = ir_reduce<3>(acc3, w, error, k++, target, s_tot, s_redf, s_val, &s_ok);
        if (threadIdx.x == 0) {
            if (!ok) {
                sc.status = MFEM_TIMEOUT;
                sc.done = 1;
            } else {
                sc.rz = s_tot[0];
                sc.thr2 = w.inner_tol * w.inner_tol * s_tot[2];
                sc.beta = 0.0;
                sc.status = (isfinite(s_tot[0]) && isfinite(s_tot[1])) ? MFEM_OK : MFEM_NONFINITE;
                sc.done = sc.status != MFEM_OK || s_tot[1] <= sc.thr2;
            }
        }
        __syncthreads();
        while (!sc.done) {
            if (it >= maxiter) break;
            float *p_new = (it & 1) ? w.p1 : w.p0;
            const float *p_old = it == 0 ? nullptr : ((it & 1) ? w.p0 : w.p1);
            const float beta = (float)sc.beta;
            double pap[1] = {0.0};
            for (int row = lo + group; row < hi; row += ngroups) {
                float y[3];
                ir_row_product<T>(bv, w, row, w.z, p_old, beta, full, y);
                if (g_lead) {
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        const float zq = __ldcg(w.z + 3 * row + q);
                        const float pq = p_old ? __fmaf_rn(beta, __ldcg(p_old + 3 * row + q), zq) : zq;
                        p_new[3 * row + q] = pq;
                        w.Ap[3 * row + q] = y[q];
                        pap[0] = fma((double)pq, (double)y[q], pap[0]);
                    }
                }
            }
            if (!ir_reduce<1>(pap, w, error, k++, target, s_tot, s_redf, s_val, &s_ok)) {
                if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
                break;
            }
            if (threadIdx.x == 0) {
                if (!isfinite(s_tot[0])) {
                    sc.status = MFEM_NONFINITE;
                    sc.done = 1;
                } else if (!(s_tot[0] > 0.0)) {
                    sc.status = MFEM_STAGNATION;
                    sc.done = 1;
                } else {
                    sc.alpha = sc.rz / s_tot[0];
                }
            }
            __syncthreads();
            if (sc.done) break;
            const float alpha = (float)sc.alpha;
            double acc2[2] = {0.0, 0.0};
            if (factor) {
                for (int row = lo + threadIdx.x; row < hi; row += blockDim.x)
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        w.e[3 * row + q] = __fmaf_rn(alpha, p_new[3 * row + q], w.e[3 * row + q]);
                        w.r[3 * row + q] = __fmaf_rn(-alpha, w.Ap[3 * row + q], w.r[3 * row + q]);
                    }
                double d[1] = {0.0};
                if (!ir_reduce<1>(d, w, error, k++, target, s_tot, s_redf, s_val, &s_ok) ||
                    !ir_apply_factor(fb, mode, w, error, k, target, s_tot, s_redf, s_val, &s_ok, lo, hi)) {
                    if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
                    break;
                }
            }
            for (int row = lo + threadIdx.x; row < hi; row += blockDim.x) {
                float r[3], z[3];
                if (factor) {
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        r[q] = w.r[3 * row + q];
                        z[q] = w.z[3 * row + q];
                    }
                } else {
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        w.e[3 * row + q] = __fmaf_rn(alpha, p_new[3 * row + q], w.e[3 * row + q]);
                        r[q] = __fmaf_rn(-alpha, w.Ap[3 * row + q], w.r[3 * row + q]);
                        w.r[3 * row + q] = r[q];
                    }
                    ir_precond(vv.Minv, mode, row, r, z);
                }
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    w.z[3 * row + q] = z[q];
                    acc2[0] = fma((double)r[q], (double)z[q], acc2[0]);
                    acc2[1] = fma((double)r[q], (double)r[q], acc2[1]);
                }
            }
            if (!ir_reduce<2>(acc2, w, error, k++, target, s_tot, s_redf, s_val, &s_ok)) {
                if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
                break;
            }
            ++it;
            if (threadIdx.x == 0) {
                if (!isfinite(s_tot[0]) || !isfinite(s_tot[1])) {
                    sc.status = MFEM_NONFINITE;
                    sc.done = 1;
                } else {
                    sc.beta = s_tot[0] / sc.rz;
                    sc.rz = s_tot[0];
                    sc.done = s_tot[1] <= sc.thr2;
                }
            }
            __syncthreads();
        }
        if (FACTOR && mode >= 2 && (sc.status == MFEM_STAGNATION || sc.status == MFEM_NONFINITE)) {
            // no barrier needed: the restart writes e = 0 and r = rhs for
            // its own rows before its first grid barrier
            it_done += it;
            mode = 1;
            __syncthreads();
            continue;
        }
        break;
    }
    if (timed_out && threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
    it += it_done;
    if (cta == 0 && threadIdx.x == 0) {
        // the outer loop adds the correction at its next residual; a broken
        // inner solve still hands over its iterate, as the reference's CG does
        w.state[2] += it;
        w.state[3] = 1;
        if (sc.status == MFEM_NONFINITE && !full) {
            // the 16-bit H broke the inner solve: restart on the fp32 H
            w.state[3] = 0;
            w.state[6] = 1;
            w.state[7] = 1;
        } else if (sc.status == MFEM_TIMEOUT || sc.status == MFEM_NONFINITE) {
            w.state[5] = sc.status;
            w.state[0] = 1;
        }
    }
}

inline int blocks_for(int n, int threads) { return (n + threads - 1) / threads; }

template <class T>
cudaError_t launch_ir_pcg(const BsrViews &bv, const VertexViews &vv, const IrWork &w, const BatchViews &fb,
                          int *error, int maxiter, int use_precond, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(w.ctas);
    cfg.blockDim = dim3(kIrThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = use_precond >= 2
                        ? cudaLaunchKernelEx(&cfg, ir_pcg_kernel<T, true>, bv, vv, w, fb, error, maxiter, use_precond)
                        : cudaLaunchKernelEx(&cfg, ir_pcg_kernel<T, false>, bv, vv, w, fb, error, maxiter,
                                             use_precond);
    count_launches(1);
    return e;
}

}  // namespace

cudaError_t ir_max_ctas(int device, int *ctas) {
    int sms = 0, occ = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    // the smallest residency of the four instantiations
    occ = 1 << 30;
    auto take = [&](const void *fn) {
        int o = 0;
        if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, kIrThreads, 0);
        occ = std::min(occ, o);
    };
    take((const void *)ir_pcg_kernel<__half, false>);
    take((const void *)ir_pcg_kernel<__half, true>);
    take((const void *)ir_pcg_kernel<__nv_bfloat16, false>);
    take((const void *)ir_pcg_kernel<__nv_bfloat16, true>);
    if (e != cudaSuccess) return e;
    *ctas = std::max(1, std::min(256, sms * std::max(1, occ)));
    return cudaSuccess;
}

int ir_residual_blocks(int n) { return std::max(1, blocks_for(n * kIrGroup, kResThreads)); }

cudaError_t launch_mixed_solve(const BsrViews &bv, const VertexViews &vv, const IrWork &w, const PcgWork &pw,
                               const BatchViews &fb, const PcgLayout &pl, const PcgLayout *single, int pcg_ctas,
                               int slot, int maxiter, int use_precond, cudaStream_t s) {
    if (bv.n == 0) return cudaSuccess;
    const bool bf16 = w.mode == kIrBf16;
    const bool fp32 = w.mode == kIrFp32;  // the inner PCG reads the fp32 H itself
    cudaError_t e;
    const int rows_per_block = 256 / 32;
    if (bf16) ir_convert_kernel<__nv_bfloat16><<<blocks_for(bv.n, rows_per_block), 256, 0, s>>>(bv, w);
    else if (!fp32) ir_convert_kernel<__half><<<blocks_for(bv.n, rows_per_block), 256, 0, s>>>(bv, w);
    ir_begin_kernel<<<blocks_for(3 * vv.n, 256), 256, 0, s>>>(vv, w);
    count_launches(fp32 ? 1 : 2);
    e = cudaGetLastError();
    // block-Jacobi on the fp32 H: the one-barrier single-reduction PCG for
    // the inner solves (4.8 us an iteration on nh_beam against the factor
    // kernel's two barriers), a launch per correction
    const bool single_inner = fp32 && use_precond == 1 && single && single->variant == PcgLayout::kSingleReduction;
    if (e == cudaSuccess && !single_inner && w.xf_hi && (w.hq_words || fp32) && pl.variant == PcgLayout::kFactor)
        // every correction inside one launch of the persistent factor PCG
        return launch_pcg_factor_refine(bv, vv, w, pw, fb, pl, pcg_ctas, slot, maxiter, use_precond, s);
    const int rb = ir_residual_blocks(vv.n);
    for (int k = 0; e == cudaSuccess && k < w.outer_max; ++k) {
        ir_residual_kernel<<<rb, kResThreads, 0, s>>>(bv, vv, w, pw, slot);
        count_launches(1);
        e = cudaGetLastError();
        if (e == cudaSuccess && single_inner)
            e = launch_pcg_inner(bv, vv, w, pw, *single, pcg_ctas, slot, maxiter, s);
        else if (e == cudaSuccess && (w.hq_words || fp32) && pl.variant == PcgLayout::kFactor)
            e = launch_pcg_factor_inner(bv, vv, w, pw, fb, pl, pcg_ctas, slot, maxiter, use_precond, s);
        else if (e == cudaSuccess)
            e = bf16 ? launch_ir_pcg<__nv_bfloat16>(bv, vv, w, fb, pw.error, maxiter, use_precond, s)
                     : launch_ir_pcg<__half>(bv, vv, w, fb, pw.error, maxiter, use_precond, s);
    }
    if (e == cudaSuccess) {
        // the last correction and the final fp64 residual
        ir_residual_kernel<<<rb, kResThreads, 0, s>>>(bv, vv, w, pw, slot);
        count_launches(1);
        e = cudaGetLastError();
    }
    return e;
}

}  // namespace mfem
