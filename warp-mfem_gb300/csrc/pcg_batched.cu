// Block-Jacobi PCG for many independent bodies in one persistent launch.
//
// The bodies share one plan: their meshes are concatenated (vertices and
// tets of body b are contiguous) so every other kernel of the step runs on
// the union unchanged, and the global system is block-diagonal by body.  The
// solve, however, is one PCG per body, each with its own alpha, beta and
// stopping test ||r_b|| <= tol ||g_b|| -- the reference's step run on each
// body separately.
//
// Each CTA works through a list of tasks.  A task is one body's PCG on a
// group of CTAs: a body small enough for one CTA is solved by it alone, with
// __syncthreads as its only barrier (several such bodies may follow each
// other on one CTA); a larger body gets a group of CTAs that split its rows
// and meet at a counter barrier of their own.  The host scheduler (api.cu)
// sizes the groups by the bodies' block counts.
//
// The iteration is the standard one of the reference's CG (two reductions:
// p.Ap, then (r, z) and (r, r)); rows gather the vectors of other rows from
// global memory (L2); sums are fixed-order, so results are deterministic for
// a given schedule.  Every wait is bounded.
#include <algorithm>

#include "block_loads.cuh"
#include "factor_apply.cuh"
#include "grid_sync.cuh"
#include "internal.h"

namespace mfem {
namespace {

constexpr int kBtGroup = 4;  // lanes per block row in the product
constexpr long long kBtWaitCycles = 8000000000ll;

__device__ __forceinline__ unsigned long long bt_ld_relaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

struct Task {
    int body, rank, size, first;
};

// Block-reduce NV partials; for a group of several CTAs also store them for
// barrier k, wait at the group's barrier and add all group partials in a
// fixed order.  tot[] is valid for every thread on return.
template <int NV>
__device__ bool bt_reduce(float (&v)[NV], const BatchViews &bw, const Task &tk, int *error, unsigned k,
                          unsigned long long &target, float *tot, float (*s_redf)[32], int *s_ok) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) s_redf[i][wid] = v[i];
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
        if (tk.size == 1) {
            if (lane == 0)
#pragma unroll
                for (int i = 0; i < NV; ++i) tot[i] = part[i];
        } else {
            float *buf = bw.partials + (size_t)(k & 1u) * bw.ctas * 4;
            if (lane == 0) {
#pragma unroll
                for (int i = 0; i < NV; ++i) buf[(size_t)(tk.first + tk.rank) * 4 + i] = part[i];
                target += tk.size;
                grid_arrive(bw.counter + tk.body);
                int ok = 1;
                const long long t0 = clock64();
                unsigned spins = 0;
                while (grid_count(bw.counter + tk.body) < target) {
                    if ((++spins & 1023u) == 0 &&
                        (*(const volatile int *)error != 0 || clock64() - t0 > kBtWaitCycles)) {
                        atomicExch(error, 1);
                        ok = 0;
                        break;
                    }
                }
                *s_ok = ok;
            }
            __syncwarp();
            // the group's partials in a fixed order (lane-strided, then a tree)
            const int ok = __shfl_sync(0xffffffffu, *s_ok, 0);
            float acc[NV];
#pragma unroll
            for (int i = 0; i < NV; ++i) acc[i] = 0.0f;
            if (ok)
                for (int b = lane; b < tk.size; b += 32)
#pragma unroll
                    for (int i = 0; i < NV; ++i) acc[i] += __ldcg(buf + (size_t)(tk.first + b) * 4 + i);
#pragma unroll
            for (int i = 0; i < NV; ++i)
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], off);
            if (lane == 0)
#pragma unroll
                for (int i = 0; i < NV; ++i) tot[i] = acc[i];
        }
    }
    __syncthreads();
    return tk.size == 1 || *s_ok != 0;
}

__device__ __forceinline__ void bt_precond(const float *Minv, int use, int row, const float r[3], float z[3]) {
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

// Loads of vectors other threads wrote during this launch: from L2 when a
// group of CTAs shares them, through L1 when one CTA owns the whole body
// (its own stores, ordered by __syncthreads).
template <bool SHARED>
__device__ __forceinline__ float bt_ld(const float *p) {
    return SHARED ? __ldcg(p) : *p;
}

// y = sum_k H[k] (z[col] + beta p_old[col]) for one row, kBtGroup lanes.
template <bool SHARED>
__device__ __forceinline__ void bt_row_product(const BsrViews &bv, int row, const float *z, const float *p_old,
                                               float beta, float y[3]) {
    const int g_lane = threadIdx.x & (kBtGroup - 1);
    const unsigned gmask = ((1u << kBtGroup) - 1u) << (threadIdx.x & (32 - kBtGroup));
    const int kb = bv.row_ptr[row], ke = bv.row_ptr[row + 1];
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
    // two blocks per lane and trip: their loads are in flight together
    for (int k = kb + g_lane; k < ke; k += 2 * kBtGroup) {
        const int k2 = k + kBtGroup;
        const bool two = k2 < ke;
        const int c = __ldg(bv.col_idx + k), c2 = two ? __ldg(bv.col_idx + k2) : c;
        float v[3], v2[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float zc = bt_ld<SHARED>(z + 3 * c + q), zc2 = bt_ld<SHARED>(z + 3 * c2 + q);
            v[q] = p_old ? __fmaf_rn(beta, bt_ld<SHARED>(p_old + 3 * c + q), zc) : zc;
            v2[q] = p_old ? __fmaf_rn(beta, bt_ld<SHARED>(p_old + 3 * c2 + q), zc2) : zc2;
        }
        if (!two) v2[0] = v2[1] = v2[2] = 0.0f;
        float h[9], h2[9];
        load_block9(bv.values, k, h);
        load_block9(bv.values, two ? k2 : k, h2);
        a0 += h[0] * v[0] + h[1] * v[1] + h[2] * v[2];
        a1 += h[3] * v[0] + h[4] * v[1] + h[5] * v[2];
        a2 += h[6] * v[0] + h[7] * v[1] + h[8] * v[2];
        a0 += h2[0] * v2[0] + h2[1] * v2[1] + h2[2] * v2[2];
        a1 += h2[3] * v2[0] + h2[4] * v2[1] + h2[5] * v2[2];
        a2 += h2[6] * v2[0] + h2[7] * v2[1] + h2[8] * v2[2];
    }
#pragma unroll
    for (int off = kBtGroup / 2; off > 0; off >>= 1) {
        a0 += __shfl_xor_sync(gmask, a0, off);
        a1 += __shfl_xor_sync(gmask, a1, off);
        a2 += __shfl_xor_sync(gmask, a2, off);
    }
    y[0] = a0;
    y[1] = a1;
    y[2] = a2;
}

// The barrier of the body between factor passes and before reading vectors
// other CTAs of the group wrote: __syncthreads for a one-CTA body, the
// group's counter barrier otherwise.
__device__ __forceinline__ bool bt_sync(const BatchViews &bw, const Task &tk, int *error, unsigned &k,
                                        unsigned long long &target, float *s_tot, float (*s_redf)[32], int *s_ok) {
    if (tk.size == 1) {
        __syncthreads();
        return true;
    }
    float d[1] = {0.0f};
    return bt_reduce<1>(d, bw, tk, error, k++, target, s_tot, s_redf, s_ok);
}

// z = M r for the CTA's rows with a factor preconditioner: M = F^T F
// (mode 2: y = F r, z = F^T y) or M = F F^T (mode 3: y = F^T r, z = F y).
// r of every row of the body is in place on entry (after a barrier); z of
// the CTA's own rows on return.
__device__ __forceinline__ bool bt_apply_factor(const BatchViews &bw, int mode, const Task &tk, int lo, int hi,
                                                int *error, unsigned &k, unsigned long long &target, float *s_tot,
                                                float (*s_redf)[32], int *s_ok) {
    const FactorForms f = factor_forms(bw, mode);
    if (tk.size > 1) factor_pass<false, kBtGroup>(f.rp0, f.c0, f.v0, bw.r, bw.y, lo, hi);
    else factor_pass<true, kBtGroup>(f.rp0, f.c0, f.v0, bw.r, bw.y, lo, hi);
    if (!bt_sync(bw, tk, error, k, target, s_tot, s_redf, s_ok)) return false;
    if (tk.size > 1) factor_pass<false, kBtGroup>(f.rp1, f.c1, f.v1, bw.y, bw.z, lo, hi);
    else factor_pass<true, kBtGroup>(f.rp1, f.c1, f.v1, bw.y, bw.z, lo, hi);
    __syncthreads();
    return true;
}

struct BtScalars {
    float alpha, beta, rz, rr, bb, thr2;
    int status, done;
};

// FACTOR: the instantiation for the factor preconditioners (use_precond 2
// or 3, with the block-Jacobi retry); the other one, for use_precond 0 or 1,
// carries none of that code.  Register caps (no spills at either): 48 lets
// 10 CTAs of 128 threads share an SM, 56 lets 9 (the kernel waits on gather
// latency, so resident warps matter); up to 512 threads a CTA (the host's
// schedules use 128 to 512).
template <bool FACTOR>
__global__ void __maxnreg__(FACTOR ? 56 : 48)
    batched_pcg_kernel(BsrViews bv, VertexViews vv, BatchViews bw, int *error, int slot, float tol, int maxiter,
                       int use_precond) {
    __shared__ float s_redf[3][32];
    __shared__ float s_tot[3];
    __shared__ BtScalars sc;
    __shared__ int s_ok;
    __shared__ unsigned long long s_base;
    const int group = threadIdx.x / kBtGroup, ngroups = blockDim.x / kBtGroup;
    const bool g_lead = (threadIdx.x & (kBtGroup - 1)) == 0;
    for (int ti = bw.task_ptr[blockIdx.x]; ti < bw.task_ptr[blockIdx.x + 1]; ++ti) {
        const int4 t4 = bw.task[ti];
        const Task tk{t4.x, t4.y, t4.z, t4.w};
        const int b0 = bw.body_row[tk.body], b1 = bw.body_row[tk.body + 1];
        const int lo = b0 + (int)(((long long)(b1 - b0) * tk.rank) / tk.size);
        const int hi = b0 + (int)(((long long)(b1 - b0) * (tk.rank + 1)) / tk.size);
        if (threadIdx.x == 0) {
            s_base = tk.size > 1 ? (bt_ld_relaxed(bw.counter + tk.body) / tk.size) * (unsigned long long)tk.size : 0;
            s_ok = *(const volatile int *)error == 0;
        }
        __syncthreads();
        SolveStats *st = bw.stats + (size_t)slot * bw.n_bodies + tk.body;
        if (!s_ok) {
            if (tk.rank == 0 && threadIdx.x == 0) *st = SolveStats{0, MFEM_TIMEOUT, 0.0f, 0.0f};
            continue;
        }
        unsigned long long target = s_base;
        unsigned k = 0;
        int mode = use_precond, it = 0, it_done = 0;
        bool timed_out = false;
        if (FACTOR && mode >= 2)  // the warm start, for a block-Jacobi retry
            for (int t3 = 3 * lo + threadIdx.x; t3 < 3 * hi; t3 += blockDim.x) bw.dx0[t3] = vv.dx[t3];
        for (;;) {  // one attempt; a factor solve that breaks down is retried with block-Jacobi
            it = 0;
            // r = g - H x0 (x0: the warm start x~ - x), z = M r
            for (int row = lo + group; row < hi; row += ngroups) {
                float y[3];
                if (tk.size > 1) bt_row_product<true>(bv, row, vv.dx, nullptr, 0.0f, y);
                else bt_row_product<false>(bv, row, vv.dx, nullptr, 0.0f, y);
                if (g_lead)
#pragma unroll
                    for (int q = 0; q < 3; ++q) bw.r[3 * row + q] = vv.rhs[3 * row + q] - y[q];
            }
            __syncthreads();
            const bool factor = FACTOR && mode >= 2;  // a factor preconditioner
            // every row's r must be in place before the factor's first pass gathers it
            if (factor && !(bt_sync(bw, tk, error, k, target, s_tot, s_redf, &s_ok) &&
                          bt_apply_factor(bw, mode, tk, lo, hi, error, k, target, s_tot, s_redf, &s_ok))) {
                timed_out = true;
                break;
            }
            float acc3[3] = {0.0f, 0.0f, 0.0f};
            for (int row = lo + threadIdx.x; row < hi; row += blockDim.x) {
                float r[3], z[3];
#pragma unroll
                for (int q = 0; q < 3; ++q) r[q] = bw.r[3 * row + q];
                if (factor) {
#pragma unroll
                    for (int q = 0; q < 3; ++q) z[q] = bw.z[3 * row + q];
                } else {
                    bt_precond(vv.Minv, mode, row, r, z);
                }
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    bw.z[3 * row + q] = z[q];
                    const float bq = vv.rhs[3 * row + q];
                    acc3[0] = __fmaf_rn(r[q], z[q], acc3[0]);
                    acc3[1] = __fmaf_rn(r[q], r[q], acc3[1]);
                    acc3[2] = __fmaf_rn(bq, bq, acc3[2]);
                }
            }
            bool ok = bt_reduce<3>(acc3, bw, tk, error, k++, target, s_tot, s_redf, &s_ok);
            if (threadIdx.x == 0) {
                if (!ok) {
                    sc.status = MFEM_TIMEOUT;
                    sc.done = 1;
                    sc.rr = 0.0f;
                    sc.bb = 1.0f;
                } else {
                    sc.rz = s_tot[0];
                    sc.rr = s_tot[1];
                    sc.bb = s_tot[2];
                    sc.thr2 = tol * tol * s_tot[2];
                    sc.beta = 0.0f;
                    sc.status =
                        (isfinite(s_tot[0]) && isfinite(s_tot[1]) && isfinite(s_tot[2])) ? MFEM_OK : MFEM_NONFINITE;
                    sc.done = sc.status != MFEM_OK || s_tot[1] <= sc.thr2;
                }
            }
            __syncthreads();
            while (!sc.done) {
                if (it >= maxiter) {
                    if (threadIdx.x == 0) sc.status = MFEM_MAXITER;
                    break;
                }
                float *p_new = (it & 1) ? bw.p1 : bw.p0;
                const float *p_old = it == 0 ? nullptr : ((it & 1) ? bw.p0 : bw.p1);
                const float beta = sc.beta;
                float pap[1] = {0.0f};
                for (int row = lo + group; row < hi; row += ngroups) {
                    float y[3];
                    if (tk.size > 1) bt_row_product<true>(bv, row, bw.z, p_old, beta, y);
                    else bt_row_product<false>(bv, row, bw.z, p_old, beta, y);
                    if (g_lead) {
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            const float zq = bw.z[3 * row + q];
                            const float pq = p_old ? __fmaf_rn(beta, p_old[3 * row + q], zq) : zq;
                            p_new[3 * row + q] = pq;
                            bw.Ap[3 * row + q] = y[q];
                            pap[0] = __fmaf_rn(pq, y[q], pap[0]);
                        }
                    }
                }
                if (!bt_reduce<1>(pap, bw, tk, error, k++, target, s_tot, s_redf, &s_ok)) {
                    if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
                    break;
                }
                if (threadIdx.x == 0) {
                    if (!isfinite(s_tot[0])) {
                        sc.status = MFEM_NONFINITE;
                        sc.done = 1;
                    } else if (!(s_tot[0] > 0.0f)) {
                        sc.status = MFEM_STAGNATION;
                        sc.done = 1;
                    } else {
                        sc.alpha = sc.rz / s_tot[0];
                    }
                }
                __syncthreads();
                if (sc.done) break;
                const float alpha = sc.alpha;
                float acc2[2] = {0.0f, 0.0f};
                if (factor) {
                    for (int row = lo + threadIdx.x; row < hi; row += blockDim.x)
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            vv.dx[3 * row + q] = __fmaf_rn(alpha, p_new[3 * row + q], vv.dx[3 * row + q]);
                            bw.r[3 * row + q] = __fmaf_rn(-alpha, bw.Ap[3 * row + q], bw.r[3 * row + q]);
                        }
                    if (!(bt_sync(bw, tk, error, k, target, s_tot, s_redf, &s_ok) &&
                          bt_apply_factor(bw, mode, tk, lo, hi, error, k, target, s_tot, s_redf, &s_ok))) {
                        if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
                        break;
                    }
                }
                for (int row = lo + threadIdx.x; row < hi; row += blockDim.x) {
                    float r[3], z[3];
                    if (factor) {
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            r[q] = bw.r[3 * row + q];
                            z[q] = bw.z[3 * row + q];
                        }
                    } else {
#pragma unroll
                        for (int q = 0; q < 3; ++q) {
                            vv.dx[3 * row + q] = __fmaf_rn(alpha, p_new[3 * row + q], vv.dx[3 * row + q]);
                            r[q] = __fmaf_rn(-alpha, bw.Ap[3 * row + q], bw.r[3 * row + q]);
                            bw.r[3 * row + q] = r[q];
                        }
                        bt_precond(vv.Minv, mode, row, r, z);
                    }
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        bw.z[3 * row + q] = z[q];
                        acc2[0] = __fmaf_rn(r[q], z[q], acc2[0]);
                        acc2[1] = __fmaf_rn(r[q], r[q], acc2[1]);
                    }
                }
                if (!bt_reduce<2>(acc2, bw, tk, error, k++, target, s_tot, s_redf, &s_ok)) {
                    if (threadIdx.x == 0) sc.status = MFEM_TIMEOUT;
                    break;
                }
                ++it;
                if (threadIdx.x == 0) {
                    sc.rr = s_tot[1];
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
                for (int t3 = 3 * lo + threadIdx.x; t3 < 3 * hi; t3 += blockDim.x) vv.dx[t3] = bw.dx0[t3];
                // every row's warm start is back before the retry's product reads it
                if (!bt_sync(bw, tk, error, k, target, s_tot, s_redf, &s_ok)) {
                    timed_out = true;
                    break;
                }
                it_done += it;
                mode = 1;
                continue;
            }
            break;
        }
        if (tk.rank == 0 && threadIdx.x == 0) {
            const float rel = sc.bb > 0.0f ? sqrtf(sc.rr / sc.bb) : sqrtf(sc.rr);
            *st = timed_out ? SolveStats{0, MFEM_TIMEOUT, 0.0f, 0.0f} : SolveStats{it_done + it, sc.status, rel, 0.0f};
        }
        __syncthreads();  // sc and s_ok are reused by the next task
    }
}

}  // namespace

cudaError_t batch_capacity(int device, int threads, bool factor, int *ctas) {
    int sms = 0, occ = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess)
        e = factor ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched_pcg_kernel<true>, threads, 0)
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched_pcg_kernel<false>, threads, 0);
    if (e != cudaSuccess) return e;
    *ctas = sms * std::max(occ, 0);
    return cudaSuccess;
}

cudaError_t launch_batched_pcg(const BsrViews &bv, const VertexViews &vv, const BatchViews &bw, int *error, int slot,
                               float tol, int maxiter, int use_precond, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(bw.ctas);
    cfg.blockDim = dim3(bw.threads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = use_precond >= 2
                        ? cudaLaunchKernelEx(&cfg, batched_pcg_kernel<true>, bv, vv, bw, error, slot, tol, maxiter,
                                             use_precond)
                        : cudaLaunchKernelEx(&cfg, batched_pcg_kernel<false>, bv, vv, bw, error, slot, tol, maxiter,
                                             use_precond);
    count_launches(1);
    return e;
}

}  // namespace mfem
