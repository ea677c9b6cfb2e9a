// Block-Jacobi preconditioned CG on the 3x3-block BSR system H dx = g, as
// one persistent cooperative kernel per solve.
//
// The reference runs warp.optim.linear.cg (check_every=0, graph-captured,
// M = block-Jacobi inverse) (src/mfem/refinement/solver.py:220-235, 581-609).
// Here every CTA owns a contiguous range of block rows and the solve loops on
// the device with no host round trip.  One iteration is two phases, each
// ended by a grid barrier that also completes a deterministic reduction:
//
//   A: w = H z (z gathered from every CTA), Ap = w + beta Ap, p = z + beta p
//      (so H p needs no extra pass), partial p.Ap
//   B: alpha = rz / p.Ap; x += alpha p; r -= alpha Ap; z = M r; partial r.z, r.r
//
// Every CTA sums the per-CTA partials in the same fixed order, so all CTAs
// take the same convergence decision.  Stopping test: ||r|| <= tol ||g||,
// checked before the first iteration and after every phase B.  Scalars
// (dot products, alpha, beta) are accumulated in float64.
//
// The grid barrier counts arrivals on a 64-bit counter that is never reset:
// the k-th barrier of a launch releases at base + k * CTAs.  Each wait is
// bounded (globaltimer); a timeout sets the sticky error flag and every CTA
// leaves, reporting MFEM_TIMEOUT.
#include "internal.h"

namespace mfem {
namespace {

constexpr int kPcgThreads = 512;
constexpr int kGroup = 16;                       // lanes per block row in the SpMV
constexpr unsigned long long kWaitLimitNs = 5000000000ull;  // 5 s per barrier wait

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int ld_volatile(const int *p) { return *(const volatile int *)p; }

// Grid barrier; false if the wait gave up (or another CTA did).
__device__ bool grid_barrier(unsigned long long *bar, unsigned long long &target, int *error, int *s_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        target += gridDim.x;
        __threadfence();
        atomicAdd(bar, 1ull);
        int ok = 1;
        if (ld_acquire(bar) < target) {
            const unsigned long long t0 = globaltimer();
            while (ld_acquire(bar) < target) {
                if (ld_volatile(error) != 0 || globaltimer() - t0 > kWaitLimitNs) {
                    atomicExch(error, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// Deterministic block reduction of up to 3 doubles; result valid in thread 0.
template <int NV>
__device__ void block_reduce(double (&v)[NV], double (*s_red)[32]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
    }
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) s_red[i][wid] = v[i];
    }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            v[i] = lane < nw ? s_red[i][lane] : 0.0;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
        }
    }
    __syncthreads();
}

// Sum of the per-CTA partials (stride 4 doubles) in a fixed order; every
// thread of the CTA gets the totals.
template <int NV>
__device__ void grid_totals(const double *part, double (&tot)[NV], double *s_tot) {
    if (threadIdx.x < 32) {
        double acc[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) acc[i] = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += 32) {
#pragma unroll
            for (int i = 0; i < NV; ++i) acc[i] += __ldcg(part + (size_t)b * 4 + i);
        }
#pragma unroll
        for (int i = 0; i < NV; ++i) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], off);
        }
        if (threadIdx.x == 0) {
#pragma unroll
            for (int i = 0; i < NV; ++i) s_tot[i] = acc[i];
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) tot[i] = s_tot[i];
    __syncthreads();
}

// y_row = sum_k H[k] v[col[k]] over one block row, by a group of kGroup
// lanes; every lane of the group returns the row's sum.
__device__ __forceinline__ void row_product(const BsrViews &bv, const float *__restrict__ vec, int row, int g_lane,
                                            unsigned gmask, float y[3]) {
    const int rb = __ldg(bv.row_ptr + row);
    const int re = __ldg(bv.row_ptr + row + 1);
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
    for (int k = rb + g_lane; k < re; k += kGroup) {
        const int col = __ldg(bv.col_idx + k);
        const float *h = bv.values + (size_t)k * 9;
        const float v0 = __ldcg(vec + 3 * col + 0);
        const float v1 = __ldcg(vec + 3 * col + 1);
        const float v2 = __ldcg(vec + 3 * col + 2);
        a0 += __ldg(h + 0) * v0 + __ldg(h + 1) * v1 + __ldg(h + 2) * v2;
        a1 += __ldg(h + 3) * v0 + __ldg(h + 4) * v1 + __ldg(h + 5) * v2;
        a2 += __ldg(h + 6) * v0 + __ldg(h + 7) * v1 + __ldg(h + 8) * v2;
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

__device__ __forceinline__ void apply_precond(const float *__restrict__ Minv, int row, const float r[3], float z[3],
                                              int use_precond) {
    if (!use_precond) {
        z[0] = r[0];
        z[1] = r[1];
        z[2] = r[2];
        return;
    }
    const float *m = Minv + (size_t)row * 9;
    z[0] = m[0] * r[0] + m[1] * r[1] + m[2] * r[2];
    z[1] = m[3] * r[0] + m[4] * r[1] + m[5] * r[2];
    z[2] = m[6] * r[0] + m[7] * r[1] + m[8] * r[2];
}

__global__ void __launch_bounds__(kPcgThreads, 1)
    pcg_kernel(BsrViews bv, const float *__restrict__ Minv, const float *__restrict__ b, float *x, PcgWork w,
               int slot, float tol, int maxiter, int use_precond) {
    __shared__ double s_red[3][32];
    __shared__ double s_tot[4];
    __shared__ int s_ok;
    __shared__ unsigned long long s_base;

    const int n = bv.n;
    const int cta = blockIdx.x;
    const int nb = gridDim.x;
    const int row_lo = (int)(((long long)n * cta) / nb);
    const int row_hi = (int)(((long long)n * (cta + 1)) / nb);
    const int g_lane = threadIdx.x & (kGroup - 1);
    const int group = threadIdx.x / kGroup;
    const int ngroups = blockDim.x / kGroup;
    const unsigned gmask = 0xffffu << (threadIdx.x & 16);
    double *partA = w.partials;
    double *partB = w.partials + (size_t)nb * 4;

    if (threadIdx.x == 0) {
        s_base = (ld_acquire(w.barrier) / (unsigned long long)nb) * (unsigned long long)nb;
        s_ok = ld_volatile(w.error) == 0;
    }
    __syncthreads();
    unsigned long long target = s_base;
    if (!s_ok) {
        if (cta == 0 && threadIdx.x == 0) {
            w.stats[slot].iterations = 0;
            w.stats[slot].status = MFEM_TIMEOUT;
            w.stats[slot].rel_residual = 0.0f;
        }
        return;
    }

    // ---- phase I: r = g - H x0, z = M r; partials r.z, r.r, g.g
    for (int row = row_lo + group; row < row_hi; row += ngroups) {
        float y[3];
        row_product(bv, x, row, g_lane, gmask, y);
        if (g_lane == 0) {
#pragma unroll
            for (int a = 0; a < 3; ++a) w.r[3 * row + a] = b[3 * row + a] - y[a];
        }
    }
    __syncthreads();
    {
        double acc[3] = {0.0, 0.0, 0.0};
        for (int row = row_lo + threadIdx.x; row < row_hi; row += blockDim.x) {
            float r[3], z[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) r[a] = w.r[3 * row + a];
            apply_precond(Minv, row, r, z, use_precond);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                w.z[3 * row + a] = z[a];
                const double bg = b[3 * row + a];
                acc[0] += (double)r[a] * (double)z[a];
                acc[1] += (double)r[a] * (double)r[a];
                acc[2] += bg * bg;
            }
        }
        block_reduce<3>(acc, s_red);
        if (threadIdx.x == 0) {
            partB[(size_t)cta * 4 + 0] = acc[0];
            partB[(size_t)cta * 4 + 1] = acc[1];
            partB[(size_t)cta * 4 + 2] = acc[2];
        }
    }
    int status = MFEM_OK;
    int it = 0;
    double rz, rr, bb;
    if (!grid_barrier(w.barrier, target, w.error, &s_ok)) {
        status = MFEM_TIMEOUT;
        rr = 0.0;
        bb = 1.0;
    } else {
        double tot[3];
        grid_totals<3>(partB, tot, s_tot);
        rz = tot[0];
        rr = tot[1];
        bb = tot[2];
        const double thr2 = (double)tol * (double)tol * bb;
        if (!isfinite(rr) || !isfinite(bb) || !isfinite(rz)) status = MFEM_NONFINITE;
        double beta = 0.0;
        bool done = (status != MFEM_OK) || rr <= thr2;
        while (!done) {
            if (it >= maxiter) {
                status = MFEM_MAXITER;
                break;
            }
            // ---- phase A: Ap = H z + beta Ap, p = z + beta p, partial p.Ap
            const float fbeta = (float)beta;
            double pap = 0.0;
            for (int row = row_lo + group; row < row_hi; row += ngroups) {
                float y[3];
                row_product(bv, w.z, row, g_lane, gmask, y);
                if (g_lane == 0) {
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const float zr = __ldcg(w.z + 3 * row + a);
                        float ap, pp;
                        if (it == 0) {
                            ap = y[a];
                            pp = zr;
                        } else {
                            ap = y[a] + fbeta * w.Ap[3 * row + a];
                            pp = zr + fbeta * w.p[3 * row + a];
                        }
                        w.Ap[3 * row + a] = ap;
                        w.p[3 * row + a] = pp;
                        pap += (double)pp * (double)ap;
                    }
                }
            }
            {
                double acc[1] = {pap};
                block_reduce<1>(acc, s_red);
                if (threadIdx.x == 0) partA[(size_t)cta * 4] = acc[0];
            }
            if (!grid_barrier(w.barrier, target, w.error, &s_ok)) {
                status = MFEM_TIMEOUT;
                break;
            }
            double totA[1];
            grid_totals<1>(partA, totA, s_tot);
            const double pAp = totA[0];
            if (!isfinite(pAp)) {
                status = MFEM_NONFINITE;
                break;
            }
            if (!(pAp > 0.0)) {
                status = MFEM_STAGNATION;
                break;
            }
            const float alpha = (float)(rz / pAp);
            // ---- phase B: x += alpha p, r -= alpha Ap, z = M r
            double acc[2] = {0.0, 0.0};
            for (int row = row_lo + threadIdx.x; row < row_hi; row += blockDim.x) {
                float r[3], z[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    x[3 * row + a] += alpha * w.p[3 * row + a];
                    r[a] = w.r[3 * row + a] - alpha * w.Ap[3 * row + a];
                    w.r[3 * row + a] = r[a];
                }
                apply_precond(Minv, row, r, z, use_precond);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    w.z[3 * row + a] = z[a];
                    acc[0] += (double)r[a] * (double)z[a];
                    acc[1] += (double)r[a] * (double)r[a];
                }
            }
            block_reduce<2>(acc, s_red);
            if (threadIdx.x == 0) {
                partB[(size_t)cta * 4 + 0] = acc[0];
                partB[(size_t)cta * 4 + 1] = acc[1];
            }
            if (!grid_barrier(w.barrier, target, w.error, &s_ok)) {
                status = MFEM_TIMEOUT;
                break;
            }
            double totB[2];
            grid_totals<2>(partB, totB, s_tot);
            ++it;
            const double rz_new = totB[0];
            rr = totB[1];
            if (!isfinite(rr) || !isfinite(rz_new)) {
                status = MFEM_NONFINITE;
                break;
            }
            beta = rz_new / rz;
            rz = rz_new;
            done = rr <= thr2;
        }
    }
    if (cta == 0 && threadIdx.x == 0) {
        w.stats[slot].iterations = it;
        w.stats[slot].status = status;
        w.stats[slot].rel_residual = (float)(bb > 0.0 ? sqrt(rr / bb) : sqrt(rr));
        w.stats[slot].reserved = 0.0f;
    }
}

}  // namespace

cudaError_t pcg_max_ctas(int device, int *ctas) {
    int sms = 0, per_sm = 0;
    cudaError_t err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (err != cudaSuccess) return err;
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pcg_kernel, kPcgThreads, 0);
    if (err != cudaSuccess) return err;
    *ctas = sms * per_sm;
    return cudaSuccess;
}

cudaError_t launch_pcg(const BsrViews &bv, const VertexViews &vv, const PcgWork &w, int ctas, int slot, float tol,
                       int maxiter, int use_precond, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(kPcgThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t err = cudaLaunchKernelEx(&cfg, pcg_kernel, bv, (const float *)vv.Minv, (const float *)vv.rhs, vv.dx, w,
                                         slot, tol, maxiter, use_precond);
    count_launches(1);
    return err;
}

}  // namespace mfem
