// Backtracking line search on the merit function of the mixed system, one
// persistent cooperative kernel per Newton iteration.
//
// The reference runs the search as a loop of small launches inside
// wp.capture_while / wp.capture_if conditional graph nodes
// (src/mfem/line_search.py:76-163; objective src/mfem/refinement/solver.py:
// 803-869, search setup 871-928).  Here the whole loop runs on the device:
//
//   merit f(x, s) = [sum_v m |x - x~|^2 / 2 + sum_pinned k |x - p|^2 / 2] / dt^2
//                 + sum_t [Psi_t(s) - lambda_t . c_t(x, s)]      (lambda fixed)
//   t  = -c (g_x . dx - lambda . G dx + (g_s + SYM lambda) . ds)
//   alpha = alpha0 tau^j for j = 0, 1, ... until (f0 - f1) + threshold >=
//   alpha t or j = max_iterations; x, s move to the last trial only if the
//   trial counter after it is < max_iterations.
//
// G is the reference's dC_dX (-dc/dx, kernels.py:159) and the reference forms
// the x-gradient as g_x - G^T lambda (solver.py:905); the slope here keeps
// that sign.
//
// The local-solve kernel (element.cu) leaves x and s untouched, stores ds and
// writes, per block, the partial sums of f0 and of the slope.  This kernel
// then evaluates one trial per round: every thread takes a grid-strided set of
// tets (gathering x + alpha dx of their four vertices, polar SVD, energy and
// constraint term) and of vertices (kinetic and attachment terms); per-thread
// sums are float64, block sums are stored per CTA and the grid waits at a
// counter barrier.  Every CTA then adds the CTA partials in the same fixed
// order, so all CTAs reach the same decision and the result is deterministic.
// The first round also carries each CTA's slice of the local-solve partials,
// so f0 and t come with the first trial at no extra barrier.
//
// With contact, the merit also carries the barrier and friction energies
// of the vertices and the barrier energies of the surface tris, evaluated at
// each trial point (solver.py:858-862), and the slope their gradients.
//
// Every wait is bounded; after a timeout the kernel sets the sticky error
// flag and leaves x and s unchanged, reporting MFEM_TIMEOUT.
#include <algorithm>

#include "grid_sync.cuh"
#include "merit.cuh"

namespace mfem {
namespace {

constexpr int kLsThreads = 256;
constexpr int kLsWarps = kLsThreads / 32;
constexpr long long kWaitCycles = 8000000000ll;  // ~4 s at 2 GHz per wait

struct LsArgs {
    TetViews tv;
    VertexViews vv;
    ContactViews cv;
    float ev;  // friction threshold eps_v dt
    float *x;
    LineSearchWork w;
    int *error;
    int slot;
    int energy;
    double inv_dt2;
};

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_volatile(const int *p) { return *(const volatile int *)p; }

__global__ void __launch_bounds__(kLsThreads, 4) line_search_kernel(LsArgs a) {
    __shared__ double s_red[3][kLsWarps];
    __shared__ double s_val[3 * kLsMaxCtas];
    __shared__ double s_tot[3];
    __shared__ int s_ok;
    __shared__ unsigned long long s_base;
    const LineSearchWork &w = a.w;
    const int nb = gridDim.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        s_base = (ld_relaxed(w.counter) / nb) * (unsigned long long)nb;
        s_ok = ld_volatile(a.error) == 0;
    }
    __syncthreads();
    if (!s_ok) {
        if (blockIdx.x == 0 && threadIdx.x == 0)
            w.stats[a.slot] = LineSearchStats{0, 0, 0.0f, MFEM_TIMEOUT, 0.0, 0.0, 0.0};
        return;
    }
    unsigned long long target = s_base;

    // this CTA's slice of the local-solve partials (f0, slope)
    double lf = 0.0, lsl = 0.0;
    {
        const int L = w.local_blocks;
        const int lo = (int)(((long long)L * blockIdx.x) / nb), hi = (int)(((long long)L * (blockIdx.x + 1)) / nb);
        for (int i = lo + (int)threadIdx.x; i < hi; i += kLsThreads) {
            lf += w.local_partials[2 * i + 0];
            lsl += w.local_partials[2 * i + 1];
        }
    }

    const int T = a.tv.n_tets, n = a.vv.n;
    const int stride = nb * kLsThreads;
    const int first = blockIdx.x * kLsThreads + threadIdx.x;
    const double thr = (double)w.threshold;
    float alpha = w.alpha0;
    double f0 = 0.0, f1 = 0.0, tslope = 0.0;
    int j = 0;
    for (;;) {
        double e = 0.0;
        for (int t = first; t < T; t += stride) e += tet_merit(a.tv, a.x, a.vv.dx, w.ds, a.energy, t, alpha);
        for (int v = first; v < n; v += stride) e += vertex_merit(a.vv, a.x, v, alpha, a.inv_dt2);
        if (a.cv.on) {
            // barrier and friction energies at the trial (Contact.evaluate_energy_only)
            for (int v = first; v < n; v += stride) {
                float xt[3];
#pragma unroll
                for (int c = 0; c < 3; ++c) xt[c] = fmaf(alpha, a.vv.dx[3 * v + c], a.x[3 * v + c]);
                e += (double)vertex_contact_energy(a.cv, a.vv, v, xt, a.ev);
            }
            for (int t = first; t < a.cv.n_tris; t += stride)
                e += (double)tri_contact_energy(a.cv, a.x, a.vv.dx, t, alpha);
        }
        double part[3] = {e, j == 0 ? lf : 0.0, j == 0 ? lsl : 0.0};
#pragma unroll
        for (int i = 0; i < 3; ++i) part[i] = warp_sum(part[i]);
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < 3; ++i) s_red[i][wid] = part[i];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double *buf = w.partials + ((size_t)(j & 1) * kLsMaxCtas + blockIdx.x) * 3;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                double acc = 0.0;
                for (int k = 0; k < kLsWarps; ++k) acc += s_red[i][k];
                buf[i] = acc;
            }
            // arrive: the partials are released before the counter moves
            target += nb;
            grid_arrive(w.counter);
            int ok = 1;
            const long long t0 = clock64();
            unsigned spins = 0;
            while (grid_count(w.counter) < target) {
                if ((++spins & 1023u) == 0 && (ld_volatile(a.error) != 0 || clock64() - t0 > kWaitCycles)) {
                    atomicExch(a.error, 1);
                    ok = 0;
                    break;
                }
            }
            s_ok = ok;
        }
        __syncthreads();
        if (!s_ok) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                w.stats[a.slot] = LineSearchStats{j + 1, 0, alpha, MFEM_TIMEOUT, 0.0, 0.0, 0.0};
            return;
        }
        // totals over the CTAs: one load per thread, then a fixed-order sum
        const double *buf = w.partials + (size_t)(j & 1) * kLsMaxCtas * 3;
        for (int i = threadIdx.x; i < 3 * nb; i += kLsThreads) s_val[i] = __ldcg(buf + i);
        __syncthreads();
        if (wid == 0) {
            double acc[3] = {0.0, 0.0, 0.0};
            for (int b = lane; b < nb; b += 32) {
#pragma unroll
                for (int i = 0; i < 3; ++i) acc[i] += s_val[3 * b + i];
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) acc[i] = warp_sum(acc[i]);
            if (lane == 0) {
#pragma unroll
                for (int i = 0; i < 3; ++i) s_tot[i] = acc[i];
            }
        }
        __syncthreads();
        if (j == 0) {
            f0 = s_tot[1];
            tslope = -(double)w.c * s_tot[2];
        }
        f1 = s_tot[0];
        // _condition_kernel (line_search.py:44-63)
        const bool more = ((f0 - f1) + thr < (double)alpha * tslope) && j < w.max_iter;
        ++j;
        if (!more) break;
        alpha *= w.tau;
        // the next round's partials use the other buffer; the round after it
        // reuses this one only after every CTA has passed the next barrier,
        // i.e. after every CTA has read these totals
    }
    const bool accepted = j < w.max_iter;  // _iteration_condition (line_search.py:66-72)
    if (accepted) {
        // every CTA has finished reading x and s for the last trial (barrier)
        for (int t = first; t < T; t += stride)
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                float *sp = a.tv.stretch + (size_t)t * 6 + i;
                *sp = fmaf(alpha, w.ds[(size_t)i * T + t], *sp);
            }
        for (int v = first; v < n; v += stride)
#pragma unroll
            for (int c = 0; c < 3; ++c) a.x[3 * v + c] = fmaf(alpha, a.vv.dx[3 * v + c], a.x[3 * v + c]);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        w.stats[a.slot] = LineSearchStats{j, accepted ? 1 : 0, alpha, MFEM_OK, f0, f1, tslope};
}

}  // namespace

int line_search_threads() { return kLsThreads; }

cudaError_t line_search_max_ctas(int device, int *ctas) {
    int sms = 0, occ = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, line_search_kernel, kLsThreads, 0);
    if (e != cudaSuccess) return e;
    *ctas = std::max(1, std::min(kLsMaxCtas, sms * std::max(occ, 1)));
    return cudaSuccess;
}

cudaError_t launch_line_search(float *x, int energy, float dt, const TetViews &tv, const VertexViews &vv,
                               const ContactViews &cv, const LineSearchWork &w, int *error, int slot,
                               cudaStream_t s) {
    LsArgs a;
    a.tv = tv;
    a.vv = vv;
    a.cv = cv;
    a.ev = (float)((double)cv.eps_v * (double)dt);
    a.x = x;
    a.w = w;
    a.error = error;
    a.slot = slot;
    a.energy = energy;
    a.inv_dt2 = 1.0 / ((double)dt * (double)dt);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(w.ctas);
    cfg.blockDim = dim3(kLsThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, line_search_kernel, a);
    count_launches(1);
    return e;
}

}  // namespace mfem
