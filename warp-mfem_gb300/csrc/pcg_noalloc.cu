// mfem_pcg_solve_noalloc: block-Jacobi PCG on a caller-provided 3x3-block
// BSR system that allocates no memory.
//
// Some callers cannot allocate device memory at the point where they need a
// solve: code that runs while a framework's caching allocator owns the GPU
// heap, real-time or embedded hosts that forbid allocation after start-up,
// and callers that hand a plain C ABI their own buffers and nothing else.
// The plan API (mfem_plan_create) allocates its workspace with cudaMalloc;
// this entry point instead keeps its scratch vectors in a fixed-size array in
// the library's own device memory (`g_pcg_noalloc_scratch` below), which
// every GPU that loads the library holds until the process exits.
//
// Limits and sharing:
//  * at most kNoAllocMaxRows block rows (vertices); larger systems are
//    rejected with MFEM_BAD_ARG and a message;
//  * every call uses the same array, and the array keeps the last call's
//    contents: each call clears what must start at zero (the barrier counter
//    and the error flag) on its stream before its kernel runs.  Calls whose
//    kernels overlap on the GPU (two streams, or two host threads) race on
//    the array and produce wrong results; serialise them.
//  * every call looks up the array's device address (cudaGetSymbolAddress)
//    with the caller's device current; the first lookup on a device loads
//    the module, so make that first call before any stream capture begins;
//  * the caller keeps the system well formed: row_ptr[0] = 0, row_ptr
//    non-decreasing with row_ptr[n] = nnzb, and 0 <= col_idx < n.  Indices
//    outside that range are not checked on the device and read the wrong
//    memory.
//
// The solve is the standard two-phase PCG (p = z + beta p, Ap, alpha; x, r
// updates, z = M r, beta), one persistent cooperative kernel with a grid
// barrier per phase; each CTA owns a contiguous range of rows and gathers the
// vectors of other rows from global memory (no shared-memory windows, so the
// caller's arrays need no padding).
#include <algorithm>
#include <string>

#include "grid_sync.cuh"
#include "internal.h"

namespace mfem {
namespace {

constexpr int kNoAllocMaxRows = 32768;  // block rows (vertices) the scratch serves
constexpr int kNaMaxCtas = 256;
constexpr int kNaThreads = 512;
constexpr int kNaGroup = 4;             // lanes per block row in the product
constexpr long long kNaWaitCycles = 8000000000ll;

// scratch layout (floats): z, p[2], r, Ap (each kNoAllocMaxRows * 3), the
// per-CTA partials [2][kNaMaxCtas][4], then the barrier counter and error flag
constexpr size_t kVec = (size_t)kNoAllocMaxRows * 3;
constexpr size_t kPartialsOff = 5 * kVec;
constexpr size_t kCounterOffBytes = (kPartialsOff + 2 * kNaMaxCtas * 4) * sizeof(float);
constexpr size_t kScratchBytes = kCounterOffBytes + 256;

}  // namespace

// The scratch array (about 2 MB).  In host code this name is only a host-side
// stand-in: the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_pcg_noalloc_scratch[kScratchBytes];

namespace {

struct NaArgs {
    int n;
    const int *row_ptr;
    const int *col_idx;
    const float *values;
    const float *Minv;  // may be null: no preconditioner
    const float *b;
    float *x;
    float *z, *p0, *p1, *r, *Ap;
    float *partials;
    unsigned long long *counter;
    int *error;
    mfem_solve_stats *stats;  // may be null
    float tol;
    int maxiter;
};

__device__ __forceinline__ unsigned long long na_ld_relaxed(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Block-reduce NV float partials, store this CTA's sums for barrier k, wait at
// the grid barrier, then sum all CTAs' partials in a fixed order into tot[].
template <int NV>
__device__ bool na_reduce(float (&v)[NV], const NaArgs &a, unsigned k, unsigned long long &target, float *tot,
                          float (*s_redf)[32], float *s_val, int *s_ok) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nb = gridDim.x;
#pragma unroll
    for (int i = 0; i < NV; ++i)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[i] += __shfl_down_sync(0xffffffffu, v[i], off);
    if (lane == 0)
#pragma unroll
        for (int i = 0; i < NV; ++i) s_redf[i][wid] = v[i];
    __syncthreads();
    float *buf = a.partials + (size_t)(k & 1u) * kNaMaxCtas * 4;
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
#pragma unroll
            for (int i = 0; i < NV; ++i) buf[(size_t)blockIdx.x * 4 + i] = part[i];
            target += nb;
            grid_arrive(a.counter);
            int ok = 1;
            const long long t0 = clock64();
            unsigned spins = 0;
            while (grid_count(a.counter) < target) {
                if ((++spins & 1023u) == 0 &&
                    (*(const volatile int *)a.error != 0 || clock64() - t0 > kNaWaitCycles)) {
                    atomicExch(a.error, 1);
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
        float acc[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) acc[i] = 0.0f;
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

__device__ __forceinline__ void na_precond(const float *Minv, int row, const float r[3], float z[3]) {
    if (!Minv) {
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

struct NaScalars {
    float alpha, beta, rz, rr, bb, thr2;
    int status, done;
};

// y_row = sum_k H[k] (z[col] + beta p_old[col]) by kNaGroup lanes; with
// p_old == nullptr the vector is z itself.
__device__ __forceinline__ void na_row_product(const NaArgs &a, int row, const float *z, const float *p_old,
                                               float beta, float y[3]) {
    const int g_lane = threadIdx.x & (kNaGroup - 1);
    const unsigned gmask = ((1u << kNaGroup) - 1u) << (threadIdx.x & (32 - kNaGroup));
    const int kb = a.row_ptr[row], ke = a.row_ptr[row + 1];
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
    for (int k = kb + g_lane; k < ke; k += kNaGroup) {
        const int c = __ldg(a.col_idx + k);
        float v[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float zc = __ldcg(z + 3 * c + q);
            v[q] = p_old ? __fmaf_rn(beta, __ldcg(p_old + 3 * c + q), zc) : zc;
        }
        const float *h = a.values + (size_t)9 * k;
        a0 += __ldg(h + 0) * v[0] + __ldg(h + 1) * v[1] + __ldg(h + 2) * v[2];
        a1 += __ldg(h + 3) * v[0] + __ldg(h + 4) * v[1] + __ldg(h + 5) * v[2];
        a2 += __ldg(h + 6) * v[0] + __ldg(h + 7) * v[1] + __ldg(h + 8) * v[2];
    }
#pragma unroll
    for (int off = kNaGroup / 2; off > 0; off >>= 1) {
        a0 += __shfl_xor_sync(gmask, a0, off);
        a1 += __shfl_xor_sync(gmask, a1, off);
        a2 += __shfl_xor_sync(gmask, a2, off);
    }
    y[0] = a0;
    y[1] = a1;
    y[2] = a2;
}

__global__ void __launch_bounds__(kNaThreads, 1) pcg_noalloc_kernel(NaArgs a) {
    __shared__ float s_redf[3][32];
    __shared__ float s_val[4 * kNaMaxCtas];
    __shared__ float s_tot[3];
    __shared__ NaScalars sc;
    __shared__ int s_ok;
    const int nb = gridDim.x, cta = blockIdx.x;
    const int lo = (int)(((long long)a.n * cta) / nb), hi = (int)(((long long)a.n * (cta + 1)) / nb);
    const int group = threadIdx.x / kNaGroup, ngroups = blockDim.x / kNaGroup;
    const bool g_lead = (threadIdx.x & (kNaGroup - 1)) == 0;
    unsigned long long target = 0;  // the counter starts at zero every call
    unsigned k = 0;
    int it = 0;

    // ---- r = b - H x0, z = M r
    for (int row = lo + group; row < hi; row += ngroups) {
        float y[3];
        na_row_product(a, row, a.x, nullptr, 0.0f, y);
        if (g_lead)
#pragma unroll
            for (int q = 0; q < 3; ++q) a.r[3 * row + q] = a.b[3 * row + q] - y[q];
    }
    __syncthreads();
    float acc3[3] = {0.0f, 0.0f, 0.0f};
    for (int row = lo + threadIdx.x; row < hi; row += blockDim.x) {
        float r[3], z[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) r[q] = a.r[3 * row + q];
        na_precond(a.Minv, row, r, z);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            a.z[3 * row + q] = z[q];
            const float bq = a.b[3 * row + q];
            acc3[0] = __fmaf_rn(r[q], z[q], acc3[0]);
            acc3[1] = __fmaf_rn(r[q], r[q], acc3[1]);
            acc3[2] = __fmaf_rn(bq, bq, acc3[2]);
        }
    }
    bool ok = na_reduce<3>(acc3, a, k++, target, s_tot, s_redf, s_val, &s_ok);
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
            sc.thr2 = a.tol * a.tol * s_tot[2];
            sc.beta = 0.0f;
            sc.status = (isfinite(s_tot[0]) && isfinite(s_tot[1]) && isfinite(s_tot[2])) ? MFEM_OK : MFEM_NONFINITE;
            sc.done = sc.status != MFEM_OK || s_tot[1] <= sc.thr2;
        }
    }
    __syncthreads();
    while (!sc.done) {
        if (it >= a.maxiter) {
            if (threadIdx.x == 0) sc.status = MFEM_MAXITER;
            break;
        }
        // ---- p = z + beta p; Ap = H p; p.Ap
        float *p_new = (it & 1) ? a.p1 : a.p0;
        const float *p_old = it == 0 ? nullptr : ((it & 1) ? a.p0 : a.p1);
        const float beta = sc.beta;
        float pap[1] = {0.0f};
        for (int row = lo + group; row < hi; row += ngroups) {
            float y[3];
            na_row_product(a, row, a.z, p_old, beta, y);
            if (g_lead) {
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const float zq = __ldcg(a.z + 3 * row + q);
                    const float pq = p_old ? __fmaf_rn(beta, __ldcg(p_old + 3 * row + q), zq) : zq;
                    p_new[3 * row + q] = pq;
                    a.Ap[3 * row + q] = y[q];
                    pap[0] = __fmaf_rn(pq, y[q], pap[0]);
                }
            }
        }
        if (!na_reduce<1>(pap, a, k++, target, s_tot, s_redf, s_val, &s_ok)) {
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
        // ---- x += alpha p; r -= alpha Ap; z = M r
        const float alpha = sc.alpha;
        float acc2[2] = {0.0f, 0.0f};
        for (int row = lo + threadIdx.x; row < hi; row += blockDim.x) {
            float r[3], z[3];
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                a.x[3 * row + q] = __fmaf_rn(alpha, p_new[3 * row + q], a.x[3 * row + q]);
                r[q] = __fmaf_rn(-alpha, a.Ap[3 * row + q], a.r[3 * row + q]);
                a.r[3 * row + q] = r[q];
            }
            na_precond(a.Minv, row, r, z);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                a.z[3 * row + q] = z[q];
                acc2[0] = __fmaf_rn(r[q], z[q], acc2[0]);
                acc2[1] = __fmaf_rn(r[q], r[q], acc2[1]);
            }
        }
        if (!na_reduce<2>(acc2, a, k++, target, s_tot, s_redf, s_val, &s_ok)) {
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
    if (cta == 0 && threadIdx.x == 0 && a.stats) {
        a.stats->iterations = it;
        a.stats->status = sc.status;
        a.stats->rel_residual = sc.bb > 0.0f ? sqrtf(sc.rr / sc.bb) : sqrtf(sc.rr);
        a.stats->reserved = 0.0f;
    }
}

}  // namespace
}  // namespace mfem

using namespace mfem;

extern "C" int mfem_pcg_solve_noalloc(int32_t n, const int32_t *d_row_ptr, const int32_t *d_col_idx,
                                      const float *d_values, const float *d_precond, const float *d_b, float *d_x,
                                      float tol, int32_t maxiter, mfem_solve_stats *d_stats, mfem_stream stream) {
    if (n <= 0 || !d_row_ptr || !d_col_idx || !d_values || !d_b || !d_x)
        return set_create_error(MFEM_BAD_ARG, "mfem_pcg_solve_noalloc: n must be > 0 and the arrays non-NULL");
    if (n > kNoAllocMaxRows)
        return set_create_error(MFEM_BAD_ARG, "mfem_pcg_solve_noalloc: " + std::to_string(n) +
                                                  " block rows exceed the fixed scratch of " +
                                                  std::to_string(kNoAllocMaxRows) + " rows");
    if (!(tol >= 0.0f) || maxiter < 0)
        return set_create_error(MFEM_BAD_ARG, "mfem_pcg_solve_noalloc: tol must be >= 0 and maxiter >= 0");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0)
        return set_create_error(MFEM_CUDA_ERROR, "mfem_pcg_solve_noalloc: no usable current device");
    // The scratch array's device address, looked up on every call with the
    // caller's device current: after a cudaDeviceReset or in a new primary
    // context the module may load at another address, so no address is
    // cached.  Only the first lookup on a device loads the module (the reason
    // that call must come before any stream capture); later ones are cheap.
    void *base = nullptr;
    e = cudaGetSymbolAddress(&base, g_pcg_noalloc_scratch);
    if (e != cudaSuccess)
        return set_create_error(MFEM_CUDA_ERROR,
                                std::string("mfem_pcg_solve_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_create_error(MFEM_CUDA_ERROR, "mfem_pcg_solve_noalloc: device query failed");
    const int ctas = std::max(1, std::min({sms, kNaMaxCtas, (n + 63) / 64}));

    float *f = static_cast<float *>(base);
    NaArgs a;
    a.n = n;
    a.row_ptr = d_row_ptr;
    a.col_idx = d_col_idx;
    a.values = d_values;
    a.Minv = d_precond;
    a.b = d_b;
    a.x = d_x;
    a.z = f;
    a.p0 = f + kVec;
    a.p1 = f + 2 * kVec;
    a.r = f + 3 * kVec;
    a.Ap = f + 4 * kVec;
    a.partials = f + kPartialsOff;
    a.counter = reinterpret_cast<unsigned long long *>(static_cast<unsigned char *>(base) + kCounterOffBytes);
    a.error = reinterpret_cast<int *>(static_cast<unsigned char *>(base) + kCounterOffBytes + 8);
    a.stats = d_stats;
    a.tol = tol;
    a.maxiter = maxiter;
    cudaStream_t s = (cudaStream_t)stream;
    // the barrier counter and the error flag start at zero every call
    e = cudaMemsetAsync(a.counter, 0, 16, s);
    if (e != cudaSuccess)
        return set_create_error(MFEM_CUDA_ERROR, std::string("mfem_pcg_solve_noalloc: ") + cudaGetErrorString(e));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(kNaThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, pcg_noalloc_kernel, a);
    count_launches(1);
    if (e != cudaSuccess)
        return set_create_error(MFEM_CUDA_ERROR, std::string("mfem_pcg_solve_noalloc: ") + cudaGetErrorString(e));
    return MFEM_OK;
}
