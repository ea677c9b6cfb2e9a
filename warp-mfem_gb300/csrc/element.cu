// Per-tet and per-vertex kernels of the global step.
//
//  element_kernel      one thread per tet: the reference's compute_constraints,
//                      energy gradient/Hessian in s, compute_H_lmbda_blocks,
//                      compute_g_lmbda and compute_H_lmbda_G_x_blocks fused,
//                      plus the element blocks G^T H_l G and rhs (H_l G)^T g_l
//                      that the assembly gathers.
//  local_solve_kernel  tets: local_solve_lambda + local_solve_stretch + s += ds;
//                      vertices: x += dx  (one launch, two index ranges).
//  local_solve_deferred_kernel  the same local solve ahead of the line search:
//                      stores ds, leaves x and s, sums the merit and slope.
//  predict_kernel      integrate_particles + state_out.assign(state_in).
//  velocity_kernel     get_particle_velocity.
#include <algorithm>

#include "merit.cuh"

namespace mfem {
namespace {

constexpr int kElementThreads = 128;
constexpr int kVertexThreads = 256;

__device__ __forceinline__ void load_vec3(const float *__restrict__ p, int i, float v[3]) {
    v[0] = p[3 * i + 0];
    v[1] = p[3 * i + 1];
    v[2] = p[3 * i + 2];
}

// Element outputs staged per warp in shared memory, so that the tet-major
// element blocks and rhs (which the assembly gathers per tet) leave in
// 16-byte stores of consecutive tets instead of 90 scalar stores 360 bytes
// apart.  Odd row strides keep the lanes' scalar writes free of bank
// conflicts.
constexpr int kElementWarps = kElementThreads / 32;
constexpr int kKeStride = kKeFloats + 1;
constexpr int kFeStride = kFeFloats + 1;
constexpr int kElementSmem = kElementWarps * 32 * (kKeStride + kFeStride) * (int)sizeof(float);
// grid of the fp64 pass: it loops over however many tets were listed
constexpr int kElementFp64Blocks = 304;

// Copies `count` floats of the warp's staged rows (row r = tet t0 + r, `per`
// floats a row, stride `stride` in shared memory) to dst = the first tet's
// output, 16 bytes a store where the destination allows.
template <int per, int stride>
__device__ __forceinline__ void warp_copy_out(const float *__restrict__ src, float *__restrict__ dst, int count,
                                              int lane) {
    const int n4 = count >> 2;
    float4 *d4 = reinterpret_cast<float4 *>(dst);
    for (int q = lane; q < n4; q += 32) {
        float v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = 4 * q + u;
            const int r = j / per;
            v[u] = src[r * stride + (j - r * per)];
        }
        d4[q] = make_float4(v[0], v[1], v[2], v[3]);
    }
    for (int j = 4 * n4 + lane; j < count; j += 32) {
        const int r = j / per;
        dst[j] = src[r * stride + (j - r * per)];
    }
}

// Everything one Newton iteration needs from tet t: the per-tet terms
// (component-major, straight to global memory) and the element blocks and
// rhs, written to ke [90] and fe [12] (shared-memory staging rows in the
// element kernel, the tet's global rows in the fp64 pass).  FP64 takes the
// polar decomposition and dS/dF in float64.  DIAG also writes H_s^-1 and
// g_lambda, which the step does not read (the local solve and the rhs use
// the cancellation-free form) but the stage diagnostics expose.  Returns
// det F in float32.
template <bool FP64, bool DIAG>
__device__ __forceinline__ float element_tet(const float *__restrict__ x, int energy, const TetViews &tv, int t,
                                             float *ke, float *fe) {
    const int T = tv.n_tets;
    const int4 tt = tv.tets[t];
    float xv[4][3];
    load_vec3(x, tt.x, xv[0]);
    load_vec3(x, tt.y, xv[1]);
    load_vec3(x, tt.z, xv[2]);
    load_vec3(x, tt.w, xv[3]);
    float Dm[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Dm[i][j] = tv.dminv[(size_t)t * 9 + i * 3 + j];
    float s[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = tv.stretch[(size_t)t * 6 + i];
    const float mu = tv.materials[(size_t)t * 3 + 0];
    const float lam = tv.materials[(size_t)t * 3 + 1];
    // rest volume 1/(6 det DmInv) (elastic_energy.py:143-145)
    const float vol = 1.0f / (6.0f * em::det3(Dm));

    float g_s[6], H_l[21];
    {
        float H_si[21];
        em::energy_terms(tv.energy_code ? (int)tv.energy_code[t] : energy, s, mu, lam, vol, g_s, H_l, H_si);
        if (DIAG) {
#pragma unroll
            for (int k = 0; k < 21; ++k) tv.H_si[(size_t)k * T + t] = H_si[k];
            // g_l = c + SYM H_s^-1 g_s (kernels.py:189-205): the second term
            // now, c added below
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                float acc = 0.0f;
#pragma unroll
                for (int j = 0; j < 6; ++j) acc += H_si[em::p21(i, j)] * g_s[j];
                tv.g_l[(size_t)i * T + t] = em::sym_w(i) * acc;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) tv.g_s[(size_t)i * T + t] = g_s[i];
#pragma unroll
    for (int k = 0; k < 21; ++k) tv.H_l[(size_t)k * T + t] = H_l[k];

    const float detF = em::deformation_det(xv, Dm);
    float c[6], G[6][12];
    if (FP64) em::element_geometry_t<double, true>(xv, Dm, s, c, G);
    else em::element_geometry_t<float, true>(xv, Dm, s, c, G);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        tv.c[(size_t)i * T + t] = c[i];
        if (DIAG) tv.g_l[(size_t)i * T + t] += c[i];
    }
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int col = 0; col < 12; ++col) tv.G[(size_t)(r * 12 + col) * T + t] = G[r][col];

    // H_l g_l = H_l c + INV_SYM g_s: the reference's product, without the
    // cancellation of H_l SYM H_s^-1 g_s (H_l = INV_SYM H_s INV_SYM), which
    // loses fp32 accuracy on tets whose H_s is nearly singular
    float w[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        float acc = em::inv_sym_w(i) * g_s[i];
#pragma unroll
        for (int j = 0; j < 6; ++j) acc += H_l[em::p21(i, j)] * c[j];
        w[i] = acc;
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        float P[6][3];  // H_l G_l
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
                float acc = 0.0f;
#pragma unroll
                for (int j = 0; j < 6; ++j) acc += H_l[em::p21(i, j)] * G[j][3 * l + b];
                P[i][b] = acc;
            }
#pragma unroll
        for (int b = 0; b < 3; ++b) {
            float acc = 0.0f;
#pragma unroll
            for (int i = 0; i < 6; ++i) acc += G[i][3 * l + b] * w[i];
            fe[3 * l + b] = acc;
        }
#pragma unroll
        for (int k = 0; k <= l; ++k) {
            float *blk = ke + ke_block(k, l) * 9;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) {
                    float acc = 0.0f;
#pragma unroll
                    for (int i = 0; i < 6; ++i) acc += G[i][3 * k + a] * P[i][b];
                    blk[a * 3 + b] = acc;
                }
        }
    }
    return detF;
}

// One thread per tet, in float32; tets with det F < 1e-3 are listed for
// element_fp64_kernel, which redoes them with the float64 polar path.
template <bool DIAG>
__global__ void __launch_bounds__(kElementThreads, 3)
    element_kernel(const float *__restrict__ x, int energy, TetViews tv) {
    extern __shared__ __align__(16) float s_stage[];
    const int T = tv.n_tets;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int t0 = blockIdx.x * blockDim.x + warp * 32;  // the warp's first tet
    if (t0 >= T) return;                                 // warp-uniform
    const int t = t0 + lane;
    float *const w_ke = s_stage + warp * 32 * kKeStride;                                   // [32][kKeStride]
    float *const w_fe = s_stage + kElementWarps * 32 * kKeStride + warp * 32 * kFeStride;  // [32][kFeStride]
    if (t < T) {
        const float detF = element_tet<false, DIAG>(x, energy, tv, t, w_ke + lane * kKeStride, w_fe + lane * kFeStride);
        if (!(detF >= em::kPolarFp64Det)) tv.degenerate[atomicAdd(tv.n_degenerate, 1u)] = t;
    }
    __syncwarp();
    const int nv = min(32, T - t0);
    warp_copy_out<kKeFloats, kKeStride>(w_ke, tv.Ke + (size_t)t0 * kKeFloats, nv * kKeFloats, lane);
    warp_copy_out<kFeFloats, kFeStride>(w_fe, tv.fe + (size_t)t0 * kFeFloats, nv * kFeFloats, lane);
}

// The listed near-degenerate or inverted tets again, with the polar
// decomposition and dS/dF in float64; overwrites the element kernel's
// float32 results of those tets.
template <bool DIAG>
__global__ void __launch_bounds__(kElementThreads)
    element_fp64_kernel(const float *__restrict__ x, int energy, TetViews tv) {
    const unsigned count = *tv.n_degenerate;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const int t = tv.degenerate[i];
        element_tet<true, DIAG>(x, energy, tv, t, tv.Ke + (size_t)t * kKeFloats, tv.fe + (size_t)t * kFeFloats);
    }
}

__global__ void __launch_bounds__(kElementThreads)
    initial_stretch_kernel(const float *__restrict__ rest_q, TetViews tv) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tv.n_tets) return;
    const int4 tt = tv.tets[t];
    float xv[4][3];
    load_vec3(rest_q, tt.x, xv[0]);
    load_vec3(rest_q, tt.y, xv[1]);
    load_vec3(rest_q, tt.z, xv[2]);
    load_vec3(rest_q, tt.w, xv[3]);
    float Dm[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) Dm[i][j] = tv.dminv[(size_t)t * 9 + i * 3 + j];
    float F[3][3], U[3][3], sig[3], V[3][3], sF[6];
    em::deformation_gradient(xv, Dm, F);
    em::polar_svd(F, U, sig, V);
    em::stretch_sym6(sig, V, sF);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        tv.stretch[(size_t)t * 6 + i] = sF[i];
        tv.lambda[(size_t)t * 6 + i] = 0.0f;
    }
}

__global__ void __launch_bounds__(kVertexThreads)
    predict_kernel(const float *__restrict__ q_in, const float *__restrict__ qd_in, float *q_out, float gx,
                   float gy, float gz, float dt, VertexViews vv) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= vv.n) return;
    float g[3] = {gx, gy, gz};
    if (vv.vertex_body) {
        // batched bodies: each body falls along its own gravity
        const float *bg = vv.body_gravity + 3 * vv.vertex_body[v];
        g[0] = bg[0];
        g[1] = bg[1];
        g[2] = bg[2];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float q = q_in[3 * v + a];
        const float qd = qd_in[3 * v + a];
        vv.x_tilde[3 * v + a] = q + qd * dt + g[a] * dt * dt / 2.0f;
        vv.x_start[3 * v + a] = q;
        q_out[3 * v + a] = q;
    }
}

// lambda and ds of tet t (local_solve_lambda, local_solve_stretch,
// kernels.py:252-283): the reference computes lambda = -H_l (g_l - G dx) and
// ds = -H_s^-1 (SYM lambda + g_s) with g_l = c + SYM H_s^-1 g_s and H_l =
// INV_SYM H_s INV_SYM.  With u = c - G dx these are exactly
//     lambda = -(H_l u + INV_SYM g_s),   ds = INV_SYM u,
// which is what is evaluated here: the reference's order forms SYM lambda +
// g_s as a difference of two large, nearly equal terms and multiplies it by
// H_s^-1, which amplifies fp32 rounding by cond(H_s) (above 1e4 for strongly
// stretched Neo-Hookean tets, where the trajectory then drifts from the exact
// one and diverges).  gdx = G dx.
__device__ __forceinline__ void local_tet(const TetViews &tv, const float *__restrict__ dx, int t, float nl[6],
                                          float ds[6], float gdx[6]) {
    const int T = tv.n_tets;
    const int4 tt = tv.tets[t];
    const int vid[4] = {tt.x, tt.y, tt.z, tt.w};
    float u[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        u[i] = tv.c[(size_t)i * T + t];
        gdx[i] = 0.0f;
    }
    // u = c - G dx, block by block (kernels.py:266-268)
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float d[3];
        load_vec3(dx, vid[k], d);
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            const float *g = tv.G + (size_t)(i * 12 + 3 * k) * T + t;
            const float gd = g[0] * d[0] + g[(size_t)T] * d[1] + g[(size_t)2 * T] * d[2];
            u[i] -= gd;
            gdx[i] += gd;
        }
    }
    float Hl[21];
#pragma unroll
    for (int k = 0; k < 21; ++k) Hl[k] = tv.H_l[(size_t)k * T + t];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        float acc = em::inv_sym_w(i) * tv.g_s[(size_t)i * T + t];
#pragma unroll
        for (int j = 0; j < 6; ++j) acc += Hl[em::p21(i, j)] * u[j];
        nl[i] = -acc;
        ds[i] = em::inv_sym_w(i) * u[i];
    }
}

__global__ void __launch_bounds__(kVertexThreads)
    local_solve_kernel(float *x, TetViews tv, VertexViews vv, int tet_blocks) {
    if ((int)blockIdx.x >= tet_blocks) {
        const int v = (blockIdx.x - tet_blocks) * blockDim.x + threadIdx.x;
        if (v >= vv.n) return;
#pragma unroll
        for (int a = 0; a < 3; ++a) x[3 * v + a] += vv.dx[3 * v + a];
        return;
    }
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tv.n_tets) return;
    float nl[6], ds[6], gdx[6];
    local_tet(tv, vv.dx, t, nl, ds, gdx);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        tv.stretch[(size_t)t * 6 + i] += ds[i];
        tv.lambda[(size_t)t * 6 + i] = nl[i];
    }
}

// The local solve ahead of the line search: x and s stay, lambda and ds are
// stored, and each block writes its sums of the merit function at (x, s)
// with the new lambda and of the slope (g_x - G^T lambda) . dx +
// (g_s + SYM lambda) . ds (solver.py:803-869, 893-915).
__global__ void __launch_bounds__(kVertexThreads)
    local_solve_deferred_kernel(const float *__restrict__ x, int energy, float dt, double inv_dt2, TetViews tv,
                                VertexViews vv, ContactViews cv, LineSearchWork w, int tet_blocks) {
    __shared__ double s_red[2][kVertexThreads / 32];
    double merit = 0.0, slope = 0.0;
    if ((int)blockIdx.x >= tet_blocks) {
        const int v = (blockIdx.x - tet_blocks) * blockDim.x + threadIdx.x;
        // contact: the energies and gradients the contact kernel left at x
        // (barrier_gradient + friction_gradient in the slope, solver.py:909)
        if (cv.on && v < cv.n_tris) merit += (double)cv.tri[(size_t)v * kTriData + 1];
        if (cv.on && v < vv.n) {
            merit += (double)cv.venergy[v];
            slope += (double)(cv.gtot[3 * v] * vv.dx[3 * v] + cv.gtot[3 * v + 1] * vv.dx[3 * v + 1] +
                              cv.gtot[3 * v + 2] * vv.dx[3 * v + 2]);
        }
        if (v < vv.n) {
            merit += vertex_merit(vv, x, v, 0.0f, inv_dt2);
            // g_x as in the assembly: m (x - x~)/dt^2 + (k x - k p)/dt^2
            const float dt2 = dt * dt;
            const float m = vv.mass[v];
            const float kp = vv.pin_k[v];
            float sl = 0.0f;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float xa = x[3 * v + a];
                const float gx = m * (xa - vv.x_tilde[3 * v + a]) / dt2 + (kp * xa + (-(kp * vv.pin_target[3 * v + a]))) / dt2;
                sl += gx * vv.dx[3 * v + a];
            }
            slope += sl;
        }
    } else {
        const int T = tv.n_tets;
        const int t = blockIdx.x * blockDim.x + threadIdx.x;
        if (t < T) {
            float nl[6], ds[6], gdx[6];
            local_tet(tv, vv.dx, t, nl, ds, gdx);
            float s[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                s[i] = tv.stretch[(size_t)t * 6 + i];
                tv.lambda[(size_t)t * 6 + i] = nl[i];
                w.ds[(size_t)i * T + t] = ds[i];
            }
            float Dm[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) Dm[i][j] = tv.dminv[(size_t)t * 9 + i * 3 + j];
            const float vol = 1.0f / (6.0f * em::det3(Dm));
            float lc = 0.0f, sl = 0.0f;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                lc += nl[i] * tv.c[(size_t)i * T + t];
                sl += (tv.g_s[(size_t)i * T + t] + em::sym_w(i) * nl[i]) * ds[i] - nl[i] * gdx[i];
            }
            merit = (double)em::elastic_energy(energy, s, tv.materials[(size_t)t * 3 + 0],
                                               tv.materials[(size_t)t * 3 + 1], vol) - (double)lc;
            slope = sl;
        }
    }
    merit = warp_sum(merit);
    slope = warp_sum(slope);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        s_red[0][wid] = merit;
        s_red[1][wid] = slope;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a0 = 0.0, a1 = 0.0;
        for (int k = 0; k < kVertexThreads / 32; ++k) {
            a0 += s_red[0][k];
            a1 += s_red[1][k];
        }
        w.local_partials[2 * blockIdx.x + 0] = a0;
        w.local_partials[2 * blockIdx.x + 1] = a1;
    }
}

__global__ void __launch_bounds__(kVertexThreads)
    velocity_kernel(const float *__restrict__ q_out, float *qd_out, float dt, VertexViews vv) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= vv.n) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) qd_out[3 * v + a] = (q_out[3 * v + a] - vv.x_start[3 * v + a]) / dt;
}

inline int blocks_for(int n, int threads) { return (n + threads - 1) / threads; }

}  // namespace

cudaError_t launch_initial_stretch(const float *rest_q, const TetViews &tv, cudaStream_t s) {
    if (tv.n_tets == 0) return cudaSuccess;
    initial_stretch_kernel<<<blocks_for(tv.n_tets, kElementThreads), kElementThreads, 0, s>>>(rest_q, tv);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_predict(const float *q_in, const float *qd_in, float *q_out, const float *gravity, float dt,
                           const VertexViews &vv, cudaStream_t s) {
    if (vv.n == 0) return cudaSuccess;
    predict_kernel<<<blocks_for(vv.n, kVertexThreads), kVertexThreads, 0, s>>>(q_in, qd_in, q_out, gravity[0],
                                                                               gravity[1], gravity[2], dt, vv);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t prepare_element_kernels() {
    cudaError_t e = cudaFuncSetAttribute(element_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kElementSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(element_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kElementSmem);
    return e;
}

cudaError_t launch_element(const float *x, int energy, const TetViews &tv, bool diagnostics, cudaStream_t s) {
    if (tv.n_tets == 0) return cudaSuccess;
    const int blocks = blocks_for(tv.n_tets, kElementThreads);
    cudaError_t e = cudaMemsetAsync(tv.n_degenerate, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    const int fix_blocks = std::min(blocks, kElementFp64Blocks);
    if (diagnostics) {
        element_kernel<true><<<blocks, kElementThreads, kElementSmem, s>>>(x, energy, tv);
        element_fp64_kernel<true><<<fix_blocks, kElementThreads, 0, s>>>(x, energy, tv);
    } else {
        element_kernel<false><<<blocks, kElementThreads, kElementSmem, s>>>(x, energy, tv);
        element_fp64_kernel<false><<<fix_blocks, kElementThreads, 0, s>>>(x, energy, tv);
    }
    count_launches(2);
    return cudaGetLastError();
}

cudaError_t launch_local_solve(float *x, const TetViews &tv, const VertexViews &vv, cudaStream_t s) {
    const int tb = blocks_for(tv.n_tets, kVertexThreads);
    const int vb = blocks_for(vv.n, kVertexThreads);
    if (tb + vb == 0) return cudaSuccess;
    local_solve_kernel<<<tb + vb, kVertexThreads, 0, s>>>(x, tv, vv, tb);
    count_launches(1);
    return cudaGetLastError();
}

int local_solve_blocks(int n_tets, int n_vertex_range) {
    return blocks_for(n_tets, kVertexThreads) + blocks_for(n_vertex_range, kVertexThreads);
}

cudaError_t launch_local_solve_deferred(const float *x, int energy, float dt, const TetViews &tv,
                                        const VertexViews &vv, const ContactViews &cv, const LineSearchWork &w,
                                        cudaStream_t s) {
    const int tb = blocks_for(tv.n_tets, kVertexThreads);
    const int vb = blocks_for(std::max(vv.n, cv.on ? cv.n_tris : 0), kVertexThreads);
    if (tb + vb == 0) return cudaSuccess;
    if (tb + vb > w.local_blocks) return cudaErrorInvalidValue;  // partials sized for fewer blocks
    const double inv_dt2 = 1.0 / ((double)dt * (double)dt);
    local_solve_deferred_kernel<<<tb + vb, kVertexThreads, 0, s>>>(x, energy, dt, inv_dt2, tv, vv, cv, w, tb);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_velocity(const float *q_out, float *qd_out, float dt, const VertexViews &vv, cudaStream_t s) {
    if (vv.n == 0) return cudaSuccess;
    velocity_kernel<<<blocks_for(vv.n, kVertexThreads), kVertexThreads, 0, s>>>(q_out, qd_out, dt, vv);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace mfem
