// Numeric assembly of the global system, without atomics.
//
// The reference builds G^T and H_lambda G as padded BSR matrices and forms
// H with bsr_mm, g with a transposed bsr_mv, then adds (M+Q)/dt^2 with
// bsr_axpy (src/mfem/refinement/solver.py:682-743).  Here the element kernel
// has already formed each tet's 10 upper 3x3 blocks of G^T H_l G and its rhs
// (H_l G)^T g_l; this kernel gathers them into the BSR slots.
//
// The symbolic phase sorted every (tet, k, l) contribution by destination
// slot and packed whole slots into warp-sized chunks.  One warp takes one
// chunk, each lane one contribution (lanes stride over the single slot of a
// chunk longer than 32), and a segmented shuffle reduction over lanes with the
// same slot yields each slot's sum in its first lane, in a fixed order, so
// the result is deterministic.  A diagonal slot's first lane also adds the
// mass/attachment term, inverts the block for the block-Jacobi
// preconditioner, and writes the vertex's rhs g = sum fe - g_x and the warm
// start dx = x~ - x.  With contact, the contribution lists also carry the
// surface tris' barrier blocks, and the diagonal lane adds the vertex's
// barrier and friction block and takes the contact gradients off the rhs.
#include "internal.h"

namespace mfem {
namespace {

constexpr int kAssembleThreads = 256;

__device__ __forceinline__ float seg_sum(float v, int lane, int last) {
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const float o = __shfl_down_sync(0xffffffffu, v, off);
        if (lane + off <= last) v += o;
    }
    return v;
}

__global__ void __launch_bounds__(kAssembleThreads)
    assemble_kernel(const float *__restrict__ x, float dt, float alpha_mass, float singular_threshold,
                    int use_precond, TetViews tv, VertexViews vv, BsrViews bv, ContactViews cv) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= bv.n_chunks) return;  // uniform per warp
    const int beg = bv.chunk_ptr[warp];
    const int end = bv.chunk_ptr[warp + 1];

    float v[9];
    float f[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int i = 0; i < 9; ++i) v[i] = 0.0f;
    int slot = -1;
    int code = 0;
    for (int c = beg + lane; c < end; c += 32) {
        code = __ldg(bv.contrib_code + c);
        slot = __ldg(bv.contrib_slot + c);
        if (code >= cv.tri_code_base) {
            // tri contact block w_i w_j k max(b'', 0) n n^T (contact.py:733-741)
            const int tc = code - cv.tri_code_base;
            const int tri = tc / 9;
            const int i = (tc - 9 * tri) / 3, j = tc - 9 * tri - 3 * i;
            const float *td = cv.tri + (size_t)tri * kTriData;
            const float hw = (td[7 + i] * td[7 + j]) * td[3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int bb = 0; bb < 3; ++bb) v[a * 3 + bb] += hw * (td[4 + a] * td[4 + bb]);
        } else if (code >= 0) {
            const int e = code >> 4;
            const int k = (code >> 2) & 3;
            const int l = code & 3;
            const bool tr = k > l;
            const float *blk = tv.Ke + (size_t)e * kKeFloats + ke_block(tr ? l : k, tr ? k : l) * 9;
            float b[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) b[i] = blk[i];
            if (tr) {
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int bb = 0; bb < 3; ++bb) v[a * 3 + bb] += b[bb * 3 + a];
            } else {
#pragma unroll
                for (int i = 0; i < 9; ++i) v[i] += b[i];
            }
            if (k == l) {
                const float *fp = tv.fe + (size_t)e * kFeFloats + 3 * k;
                f[0] += fp[0];
                f[1] += fp[1];
                f[2] += fp[2];
            }
        }
    }
    const unsigned peers = __match_any_sync(0xffffffffu, slot);
    const int last = 31 - __clz(peers);
#pragma unroll
    for (int i = 0; i < 9; ++i) v[i] = seg_sum(v[i], lane, last);
#pragma unroll
    for (int i = 0; i < 3; ++i) f[i] = seg_sum(f[i], lane, last);
    if (slot < 0 || lane != __ffs(peers) - 1) return;

    bool diag;
    int row = 0;
    if (code >= cv.tri_code_base) {
        const int tc = code - cv.tri_code_base;
        const int tri = tc / 9;
        const int i = (tc - 9 * tri) / 3, j = tc - 9 * tri - 3 * i;
        diag = (i == j);
        if (diag) row = cv.tris[3 * tri + i];
    } else if (code >= 0) {
        const int e = code >> 4;
        const int k = (code >> 2) & 3;
        const int l = code & 3;
        diag = (k == l);
        if (diag) {
            const int4 tt = tv.tets[e];
            row = (k == 0) ? tt.x : (k == 1) ? tt.y : (k == 2) ? tt.z : tt.w;
        }
    } else {
        diag = true;
        row = -code - 1;
    }
    if (diag) {
        // H += (M + Q) / dt^2 on the diagonal (solver.py:737-743)
        const float hd = alpha_mass * vv.hess_diag[row];
        v[0] += hd;
        v[4] += hd;
        v[8] += hd;
        // + the vertex's barrier and friction blocks (solver.py:745-779)
        float gc[3] = {0.0f, 0.0f, 0.0f};
        if (cv.on) {
#pragma unroll
            for (int i = 0; i < 9; ++i) v[i] += cv.vblock[9 * row + i];
#pragma unroll
            for (int a = 0; a < 3; ++a) gc[a] = cv.vgrad[3 * row + a];
            // tri barrier gradients scattered with the barycentric weights
            for (int k = cv.vt_ptr[row]; k < cv.vt_ptr[row + 1]; ++k) {
                const int code3 = cv.vt_code[k];
                const int tri = code3 / 3, corner = code3 - 3 * tri;
                const float *td = cv.tri + (size_t)tri * kTriData;
                const float gw = td[7 + corner] * td[2];
#pragma unroll
                for (int a = 0; a < 3; ++a) gc[a] += gw * td[4 + a];
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) cv.gtot[3 * row + a] = gc[a];
        }
        // block-Jacobi inverse, identity for |det| < threshold (kernels.py:32-53)
        const float c00 = v[4] * v[8] - v[5] * v[7];
        const float c01 = v[5] * v[6] - v[3] * v[8];
        const float c02 = v[3] * v[7] - v[4] * v[6];
        const float det = v[0] * c00 + v[1] * c01 + v[2] * c02;
        float *M = vv.Minv + (size_t)row * 9;
        if (!use_precond || !(fabsf(det) >= singular_threshold)) {
#pragma unroll
            for (int i = 0; i < 9; ++i) M[i] = (i % 4 == 0) ? 1.0f : 0.0f;
        } else {
            const float id = 1.0f / det;
            M[0] = c00 * id;
            M[1] = (v[2] * v[7] - v[1] * v[8]) * id;
            M[2] = (v[1] * v[5] - v[2] * v[4]) * id;
            M[3] = c01 * id;
            M[4] = (v[0] * v[8] - v[2] * v[6]) * id;
            M[5] = (v[2] * v[3] - v[0] * v[5]) * id;
            M[6] = c02 * id;
            M[7] = (v[1] * v[6] - v[0] * v[7]) * id;
            M[8] = (v[0] * v[4] - v[1] * v[3]) * id;
        }
        // g = sum fe - g_x, g_x = m (x - x~)/dt^2 + (k x - k p)/dt^2
        // (kernels.py:172-185; boundary_condition.py:73-80; solver.py:726-733, 946-947)
        const float dt2 = dt * dt;
        const float m = vv.mass[row];
        const float kp = vv.pin_k[row];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float xa = x[3 * row + a];
            const float xt = vv.x_tilde[3 * row + a];
            const float pt = vv.pin_target[3 * row + a];
            const float gx = m * (xa - xt) / dt2 + (kp * xa + (-(kp * pt))) / dt2;
            // - barrier and friction gradients (solver.py:734-735)
            vv.rhs[3 * row + a] = (f[a] - gx) - gc[a];
            vv.dx[3 * row + a] = xt - xa;
        }
    }
    float *out = bv.values + (size_t)slot * 9;
#pragma unroll
    for (int i = 0; i < 9; ++i) out[i] = v[i];
}

__global__ void true_residual_kernel(BsrViews bv, const float *__restrict__ rhs, const float *__restrict__ dx,
                                     double *out) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, bb = 0.0;
    if (row < bv.n) {
        double acc[3] = {0.0, 0.0, 0.0};
        for (int k = bv.row_ptr[row]; k < bv.row_ptr[row + 1]; ++k) {
            const int col = bv.col_idx[k];
            const float *h = bv.values + (size_t)k * 9;
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
                for (int b = 0; b < 3; ++b) acc[a] += (double)h[a * 3 + b] * (double)dx[3 * col + b];
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double g = rhs[3 * row + a];
            const double r = g - acc[a];
            rr += r * r;
            bb += g * g;
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rr += __shfl_down_sync(0xffffffffu, rr, off);
        bb += __shfl_down_sync(0xffffffffu, bb, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out + 0, rr);
        atomicAdd(out + 1, bb);
    }
}

}  // namespace

cudaError_t launch_assemble(const float *x, float dt, float singular_threshold, int use_precond,
                            const TetViews &tv, const VertexViews &vv, const BsrViews &bv, const ContactViews &cv,
                            cudaStream_t s) {
    if (bv.n_chunks == 0) return cudaSuccess;
    const int warps_per_block = kAssembleThreads / 32;
    const int blocks = (bv.n_chunks + warps_per_block - 1) / warps_per_block;
    // alpha = 1/(dt*dt) computed in double and rounded once, as the float32
    // bsr_axpy scale of the reference (solver.py:737-743)
    const float alpha_mass = (float)(1.0 / ((double)dt * (double)dt));
    assemble_kernel<<<blocks, kAssembleThreads, 0, s>>>(x, dt, alpha_mass, singular_threshold, use_precond, tv, vv,
                                                        bv, cv);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_true_residual(const BsrViews &bv, const VertexViews &vv, double *out, cudaStream_t s) {
    cudaError_t err = cudaMemsetAsync(out, 0, 2 * sizeof(double), s);
    if (err != cudaSuccess) return err;
    if (bv.n == 0) return cudaSuccess;
    true_residual_kernel<<<(bv.n + 255) / 256, 256, 0, s>>>(bv, vv.rhs, vv.dx, out);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace mfem
