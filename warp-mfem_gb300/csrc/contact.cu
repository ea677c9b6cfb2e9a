// Contact kernels of the global step.
//
//  contact_begin_kernel  start of a step: the normal force, normal and shape
//                        of each vertex's contact at x_start, frozen for the
//                        lagged friction (Contact.begin_step,
//                        src/mfem/refinement/contact.py:937-967, 261-301).
//  contact_kernel        each Newton iteration at x, one launch with two index
//                        ranges: per vertex the barrier (Gauss-Newton block
//                        k max(b'', 0) n n^T) and the friction (block
//                        mu lambda f1/y (I - n n^T)) (contact.py:98-164,
//                        190-233, 304-354); per surface tri the closest point
//                        to each capsule axis and its barrier (contact.py:
//                        554-741).  The assembly adds the vertex blocks on the
//                        diagonal, the tri blocks w_i w_j k max(b'', 0) n n^T
//                        on the tri's vertex pairs, and subtracts the
//                        gradients from the rhs.
#include "contact_terms.cuh"

namespace mfem {
namespace {

constexpr int kContactThreads = 128;

__device__ __forceinline__ void load3(const float *p, int i, float v[3]) {
    v[0] = p[3 * i + 0];
    v[1] = p[3 * i + 1];
    v[2] = p[3 * i + 2];
}

__global__ void __launch_bounds__(kContactThreads) contact_begin_kernel(ContactViews cv, VertexViews vv) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= vv.n) return;
    float x[3], n[3];
    load3(vv.x_start, v, x);
    int sid;
    const float d = vertex_distance(cv, x, n, sid);
    float lam = 0.0f;
    if (d < cv.d1) {
        float e, de, d2e;
        ct::barrier(d, cv.d0, cv.d1, cv.q, e, de, d2e);
        // -k b'(d): the outward normal force of the barrier
        lam = cv.k * fmaxf(-de, 0.0f);
    } else {
        n[0] = n[1] = n[2] = 0.0f;
        sid = -1;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) cv.normal_lagged[3 * v + i] = n[i];
    cv.force_lagged[v] = lam;
    cv.shape_lagged[v] = sid;
}

__global__ void __launch_bounds__(kContactThreads)
    contact_kernel(const float *__restrict__ x, float ev, ContactViews cv, VertexViews vv, int vertex_blocks) {
    if ((int)blockIdx.x < vertex_blocks) {
        const int v = blockIdx.x * blockDim.x + threadIdx.x;
        if (v >= vv.n) return;
        float xv[3];
        load3(x, v, xv);
        float E = 0.0f, g[3] = {0.0f, 0.0f, 0.0f}, H[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) H[i] = 0.0f;
        if (cv.n_shapes > 0) {
            float n[3];
            int sid;
            const float d = vertex_distance(cv, xv, n, sid);
            if (d < cv.d1) {
                float e, de, d2e;
                ct::barrier(d, cv.d0, cv.d1, cv.q, e, de, d2e);
                E = cv.k * e;
                const float gs = cv.k * de, hs = cv.k * fmaxf(d2e, 0.0f);
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    g[a] = gs * n[a];
#pragma unroll
                    for (int b = 0; b < 3; ++b) H[3 * a + b] = hs * (n[a] * n[b]);
                }
            }
        }
        if (cv.friction) {
            float ut[3];
            const float scale = friction_sliding(cv, vv, v, xv, ut);
            if (scale > 0.0f) {
                const float y = ct::len3(ut);
                const float f1y = ct::friction_f1_over_y(y, ev);
                const float *nl = cv.normal_lagged + 3 * v;
                E += scale * ct::friction_f0(y, ev);
                const float c = scale * f1y;
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    g[a] += c * ut[a];
#pragma unroll
                    for (int b = 0; b < 3; ++b) H[3 * a + b] += c * ((a == b ? 1.0f : 0.0f) - nl[a] * nl[b]);
                }
            }
        }
        cv.venergy[v] = E;
#pragma unroll
        for (int a = 0; a < 3; ++a) cv.vgrad[3 * v + a] = g[a];
#pragma unroll
        for (int i = 0; i < 9; ++i) cv.vblock[9 * v + i] = H[i];
        return;
    }
    const int t = (blockIdx.x - vertex_blocks) * blockDim.x + threadIdx.x;
    if (t >= cv.n_tris) return;
    float p[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) load3(x, cv.tris[3 * t + k], p[k]);
    float w[3], n[3];
    int sid;
    const float d = tri_contact_geometry(cv, p[0], p[1], p[2], w, n, sid);
    float e = 0.0f, de = 0.0f, d2e = 0.0f;
    if (d < cv.d1) ct::barrier(d, cv.d0, cv.d1, cv.q, e, de, d2e);
    float *o = cv.tri + (size_t)t * kTriData;
    o[0] = d;
    o[1] = cv.k * e;
    o[2] = cv.k * de;
    o[3] = cv.k * fmaxf(d2e, 0.0f);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        o[4 + i] = n[i];
        o[7 + i] = w[i];
    }
    o[10] = (float)sid;
    o[11] = 0.0f;
}

inline int blocks_for(int n, int threads) { return (n + threads - 1) / threads; }

}  // namespace

cudaError_t launch_contact_begin(const ContactViews &cv, const VertexViews &vv, cudaStream_t s) {
    if (!cv.on || !cv.friction || cv.n_shapes == 0 || vv.n == 0) return cudaSuccess;
    contact_begin_kernel<<<blocks_for(vv.n, kContactThreads), kContactThreads, 0, s>>>(cv, vv);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_contact(const float *x, float dt, const ContactViews &cv, const VertexViews &vv, cudaStream_t s) {
    if (!cv.on) return cudaSuccess;
    const int vb = blocks_for(vv.n, kContactThreads);
    const int tb = blocks_for(cv.n_tris, kContactThreads);
    if (vb + tb == 0) return cudaSuccess;
    // the friction's static threshold eps_v dt (contact.py:1045)
    const float ev = (float)((double)cv.eps_v * (double)dt);
    contact_kernel<<<vb + tb, kContactThreads, 0, s>>>(x, ev, cv, vv, vb);
    count_launches(1);
    return cudaGetLastError();
}

}  // namespace mfem
