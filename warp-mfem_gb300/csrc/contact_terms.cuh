// Contact terms of one vertex or one surface tri against the plan's rigid
// shapes, shared by the contact kernel (energy, gradient, Hessian at x), the
// local solve and the line search (energy at trial points).
// Reference: src/mfem/refinement/contact.py:98-164, 190-233, 304-354, 554-622.
#pragma once

#include "contact.cuh"
#include "internal.h"

namespace mfem {

// Minimum signed distance of x over the shapes, its world gradient and the
// shape index (-1 when no shape takes part) (compute_distance).
__device__ __forceinline__ float vertex_distance(const ContactViews &cv, const float x[3], float n[3], int &sid) {
    float d_min = 1.0e8f;
    sid = -1;
    n[0] = n[1] = n[2] = 0.0f;
    for (int s = 0; s < cv.n_shapes; ++s) {
        float X[7], d, g[3];
        ct::shape_world(cv.pose + 7 * s, cv.body[s], cv.body_q, X);
        if (!ct::shape_distance(cv.type[s], X, cv.scale + 3 * s, x, d, g)) continue;
        if (d < d_min) {
            d_min = d;
            n[0] = g[0];
            n[1] = g[1];
            n[2] = g[2];
            sid = s;
        }
    }
    return d_min;
}

// Tangential sliding of vertex v at x against its lagged normal, and the
// friction scale mu lambda_n (0 when the vertex has no lagged contact).
__device__ __forceinline__ float friction_sliding(const ContactViews &cv, const VertexViews &vv, int v,
                                                  const float x[3], float ut[3]) {
    const float lam = cv.force_lagged[v];
    const int sid = cv.shape_lagged[v];
    if (!(lam > 0.0f) || sid < 0) return 0.0f;
    const float mu = cv.mu[sid];
    if (!(mu > 0.0f)) return 0.0f;
    const float *nl = cv.normal_lagged + 3 * v;
    float u[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) u[i] = x[i] - vv.x_start[3 * v + i];
    const float un = u[0] * nl[0] + u[1] * nl[1] + u[2] * nl[2];
#pragma unroll
    for (int i = 0; i < 3; ++i) ut[i] = u[i] - un * nl[i];
    return mu * lam;
}

// Barrier + friction energy of vertex v at the point x
// (evaluate_barrier_energy_only, evaluate_friction_energy_only).
__device__ __forceinline__ float vertex_contact_energy(const ContactViews &cv, const VertexViews &vv, int v,
                                                       const float x[3], float ev) {
    float e_total = 0.0f;
    if (cv.n_shapes > 0) {
        float n[3];
        int sid;
        const float d = vertex_distance(cv, x, n, sid);
        if (d < cv.d1) {
            float e, de, d2e;
            ct::barrier(d, cv.d0, cv.d1, cv.q, e, de, d2e);
            e_total = cv.k * e;
        }
    }
    if (cv.friction) {
        float ut[3];
        const float scale = friction_sliding(cv, vv, v, x, ut);
        if (scale > 0.0f) e_total += scale * ct::friction_f0(ct::len3(ut), ev);
    }
    return e_total;
}

// Signed distance of tri abc to the nearest capsule, barycentric weights of
// its closest point, the direction the distance grows in and the shape
// (tri_capsule_contact, contact.py:554-622).
__device__ __forceinline__ float tri_contact_geometry(const ContactViews &cv, const float a[3], const float b[3],
                                                      const float c[3], float w[3], float n[3], int &sid) {
    float d_min = 1.0e8f;
    sid = -1;
    w[0] = w[1] = w[2] = 1.0f / 3.0f;
    n[0] = n[1] = n[2] = 0.0f;
    for (int s = 0; s < cv.n_shapes; ++s) {
        if (cv.type[s] != ct::kShapeCapsule) continue;
        float X[7];
        ct::shape_world(cv.pose + 7 * s, cv.body[s], cv.body_q, X);
        const float radius = cv.scale[3 * s + 0], hh = cv.scale[3 * s + 1];
        const float lo[3] = {0.0f, 0.0f, -hh}, hi[3] = {0.0f, 0.0f, hh};
        float p0[3], p1[3];
        ct::quat_rotate(X + 3, lo, p0);
        ct::quat_rotate(X + 3, hi, p1);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            p0[i] += X[i];
            p1[i] += X[i];
        }
        float wb[3], q[3];
        bool hit;
        const float dist = ct::closest_point_triangle_segment(a, b, c, p0, p1, wb, q, hit);
        const float d = dist - radius;
        if (d < d_min) {
            float p[3], nn[3];
            ct::bary_point(wb, a, b, c, p);
            if (!hit && dist > 1.0e-8f) {
#pragma unroll
                for (int i = 0; i < 3; ++i) nn[i] = (p[i] - q[i]) / dist;
            } else {
                // the axis pierces the tri: its normal, turned toward the
                // nearer axis end
                float e1[3], e2[3];
                ct::sub3(b, a, e1);
                ct::sub3(c, a, e2);
                ct::cross3(e1, e2, nn);
                const float l = ct::len3(nn);
                if (l > 1.0e-20f) {
                    nn[0] /= l;
                    nn[1] /= l;
                    nn[2] /= l;
                } else {
                    ct::set3(nn, 0.0f, 0.0f, 1.0f);
                }
                float axis[3], pp[3];
                ct::sub3(p1, p0, axis);
                ct::sub3(p, p0, pp);
                const float t = ct::dot3(pp, axis) / fmaxf(ct::dot3(axis, axis), 1.0e-20f);
                float toward[3] = {axis[0], axis[1], axis[2]};
                if (t < 0.5f) ct::set3(toward, -axis[0], -axis[1], -axis[2]);
                if (ct::dot3(nn, toward) < 0.0f) ct::set3(nn, -nn[0], -nn[1], -nn[2]);
            }
            d_min = d;
            ct::set3(w, wb[0], wb[1], wb[2]);
            ct::set3(n, nn[0], nn[1], nn[2]);
            sid = s;
        }
    }
    return d_min;
}

// Tri barrier energy of tri t at x + alpha dx (evaluate_tri_barrier_energy_only).
__device__ __forceinline__ float tri_contact_energy(const ContactViews &cv, const float *x, const float *dx, int t,
                                                    float alpha) {
    float p[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int vi = cv.tris[3 * t + k];
#pragma unroll
        for (int i = 0; i < 3; ++i) p[k][i] = fmaf(alpha, dx[3 * vi + i], x[3 * vi + i]);
    }
    float w[3], n[3];
    int sid;
    const float d = tri_contact_geometry(cv, p[0], p[1], p[2], w, n, sid);
    if (!(d < cv.d1)) return 0.0f;
    float e, de, d2e;
    ct::barrier(d, cv.d0, cv.d1, cv.q, e, de, d2e);
    return cv.k * e;
}

}  // namespace mfem
