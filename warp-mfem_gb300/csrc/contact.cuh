// Contact against rigid shapes, fp32, host + device: signed distances to
// planes and capsules, the log barrier with its quadratic extrapolation, the
// lagged friction potential and the tri / capsule-axis closest points.
//
// Reference: src/mfem/refinement/contact.py (barrier :16-32, friction
// :34-60, compute_distance :98-164, lagged normal force :261-301, friction
// :304-354, tri geometry :417-622, tri barrier :684-741), the SDFs of
// src/mfem/ipc/distance.py:5-57 and the segment/segment closest points of
// src/mfem/collision.py:277-322.
//
// A pose is 7 floats (px, py, pz, qx, qy, qz, qw): x_world = p + R(q) x_local.
#pragma once

#include "element_math.cuh"

namespace mfem {
namespace ct {

constexpr int kShapePlane = 0;
constexpr int kShapeCapsule = 1;

MFEM_HD void quat_rotate(const float q[4], const float v[3], float out[3]) {
    // v + 2 w (u x v) + 2 u x (u x v), u = (qx, qy, qz)
    const float ux = q[0], uy = q[1], uz = q[2], w = q[3];
    const float tx = 2.0f * (uy * v[2] - uz * v[1]);
    const float ty = 2.0f * (uz * v[0] - ux * v[2]);
    const float tz = 2.0f * (ux * v[1] - uy * v[0]);
    out[0] = v[0] + w * tx + (uy * tz - uz * ty);
    out[1] = v[1] + w * ty + (uz * tx - ux * tz);
    out[2] = v[2] + w * tz + (ux * ty - uy * tx);
}

MFEM_HD void quat_rotate_inv(const float q[4], const float v[3], float out[3]) {
    const float qc[4] = {-q[0], -q[1], -q[2], q[3]};
    quat_rotate(qc, v, out);
}

MFEM_HD void quat_mul(const float a[4], const float b[4], float o[4]) {
    o[0] = a[3] * b[0] + a[0] * b[3] + a[1] * b[2] - a[2] * b[1];
    o[1] = a[3] * b[1] - a[0] * b[2] + a[1] * b[3] + a[2] * b[0];
    o[2] = a[3] * b[2] + a[0] * b[1] - a[1] * b[0] + a[2] * b[3];
    o[3] = a[3] * b[3] - a[0] * b[0] - a[1] * b[1] - a[2] * b[2];
}

// World pose of a shape: its body's pose times the shape's local pose
// (identity body for body < 0) (contact.py:120-126).
MFEM_HD void shape_world(const float *local, int body, const float *body_q, float X[7]) {
    if (body < 0) {
#pragma unroll
        for (int i = 0; i < 7; ++i) X[i] = local[i];
        return;
    }
    const float *B = body_q + 7 * body;
    float rp[3];
    quat_rotate(B + 3, local, rp);
    X[0] = B[0] + rp[0];
    X[1] = B[1] + rp[1];
    X[2] = B[2] + rp[2];
    quat_mul(B + 3, local + 3, X + 3);
}

// Signed distance of world point x to one shape and the world-space
// gradient; returns false for shape types that do not take part.
MFEM_HD bool shape_distance(int type, const float X[7], const float *scale, const float x[3], float &d,
                            float n[3]) {
    const float rel[3] = {x[0] - X[0], x[1] - X[1], x[2] - X[2]};
    float xl[3];
    quat_rotate_inv(X + 3, rel, xl);
    float nl[3] = {0.0f, 0.0f, 1.0f};
    if (type == kShapeCapsule) {
        // capsule along local +Z (ipc/distance.py:5-39)
        const float hh = scale[1];
        const float az = fminf(fmaxf(xl[2], -hh), hh);
        const float df[3] = {xl[0], xl[1], xl[2] - az};
        const float rho = sqrtf(df[0] * df[0] + df[1] * df[1] + df[2] * df[2]);
        if (rho > 1.0e-8f) {
            nl[0] = df[0] / rho;
            nl[1] = df[1] / rho;
            nl[2] = df[2] / rho;
        }
        d = rho - scale[0];
    } else if (type == kShapePlane) {
        // plane through the origin, normal local +Z (ipc/distance.py:42-57)
        d = xl[2];
    } else {
        return false;
    }
    quat_rotate(X + 3, nl, n);
    return true;
}

// Log barrier with quadratic extrapolation below d0 (contact.py:16-32);
// q = (b(d0), b'(d0), b''(d0)).
MFEM_HD void barrier(float d, float d0, float d1, const float q[3], float &e, float &de, float &d2e) {
    e = de = d2e = 0.0f;
    if (d < d1 && d > d0) {
        const float l = logf(d / d1);
        const float a = d - d1;
        e = -a * a * l;
        de = -(2.0f * a * l + a * a / d);
        d2e = -(2.0f * l + 4.0f * a / d - a * a / (d * d));
    } else if (d <= d0) {
        const float a = d - d0;
        e = q[0] + q[1] * a + 0.5f * q[2] * a * a;
        de = q[1] + q[2] * a;
        d2e = q[2];
    }
}

// Smoothed friction potential f0 and f1(y)/y (IPC's mollifier;
// contact.py:34-60), ev = eps_v dt.
MFEM_HD float friction_f0(float y, float ev) {
    if (y >= ev) return y;
    return -y * y * y / (3.0f * ev * ev) + y * y / ev + ev / 3.0f;
}

MFEM_HD float friction_f1_over_y(float y, float ev) {
    if (y >= ev) return 1.0f / fmaxf(y, 1.0e-12f);
    return -y / (ev * ev) + 2.0f / ev;
}

MFEM_HD float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

MFEM_HD void sub3(const float a[3], const float b[3], float o[3]) {
    o[0] = a[0] - b[0];
    o[1] = a[1] - b[1];
    o[2] = a[2] - b[2];
}

MFEM_HD void cross3(const float a[3], const float b[3], float o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

MFEM_HD float len3(const float a[3]) { return sqrtf(dot3(a, a)); }

MFEM_HD void set3(float o[3], float a, float b, float c) {
    o[0] = a;
    o[1] = b;
    o[2] = c;
}

// Barycentric weights of the point of tri abc closest to x (Ericson,
// "Real-Time Collision Detection" 5.1.5; contact.py:417-462).
MFEM_HD void closest_point_triangle_bary(const float x[3], const float a[3], const float b[3], const float c[3],
                                         float w[3]) {
    float ab[3], ac[3], ax[3];
    sub3(b, a, ab);
    sub3(c, a, ac);
    sub3(x, a, ax);
    const float d1 = dot3(ab, ax), d2 = dot3(ac, ax);
    if (d1 <= 0.0f && d2 <= 0.0f) return set3(w, 1.0f, 0.0f, 0.0f);
    float bx[3];
    sub3(x, b, bx);
    const float d3 = dot3(ab, bx), d4 = dot3(ac, bx);
    if (d3 >= 0.0f && d4 <= d3) return set3(w, 0.0f, 1.0f, 0.0f);
    float cx[3];
    sub3(x, c, cx);
    const float d5 = dot3(ab, cx), d6 = dot3(ac, cx);
    if (d6 >= 0.0f && d5 <= d6) return set3(w, 0.0f, 0.0f, 1.0f);
    const float vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0f && d1 >= 0.0f && d3 <= 0.0f) {
        const float v = d1 / (d1 - d3);
        return set3(w, 1.0f - v, v, 0.0f);
    }
    const float vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0f && d2 >= 0.0f && d6 <= 0.0f) {
        const float t = d2 / (d2 - d6);
        return set3(w, 1.0f - t, 0.0f, t);
    }
    const float va = d3 * d6 - d5 * d4;
    if (va <= 0.0f && (d4 - d3) >= 0.0f && (d5 - d6) >= 0.0f) {
        const float t = (d4 - d3) / ((d4 - d3) + (d5 - d6));
        return set3(w, 0.0f, 1.0f - t, t);
    }
    const float total = va + vb + vc;
    if (total <= 0.0f) return set3(w, 1.0f / 3.0f, 1.0f / 3.0f, 1.0f / 3.0f);
    const float v = vb / total, t = vc / total;
    set3(w, 1.0f - v - t, v, t);
}

// Segment p0p1 against tri abc (Moller-Trumbore; contact.py:465-494).
MFEM_HD bool segment_triangle_intersect(const float p0[3], const float p1[3], const float a[3], const float b[3],
                                        const float c[3], float w[3]) {
    float dir[3], e1[3], e2[3], pv[3];
    sub3(p1, p0, dir);
    sub3(b, a, e1);
    sub3(c, a, e2);
    cross3(dir, e2, pv);
    const float det = dot3(e1, pv);
    const float scale = len3(dir) * len3(e1) * len3(e2);
    if (fabsf(det) <= 1.0e-7f * scale + 1.0e-30f) return false;
    const float inv = 1.0f / det;
    float tv[3], qv[3];
    sub3(p0, a, tv);
    const float u = dot3(tv, pv) * inv;
    if (u < 0.0f || u > 1.0f) return false;
    cross3(tv, e1, qv);
    const float v = dot3(dir, qv) * inv;
    if (v < 0.0f || u + v > 1.0f) return false;
    const float t = dot3(e2, qv) * inv;
    if (t < 0.0f || t > 1.0f) return false;
    set3(w, 1.0f - u - v, u, v);
    return true;
}

// Closest points of segments p1q1 and p2q2 (Ericson 5.1.9;
// collision.py:277-322); returns the parameter s on the first.
MFEM_HD float closest_point_segment_segment(const float p1[3], const float q1[3], const float p2[3],
                                            const float q2[3], float c1[3], float c2[3]) {
    float d1[3], d2[3], r[3];
    sub3(q1, p1, d1);
    sub3(q2, p2, d2);
    sub3(p1, p2, r);
    const float a = dot3(d1, d1), e = dot3(d2, d2), f = dot3(d2, r);
    const float eps = 1.0e-8f;
    float s = 0.0f, t = 0.0f;
    if (a <= eps && e <= eps) {
    } else if (a <= eps) {
        t = fminf(fmaxf(f / e, 0.0f), 1.0f);
    } else {
        const float c = dot3(d1, r);
        if (e <= eps) {
            s = fminf(fmaxf(-c / a, 0.0f), 1.0f);
        } else {
            const float b = dot3(d1, d2);
            const float denom = a * e - b * b;
            s = denom > eps ? fminf(fmaxf((b * f - c * e) / denom, 0.0f), 1.0f) : 0.0f;
            t = (b * s + f) / e;
            if (t < 0.0f) {
                t = 0.0f;
                s = fminf(fmaxf(-c / a, 0.0f), 1.0f);
            } else if (t > 1.0f) {
                t = 1.0f;
                s = fminf(fmaxf((b - c) / a, 0.0f), 1.0f);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        c1[i] = p1[i] + s * d1[i];
        c2[i] = p2[i] + t * d2[i];
    }
    return s;
}

MFEM_HD void bary_point(const float w[3], const float a[3], const float b[3], const float c[3], float p[3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i) p[i] = w[0] * a[i] + w[1] * b[i] + w[2] * c[i];
}

// Closest points of tri abc and segment p0p1 over the five candidates
// (contact.py:497-551).  Returns the distance; w, q, hit as the reference.
MFEM_HD float closest_point_triangle_segment(const float a[3], const float b[3], const float c[3], const float p0[3],
                                             const float p1[3], float w[3], float q[3], bool &hit) {
    float p[3], t3[3];
    closest_point_triangle_bary(p0, a, b, c, w);
    set3(q, p0[0], p0[1], p0[2]);
    bary_point(w, a, b, c, p);
    sub3(p, p0, t3);
    float best = len3(t3);
    float wc[3];
    closest_point_triangle_bary(p1, a, b, c, wc);
    bary_point(wc, a, b, c, p);
    sub3(p, p1, t3);
    float d = len3(t3);
    if (d < best) {
        best = d;
        set3(w, wc[0], wc[1], wc[2]);
        set3(q, p1[0], p1[1], p1[2]);
    }
    float c1[3], c2[3];
    const float *ea[3] = {a, b, c};
    const float *eb[3] = {b, c, a};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float s = closest_point_segment_segment(ea[k], eb[k], p0, p1, c1, c2);
        sub3(c1, c2, t3);
        d = len3(t3);
        if (d < best) {
            best = d;
            if (k == 0) set3(w, 1.0f - s, s, 0.0f);
            else if (k == 1) set3(w, 0.0f, 1.0f - s, s);
            else set3(w, s, 0.0f, 1.0f - s);
            set3(q, c2[0], c2[1], c2[2]);
        }
    }
    float wh[3];
    hit = segment_triangle_intersect(p0, p1, a, b, c, wh);
    if (hit) {
        best = 0.0f;
        set3(w, wh[0], wh[1], wh[2]);
        bary_point(w, a, b, c, q);
    }
    return best;
}

}  // namespace ct
}  // namespace mfem
