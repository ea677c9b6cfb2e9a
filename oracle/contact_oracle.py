"""CPU oracle for the reference's contact terms -- TEST INFRASTRUCTURE ONLY.

Restates, in numpy, the per-vertex barrier against rigid shapes, the lagged
friction and the per-tri barrier against capsules of
src/mfem/refinement/contact.py (and the SDFs of src/mfem/ipc/distance.py, the
segment/segment closest points of src/mfem/collision.py:277-322):

====================================  ===========================================
function                              reference
====================================  ===========================================
barrier (log barrier + quadratic      contact.py:16-32
  extrapolation below d0)
friction_f0, friction_f1_over_y       contact.py:34-60
capsule_sdf, plane_sdf                ipc/distance.py:5-57
vertex distance over shapes           contact.py:98-164 (compute_distance)
vertex barrier (Gauss-Newton)         contact.py:190-233
lagged normal force (begin_step)      contact.py:261-301, 937-967
friction energy / gradient / Hessian  contact.py:304-354
closest point on a tri                contact.py:417-462
segment / tri intersection            contact.py:465-494
closest points tri / segment          contact.py:497-551; collision.py:277-322
tri / capsule contact                 contact.py:554-622
tri barrier                           contact.py:684-741
====================================  ===========================================

Warp's transforms (warp-lang 1.15.0, not part of the reference tree) are
restated from their published definition: a transform is (p, q) with the
quaternion q = (x, y, z, w); transform_point(T, v) = p + R(q) v,
transform_multiply(A, B) = (p_A + R(q_A) p_B, q_A q_B).

Shape types are this repository's own codes (SHAPE_PLANE, SHAPE_CAPSULE);
Newton's GeoType values are mapped to them by the binding.  Everything is
evaluated in the oracle's dtype; scalar paths follow the reference's branch
structure exactly.

Pinning: the tri geometry and tri barrier are checked against the reference's
own tests (tests/test_tri_contact.py), restated in
tests/test_oracle_contact.py.  The vertex barrier and the friction have no
reference test; they are pinned by finite differences of their own energies.
"""
from __future__ import annotations

import math

import numpy as np

SHAPE_PLANE = 0
SHAPE_CAPSULE = 1


# ---------------------------------------------------------------------------
# transforms
# ---------------------------------------------------------------------------


def quat_to_matrix(q):
    x, y, z, w = (float(v) for v in q)
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def quat_mul(a, b):
    x1, y1, z1, w1 = a
    x2, y2, z2, w2 = b
    return np.array([
        w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2,
        w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2,
        w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2,
        w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2,
    ])


def transform_multiply(A, B):
    """A, B: 7-vectors (px, py, pz, qx, qy, qz, qw)."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    p = A[:3] + quat_to_matrix(A[3:]) @ B[:3]
    return np.concatenate([p, quat_mul(A[3:], B[3:])])


def shape_world(shape, body_q):
    """World transform of a shape: its body's pose (identity for body < 0)
    times the shape's local transform (contact.py:120-126)."""
    body = shape["body"]
    if body >= 0:
        return transform_multiply(body_q[body], shape["transform"])
    return np.asarray(shape["transform"], dtype=np.float64)


# ---------------------------------------------------------------------------
# scalar pieces
# ---------------------------------------------------------------------------


def barrier(d, d0, d1, b_d0, db_d0, d2b_d0):
    """contact.py:16-32."""
    if d1 > d > d0:
        l = math.log(d / d1)
        e = -(d - d1) * (d - d1) * l
        de = -(2.0 * (d - d1) * l + (d - d1) * (d - d1) / d)
        d2e = -(2.0 * l + 4.0 * (d - d1) / d - (d - d1) * (d - d1) / (d * d))
        return e, de, d2e
    if d <= d0:
        return (b_d0 + db_d0 * (d - d0) + 0.5 * d2b_d0 * (d - d0) * (d - d0), db_d0 + d2b_d0 * (d - d0), d2b_d0)
    return 0.0, 0.0, 0.0


def barrier_coefficients(d0, d1):
    """The quadratic extrapolation's (b, b', b'') at d0 (contact.py:799)."""
    return barrier(d0, 0.0, d1, 0.0, 0.0, 0.0)


def friction_f0(y, ev):
    if y >= ev:
        return y
    return -y * y * y / (3.0 * ev * ev) + y * y / ev + ev / 3.0


def friction_f1_over_y(y, ev):
    if y >= ev:
        return 1.0 / max(y, 1.0e-12)
    return -y / (ev * ev) + 2.0 / ev


def capsule_sdf(p, radius, half_height):
    """(d, n) of a capsule along local +Z (ipc/distance.py:5-39)."""
    eps = 1.0e-8
    az = min(max(p[2], -half_height), half_height)
    diff = np.array([p[0], p[1], p[2] - az])
    rho = float(np.linalg.norm(diff))
    n = diff / rho if rho > eps else np.array([0.0, 0.0, 1.0])
    return rho - radius, n


def plane_sdf(p):
    return float(p[2]), np.array([0.0, 0.0, 1.0])


def vertex_distance(x, shapes, body_q):
    """Minimum signed distance of point x to the shapes, world gradient and
    shape index (-1 if none) (contact.py:98-164)."""
    d_min, g_min, sid = 1.0e8, np.zeros(3), -1
    for i, sh in enumerate(shapes):
        X = shape_world(sh, body_q)
        R = quat_to_matrix(X[3:])
        xl = R.T @ (np.asarray(x, dtype=np.float64) - X[:3])
        if sh["type"] == SHAPE_CAPSULE:
            d, nl = capsule_sdf(xl, sh["scale"][0], sh["scale"][1])
        elif sh["type"] == SHAPE_PLANE:
            d, nl = plane_sdf(xl)
        else:
            continue
        if d < d_min:
            d_min, g_min, sid = d, R @ nl, i
    return d_min, g_min, sid


def vertex_distances(x, shapes, body_q):
    """vertex_distance for every row of x at once: d [n], gradient [n, 3],
    shape [n] (the first shape reaching the minimum, as the scalar loop)."""
    x = np.asarray(x, dtype=np.float64)
    n = x.shape[0]
    d_min = np.full(n, 1.0e8)
    g_min = np.zeros((n, 3))
    sid = np.full(n, -1)
    for i, sh in enumerate(shapes):
        X = shape_world(sh, body_q)
        R = quat_to_matrix(X[3:])
        xl = (x - X[:3]) @ R
        if sh["type"] == SHAPE_CAPSULE:
            hh = sh["scale"][1]
            az = np.clip(xl[:, 2], -hh, hh)
            diff = np.stack([xl[:, 0], xl[:, 1], xl[:, 2] - az], axis=1)
            rho = np.linalg.norm(diff, axis=1)
            nl = np.where((rho > 1.0e-8)[:, None], diff / np.maximum(rho, 1e-300)[:, None], np.array([0.0, 0.0, 1.0]))
            d = rho - sh["scale"][0]
        elif sh["type"] == SHAPE_PLANE:
            d = xl[:, 2].copy()
            nl = np.tile(np.array([0.0, 0.0, 1.0]), (n, 1))
        else:
            continue
        better = d < d_min
        d_min = np.where(better, d, d_min)
        g_min = np.where(better[:, None], nl @ R.T, g_min)
        sid = np.where(better, i, sid)
    return d_min, g_min, sid


def barrier_vec(d, d0, d1, coeffs):
    """barrier() on an array: (e, de, d2e)."""
    d = np.asarray(d, dtype=np.float64)
    b0, b1, b2 = coeffs
    mid = (d < d1) & (d > d0)
    lo = d <= d0
    ds = np.where(mid, d, d1)
    l = np.log(ds / d1)
    a = ds - d1
    e = np.where(mid, -a * a * l, 0.0)
    de = np.where(mid, -(2.0 * a * l + a * a / ds), 0.0)
    d2e = np.where(mid, -(2.0 * l + 4.0 * a / ds - a * a / (ds * ds)), 0.0)
    t = d - d0
    e = np.where(lo, b0 + b1 * t + 0.5 * b2 * t * t, e)
    de = np.where(lo, b1 + b2 * t, de)
    d2e = np.where(lo, b2, d2e)
    return e, de, d2e


# ---------------------------------------------------------------------------
# tri geometry
# ---------------------------------------------------------------------------


def closest_point_triangle_bary(x, a, b, c):
    """contact.py:417-462 (Ericson, Real-Time Collision Detection 5.1.5)."""
    ab, ac, ax = b - a, c - a, x - a
    d1, d2 = ab @ ax, ac @ ax
    if d1 <= 0.0 and d2 <= 0.0:
        return np.array([1.0, 0.0, 0.0])
    bx = x - b
    d3, d4 = ab @ bx, ac @ bx
    if d3 >= 0.0 and d4 <= d3:
        return np.array([0.0, 1.0, 0.0])
    cx = x - c
    d5, d6 = ab @ cx, ac @ cx
    if d6 >= 0.0 and d5 <= d6:
        return np.array([0.0, 0.0, 1.0])
    vc = d1 * d4 - d3 * d2
    if vc <= 0.0 and d1 >= 0.0 and d3 <= 0.0:
        v = d1 / (d1 - d3)
        return np.array([1.0 - v, v, 0.0])
    vb = d5 * d2 - d1 * d6
    if vb <= 0.0 and d2 >= 0.0 and d6 <= 0.0:
        w = d2 / (d2 - d6)
        return np.array([1.0 - w, 0.0, w])
    va = d3 * d6 - d5 * d4
    if va <= 0.0 and (d4 - d3) >= 0.0 and (d5 - d6) >= 0.0:
        w = (d4 - d3) / ((d4 - d3) + (d5 - d6))
        return np.array([0.0, 1.0 - w, w])
    total = va + vb + vc
    if total <= 0.0:
        return np.array([1.0, 1.0, 1.0]) / 3.0
    v, w = vb / total, vc / total
    return np.array([1.0 - v - w, v, w])


def segment_triangle_intersect(p0, p1, a, b, c):
    """contact.py:465-494 (Moller-Trumbore on a segment)."""
    direction = p1 - p0
    e1, e2 = b - a, c - a
    pv = np.cross(direction, e2)
    det = e1 @ pv
    scale = np.linalg.norm(direction) * np.linalg.norm(e1) * np.linalg.norm(e2)
    if abs(det) <= 1.0e-7 * scale + 1.0e-30:
        return 0, np.zeros(3)
    inv = 1.0 / det
    tv = p0 - a
    u = (tv @ pv) * inv
    if u < 0.0 or u > 1.0:
        return 0, np.zeros(3)
    qv = np.cross(tv, e1)
    v = (direction @ qv) * inv
    if v < 0.0 or u + v > 1.0:
        return 0, np.zeros(3)
    t = (e2 @ qv) * inv
    if t < 0.0 or t > 1.0:
        return 0, np.zeros(3)
    return 1, np.array([1.0 - u - v, u, v])


def closest_point_segment_segment(p1, q1, p2, q2):
    """collision.py:277-322 (Ericson 5.1.9): (c1, c2, s)."""
    d1, d2, r = q1 - p1, q2 - p2, p1 - p2
    a, e, f = d1 @ d1, d2 @ d2, d2 @ r
    eps = 1.0e-8
    if a <= eps and e <= eps:
        s = t = 0.0
    elif a <= eps:
        s = 0.0
        t = min(max(f / e, 0.0), 1.0)
    else:
        c = d1 @ r
        if e <= eps:
            t = 0.0
            s = min(max(-c / a, 0.0), 1.0)
        else:
            b = d1 @ d2
            denom = a * e - b * b
            s = min(max((b * f - c * e) / denom, 0.0), 1.0) if denom > eps else 0.0
            t = (b * s + f) / e
            if t < 0.0:
                t = 0.0
                s = min(max(-c / a, 0.0), 1.0)
            elif t > 1.0:
                t = 1.0
                s = min(max((b - c) / a, 0.0), 1.0)
    return p1 + s * d1, p2 + t * d2, s


def closest_point_triangle_segment(a, b, c, p0, p1):
    """contact.py:497-551: (bary on the tri, point on the segment, distance, hit)."""
    best_bary = closest_point_triangle_bary(p0, a, b, c)
    best_q = p0
    best_d = np.linalg.norm(best_bary[0] * a + best_bary[1] * b + best_bary[2] * c - p0)
    bary = closest_point_triangle_bary(p1, a, b, c)
    d = np.linalg.norm(bary[0] * a + bary[1] * b + bary[2] * c - p1)
    if d < best_d:
        best_d, best_bary, best_q = d, bary, p1
    for (u, v, make) in ((a, b, lambda s: np.array([1.0 - s, s, 0.0])),
                         (b, c, lambda s: np.array([0.0, 1.0 - s, s])),
                         (c, a, lambda s: np.array([s, 0.0, 1.0 - s]))):
        c1, c2, s = closest_point_segment_segment(u, v, p0, p1)
        d = np.linalg.norm(c1 - c2)
        if d < best_d:
            best_d, best_bary, best_q = d, make(s), c2
    hit, hb = segment_triangle_intersect(p0, p1, a, b, c)
    if hit == 1:
        best_d, best_bary = 0.0, hb
        best_q = hb[0] * a + hb[1] * b + hb[2] * c
    return best_bary, best_q, float(best_d), hit


def tri_capsule_contact(a, b, c, shapes, body_q):
    """contact.py:554-622: (d, bary, n, shape) over the capsule shapes."""
    d_min, bary_min, n_min, id_min = 1.0e8, np.array([1.0, 1.0, 1.0]) / 3.0, np.zeros(3), -1
    for i, sh in enumerate(shapes):
        if sh["type"] != SHAPE_CAPSULE:
            continue
        X = shape_world(sh, body_q)
        R = quat_to_matrix(X[3:])
        radius, hh = sh["scale"][0], sh["scale"][1]
        p0 = X[:3] + R @ np.array([0.0, 0.0, -hh])
        p1 = X[:3] + R @ np.array([0.0, 0.0, hh])
        bary, q, dist, hit = closest_point_triangle_segment(a, b, c, p0, p1)
        d = dist - radius
        if d < d_min:
            p = bary[0] * a + bary[1] * b + bary[2] * c
            if hit == 0 and dist > 1.0e-8:
                n = (p - q) / dist
            else:
                n = np.cross(b - a, c - a)
                nl = np.linalg.norm(n)
                n = n / nl if nl > 1.0e-20 else np.array([0.0, 0.0, 1.0])
                axis = p1 - p0
                t = ((p - p0) @ axis) / max(axis @ axis, 1.0e-20)
                toward = axis if t >= 0.5 else -axis
                if n @ toward < 0.0:
                    n = -n
            d_min, bary_min, n_min, id_min = d, bary, n, i
    return d_min, bary_min, n_min, id_min


# ---------------------------------------------------------------------------
# the contact terms of one Newton iteration
# ---------------------------------------------------------------------------


class ContactOracle:
    """Contact state of one solver: shapes, lagged friction snapshot and the
    evaluation of energy, gradient and Hessian blocks at x."""

    def __init__(self, shapes, d0=1.0e-2, d1=1.0e-1, stiffness=1.0e7, friction_mu=0.0, friction_eps_v=1.0e-3,
                 tris=None, tri_contact=True):
        self.shapes = [dict(type=int(s["type"]), transform=np.asarray(s["transform"], dtype=np.float64),
                            scale=np.asarray(s["scale"], dtype=np.float64), body=int(s["body"])) for s in shapes]
        mu = np.asarray(friction_mu, dtype=np.float64)
        self.mu = np.full(len(self.shapes), float(mu)) if mu.ndim == 0 else mu
        self.d0, self.d1, self.k, self.eps_v = float(d0), float(d1), float(stiffness), float(friction_eps_v)
        self.coeffs = barrier_coefficients(self.d0, self.d1)
        self.tris = None if tris is None else np.asarray(tris, dtype=np.int64)
        self.tri_contact = bool(tri_contact) and self.tris is not None and len(self.tris) > 0
        self.x_start = None
        self.normal_lagged = None
        self.force_lagged = None
        self.shape_lagged = None

    def begin_step(self, x, body_q):
        """contact.py:937-967: snapshot x_start and, when any shape has
        friction, the lagged normal force, normal and shape."""
        n = x.shape[0]
        self.x_start = np.array(x, dtype=np.float64)
        if self.normal_lagged is None:
            self.normal_lagged = np.zeros((n, 3))
            self.force_lagged = np.zeros(n)
            self.shape_lagged = np.full(n, -1)
        if len(self.shapes) == 0 or self.mu.max() <= 0.0:
            return
        d, g, sid = vertex_distances(x, self.shapes, body_q)
        _, de, _ = barrier_vec(d, self.d0, self.d1, self.coeffs)
        near = d < self.d1
        self.force_lagged = np.where(near, self.k * np.maximum(-de, 0.0), 0.0)
        self.normal_lagged = np.where(near[:, None], g, 0.0)
        self.shape_lagged = np.where(near, sid, -1)

    def vertex_terms(self, x, body_q, dt):
        """Per-vertex barrier and friction: energy [n], gradient [n, 3],
        diagonal Hessian blocks [n, 3, 3] (contact.py:190-233, 304-354)."""
        x = np.asarray(x, dtype=np.float64)
        n = x.shape[0]
        E, g, H = np.zeros(n), np.zeros((n, 3)), np.zeros((n, 3, 3))
        ev = self.eps_v * dt
        if len(self.shapes) > 0:
            d, gd, _ = vertex_distances(x, self.shapes, body_q)
            e, de, d2e = barrier_vec(d, self.d0, self.d1, self.coeffs)
            near = d < self.d1
            E += np.where(near, self.k * e, 0.0)
            g += np.where(near[:, None], self.k * de[:, None] * gd, 0.0)
            H += np.where(near[:, None, None], self.k * np.maximum(d2e, 0.0)[:, None, None]
                          * gd[:, :, None] * gd[:, None, :], 0.0)
        if self.force_lagged is not None and len(self.shapes) > 0:
            sid = self.shape_lagged
            mu = np.where(sid >= 0, self.mu[np.maximum(sid, 0)], 0.0)
            act = (self.force_lagged > 0.0) & (sid >= 0) & (mu > 0.0)
            if act.any():
                nv = self.normal_lagged
                u = x - self.x_start
                ut = u - np.sum(u * nv, axis=1)[:, None] * nv
                y = np.linalg.norm(ut, axis=1)
                scale = mu * self.force_lagged
                f1y = np.where(y >= ev, 1.0 / np.maximum(y, 1.0e-12), -y / (ev * ev) + 2.0 / ev) if ev > 0 else \
                    1.0 / np.maximum(y, 1.0e-12)
                f0 = np.where(y >= ev, y, -y * y * y / (3.0 * ev * ev) + y * y / ev + ev / 3.0) if ev > 0 else y
                E += np.where(act, scale * f0, 0.0)
                g += np.where(act[:, None], (scale * f1y)[:, None] * ut, 0.0)
                P = np.eye(3)[None] - nv[:, :, None] * nv[:, None, :]
                H += np.where(act[:, None, None], (scale * f1y)[:, None, None] * P, 0.0)
        return E, g, H

    def tri_terms(self, x, body_q):
        """Per-tri barrier against capsules: energy [m], vertex gradient
        [n, 3] (scattered with the barycentric weights) and the blocks
        [(vi, vj, 3x3)] (contact.py:684-741)."""
        n = x.shape[0]
        g = np.zeros((n, 3))
        E = np.zeros(0 if self.tris is None else len(self.tris))
        blocks = []
        if not self.tri_contact:
            return E, g, blocks
        far = self._far_tris(x, body_q)
        for t, (i0, i1, i2) in enumerate(self.tris):
            if far[t]:
                # provably d >= d1 for every capsule: zero energy, gradient
                # and blocks, as the full evaluation gives
                continue
            d, w, nv, _ = tri_capsule_contact(x[i0], x[i1], x[i2], self.shapes, body_q)
            e = de = d2e = 0.0
            if d < self.d1:
                e, de, d2e = barrier(d, self.d0, self.d1, *self.coeffs)
            E[t] = self.k * e
            gt = self.k * de * nv
            h = self.k * max(d2e, 0.0) * np.outer(nv, nv)
            idx = (i0, i1, i2)
            for a in range(3):
                g[idx[a]] += w[a] * gt
                for b in range(3):
                    blocks.append((idx[a], idx[b], (w[a] * w[b]) * h))
        return E, g, blocks

    def _far_tris(self, x, body_q):
        """Tris whose distance to every capsule is provably >= d1: the
        nearest vertex's distance to the axis segment minus the longest edge
        minus the radius."""
        x = np.asarray(x, dtype=np.float64)
        a, b, c = x[self.tris[:, 0]], x[self.tris[:, 1]], x[self.tris[:, 2]]
        edge = np.maximum(np.maximum(np.linalg.norm(b - a, axis=1), np.linalg.norm(c - b, axis=1)),
                          np.linalg.norm(a - c, axis=1))
        far = np.ones(len(self.tris), dtype=bool)
        for sh in self.shapes:
            if sh["type"] != SHAPE_CAPSULE:
                continue
            X = shape_world(sh, body_q)
            R = quat_to_matrix(X[3:])
            hh = sh["scale"][1]
            p0 = X[:3] + R @ np.array([0.0, 0.0, -hh])
            axis = R @ np.array([0.0, 0.0, 2.0 * hh])
            dmin = np.full(len(self.tris), np.inf)
            for v in (a, b, c):
                t = np.clip(((v - p0) @ axis) / max(axis @ axis, 1e-300), 0.0, 1.0)
                dmin = np.minimum(dmin, np.linalg.norm(v - (p0 + t[:, None] * axis), axis=1))
            far &= dmin - edge - sh["scale"][0] >= self.d1
        return far

    def energy(self, x, body_q, dt):
        """Barrier + friction energy at x (contact.py:1050-1106)."""
        Ev, _, _ = self.vertex_terms(x, body_q, dt)
        Et, _, _ = self.tri_terms(x, body_q)
        return float(Ev.sum() + Et.sum())


def boundary_tris(tets, x):
    """Surface triangles of a tet mesh (faces that belong to one tet),
    ordered (sorted by their vertex triple) and oriented with the outward
    normal (b - a) x (c - a)."""
    tets = np.asarray(tets, dtype=np.int64)
    faces = {}
    local = ((1, 2, 3, 0), (0, 3, 2, 1), (0, 1, 3, 2), (0, 2, 1, 3))
    for t in tets:
        for a, b, c, opp in local:
            f = (t[a], t[b], t[c])
            key = tuple(sorted(f))
            if key in faces:
                faces[key] = None
            else:
                faces[key] = (f, t[opp])
    out = []
    for key in sorted(k for k, v in faces.items() if v is not None):
        (a, b, c), opp = faces[key]
        nrm = np.cross(x[b] - x[a], x[c] - x[a])
        if nrm @ (x[opp] - x[a]) > 0.0:
            b, c = c, b
        out.append((a, b, c))
    return np.asarray(out, dtype=np.int32).reshape(-1, 3)
