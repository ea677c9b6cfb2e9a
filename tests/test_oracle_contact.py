"""The contact oracle (src/mfem/refinement/contact.py) on the CPU.

The tri geometry and the tri barrier are checked with the inputs and
assertions of the reference's own tests (tests/test_tri_contact.py:72-277).
The vertex barrier and the lagged friction, which no reference test covers,
are checked against finite differences of their own energies, and a solver
step with contact against a float64 sanity bar.
"""
import math

import numpy as np
import pytest

from mfem_gb300 import beams
from oracle import contact_oracle as C
from oracle import mfem_oracle as O

D0, D1, STIFFNESS, RADIUS, HALF_HEIGHT = 0.05, 0.2, 10.0, 0.1, 0.5
TRI = (np.array([0.0, 0.0, 0.0]), np.array([2.0, 0.0, 0.0]), np.array([0.0, 2.0, 0.0]))


def _closest(p0, p1):
    return C.closest_point_triangle_segment(*TRI, np.asarray(p0, float), np.asarray(p1, float))


def test_closest_face_interior():
    bary, q, d, hit = _closest((0.5, 0.5, 0.3), (0.5, 0.5, 1.3))
    assert hit == 0 and d == pytest.approx(0.3, abs=1e-6)
    assert bary == pytest.approx([0.5, 0.25, 0.25], abs=1e-6)
    assert q == pytest.approx([0.5, 0.5, 0.3], abs=1e-6)


def test_closest_edge_crossing():
    bary, q, d, hit = _closest((1.0, -1.0, 0.4), (1.0, 1.0, 0.4))
    assert hit == 0 and d == pytest.approx(0.4, abs=1e-6)
    assert bary.max() < 1.0 - 1e-6


def test_closest_vertex():
    bary, q, d, hit = _closest((-1.0, -1.0, 0.0), (-1.0, -1.0, 1.0))
    assert hit == 0 and d == pytest.approx(math.sqrt(2.0), abs=1e-6)
    assert bary == pytest.approx([1.0, 0.0, 0.0], abs=1e-6)


def test_segment_pierces_face():
    bary, q, d, hit = _closest((0.5, 0.5, -1.0), (0.5, 0.5, 1.0))
    assert hit == 1 and d == 0.0
    assert bary == pytest.approx([0.5, 0.25, 0.25], abs=1e-6)
    assert q == pytest.approx([0.5, 0.5, 0.0], abs=1e-6)


def _capsule(pos, rot=(0.0, 0.0, 0.0, 1.0)):
    shapes = [dict(type=C.SHAPE_CAPSULE, transform=[0, 0, 0, 0, 0, 0, 1], scale=[RADIUS, HALF_HEIGHT, 0.0], body=0)]
    body_q = np.array([list(pos) + list(rot)], dtype=np.float64)
    return shapes, body_q


def _tri_barrier(verts, capsule_pos, rot=(0.0, 0.0, 0.0, 1.0)):
    shapes, body_q = _capsule(capsule_pos, rot)
    co = C.ContactOracle(shapes, d0=D0, d1=D1, stiffness=STIFFNESS, tris=[[0, 1, 2]])
    x = np.asarray(verts, dtype=np.float64)
    E, g, blocks = co.tri_terms(x, body_q)
    H = np.zeros((3, 3, 3, 3))
    for i, j, b in blocks:
        H[i, j] += b
    d, bary, n, _ = C.tri_capsule_contact(x[0], x[1], x[2], shapes, body_q)
    return float(E[0]), g, H, d, bary, n


BIG_TRI = [(-3.0, -3.0, 0.0), (3.0, -3.0, 0.0), (0.0, 3.0, 0.0)]
GAP = 0.08
CAPSULE_ABOVE_CENTRE = (0.0, -1.0, GAP + RADIUS + HALF_HEIGHT)


def test_tri_barrier_catches_what_vertices_miss():
    shapes, body_q = _capsule(CAPSULE_ABOVE_CENTRE)
    assert min(C.vertex_distance(np.array(v), shapes, body_q)[0] for v in BIG_TRI) > D1
    e, g, H, d, bary, n = _tri_barrier(BIG_TRI, CAPSULE_ABOVE_CENTRE)
    assert d == pytest.approx(GAP, abs=1e-5)
    assert n == pytest.approx([0.0, 0.0, -1.0], abs=1e-5)
    assert e > 0.0 and bary.sum() == pytest.approx(1.0, abs=1e-6)
    assert (g[:, 2] > 0.0).all()
    total = g.sum(axis=0)
    assert np.abs(total[:2]).max() < 1e-4 * abs(total[2])


def test_tri_barrier_axis_through_face_is_deepest_penetration():
    e_touch = _tri_barrier(BIG_TRI, (0.0, -1.0, HALF_HEIGHT + RADIUS))[0]
    e_pierce, _, _, d, _, _ = _tri_barrier(BIG_TRI, (0.0, -1.0, 0.0))
    assert d == pytest.approx(-RADIUS, abs=1e-6)
    assert e_pierce > e_touch > 0.0


def _quat_axis_angle(axis, degrees):
    axis = np.asarray(axis, dtype=np.float64)
    axis /= np.linalg.norm(axis)
    half = np.radians(degrees) / 2.0
    return (*(np.sin(half) * axis), np.cos(half))


TRI_FD_CASES = [
    (BIG_TRI, (0.3, -0.8, GAP + RADIUS + HALF_HEIGHT), (0.1, 0.05, 0.0, 0.9937)),
    (BIG_TRI, (0.4, -3.3, 0.1), tuple(C.quat_mul(_quat_axis_angle((0.0, 0.0, 1.0), 15.0),
                                                  _quat_axis_angle((0.0, 1.0, 0.0), 90.0)))),
]


@pytest.mark.parametrize("verts,capsule_pos,rot", TRI_FD_CASES)
def test_tri_barrier_gradient_matches_finite_difference(verts, capsule_pos, rot):
    rot = tuple(np.asarray(rot) / np.linalg.norm(rot))
    e, g, H, d, bary, _ = _tri_barrier(verts, capsule_pos, rot)
    assert 0.0 < d < D1 and bary.max() < 1.0 - 1e-4
    v = np.asarray(verts, dtype=np.float64)
    fd = np.zeros((3, 3))
    h = 1e-3
    for i in range(3):
        for k in range(3):
            vp, vm = v.copy(), v.copy()
            vp[i, k] += h
            vm[i, k] -= h
            fd[i, k] = (_tri_barrier(vp, capsule_pos, rot)[0] - _tri_barrier(vm, capsule_pos, rot)[0]) / (2 * h)
    assert np.abs(g - fd).max() < 2e-2 * np.abs(fd).max()
    H9 = H.transpose(0, 2, 1, 3).reshape(9, 9)
    assert np.allclose(H9, H9.T, atol=1e-6 * np.abs(H9).max())
    assert np.linalg.eigvalsh(H9).min() > -1e-5 * np.abs(H9).max()


# ---------------------------------------------------------------------------
# vertex barrier and friction (no reference test: finite differences)
# ---------------------------------------------------------------------------


def test_barrier_is_c1_at_d0_and_zero_at_d1():
    c = C.barrier_coefficients(D0, D1)
    for eps in (1e-7, 1e-9):
        lo = C.barrier(D0 - eps, D0, D1, *c)
        hi = C.barrier(D0 + eps, D0, D1, *c)
        assert lo[0] == pytest.approx(hi[0], rel=1e-5) and lo[1] == pytest.approx(hi[1], rel=1e-4)
    assert C.barrier(D1, D0, D1, *c) == (0.0, 0.0, 0.0)
    assert C.barrier(D1 - 1e-9, D0, D1, *c)[0] == pytest.approx(0.0, abs=1e-12)


def _shapes_ground_and_capsule():
    # ground plane y = -0.05 (local +Z turned to world +Y), a capsule lying
    # along world x above the beam on a moving body
    q_plane = _quat_axis_angle((1.0, 0.0, 0.0), -90.0)
    q_caps = _quat_axis_angle((0.0, 1.0, 0.0), 90.0)
    shapes = [dict(type=C.SHAPE_PLANE, transform=[0.0, -0.05, 0.0, *q_plane], scale=[0, 0, 0], body=-1),
              dict(type=C.SHAPE_CAPSULE, transform=[0, 0, 0, *q_caps], scale=[0.05, 0.2, 0.0], body=0)]
    body_q = np.array([[0.5, 0.27, 0.1, 0.0, 0.0, 0.0, 1.0]])
    return shapes, body_q


def test_plane_and_capsule_distances():
    shapes, body_q = _shapes_ground_and_capsule()
    d, g, sid = C.vertex_distance(np.array([0.3, 0.0, 0.0]), shapes[:1], body_q)
    assert sid == 0 and d == pytest.approx(0.05) and g == pytest.approx([0.0, 1.0, 0.0])
    # beside the capsule's cylinder: distance to the axis minus the radius
    d, g, sid = C.vertex_distance(np.array([0.5, 0.2, 0.1]), shapes[1:], body_q)
    assert sid == 0 and d == pytest.approx(0.07 - 0.05) and g == pytest.approx([0.0, -1.0, 0.0])
    # beyond the end cap (axis from x = 0.3 to 0.7)
    d, _, _ = C.vertex_distance(np.array([0.8, 0.27, 0.1]), shapes[1:], body_q)
    assert d == pytest.approx(0.1 - 0.05)


def _vertex_energy(co, x, body_q, dt):
    return co.vertex_terms(x, body_q, dt)[0].sum()


@pytest.mark.parametrize("mu", [0.0, 0.4])
def test_vertex_barrier_and_friction_gradients_match_finite_differences(mu):
    shapes, body_q = _shapes_ground_and_capsule()
    co = C.ContactOracle(shapes, d0=0.01, d1=0.1, stiffness=1e3, friction_mu=mu, friction_eps_v=1e-1)
    rng = np.random.default_rng(0)
    x0 = np.array([[0.3, 0.0, 0.0], [0.5, 0.19, 0.12], [0.45, -0.03, 0.05], [0.62, 0.2, 0.08]])
    dt = 1.0 / 60.0
    co.begin_step(x0, body_q)
    if mu > 0.0:
        assert (co.force_lagged > 0).sum() >= 3
    x = x0 + rng.normal(0, 2e-3, x0.shape)
    E, g, H = co.vertex_terms(x, body_q, dt)
    h = 1e-6
    fd = np.zeros_like(x)
    for v in range(x.shape[0]):
        for k in range(3):
            xp, xm = x.copy(), x.copy()
            xp[v, k] += h
            xm[v, k] -= h
            fd[v, k] = (_vertex_energy(co, xp, body_q, dt) - _vertex_energy(co, xm, body_q, dt)) / (2 * h)
    assert np.abs(g - fd).max() <= 1e-5 * np.abs(fd).max()
    for v in range(x.shape[0]):
        assert np.linalg.eigvalsh(H[v]).min() >= -1e-9 * max(1.0, np.abs(H[v]).max())


def test_boundary_tris_are_closed_and_outward():
    mesh = beams.build_beam("cantilever", cells=(3, 2, 2))
    tris = C.boundary_tris(mesh.tet_indices, mesh.rest_q.astype(np.float64))
    x = mesh.rest_q.astype(np.float64)
    # every edge of a closed surface is shared by exactly two tris
    edges = {}
    for t in tris:
        for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
            edges[tuple(sorted((a, b)))] = edges.get(tuple(sorted((a, b))), 0) + 1
    assert set(edges.values()) == {2}
    # outward: the signed volume enclosed is the mesh volume
    vol = sum(np.dot(x[a], np.cross(x[b], x[c])) for a, b, c in tris) / 6.0
    Dm = np.stack([x[mesh.tet_indices[:, k]] - x[mesh.tet_indices[:, 0]] for k in (1, 2, 3)], axis=2)
    assert vol == pytest.approx(np.abs(np.linalg.det(Dm)).sum() / 6.0, rel=1e-9)


def test_oracle_step_with_ground_contact_stops_the_fall():
    """A free beam (nothing pinned) dropped 2 cm above a ground plane stays
    above it: the barrier holds every vertex at d > 0."""
    mesh = beams.build_beam("cantilever", cells=(4, 2, 2))
    mesh.particle_inv_mass[:] = 1.0 / mesh.particle_mass
    q_plane = _quat_axis_angle((1.0, 0.0, 0.0), -90.0)
    shapes = [dict(type=C.SHAPE_PLANE, transform=[0.0, -0.02, 0.0, *q_plane], scale=[0, 0, 0], body=-1)]
    tris = C.boundary_tris(mesh.tet_indices, mesh.rest_q.astype(np.float64))
    co = C.ContactOracle(shapes, d0=1e-3, d1=1e-2, stiffness=1e6, friction_mu=0.3, tris=tris)
    S = O.OracleSolver(mesh, dtype=np.float64, contact=co)
    q, qd = mesh.q0.astype(np.float64), mesh.qd0.astype(np.float64)
    for _ in range(30):
        q, qd = S.step(q, qd, mesh.spec.dt)
    assert q[:, 1].min() > -0.02
    assert np.abs(qd).max() < 0.5
