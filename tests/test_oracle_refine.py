"""The refinement oracle on CPU: the reference's scoring known answers and the
properties its whole-run tests check.

Scoring: tests/test_refine_scoring.py of the reference (two tets sharing the
face (0, 1, 2), h_min = 0.1, d1 = 0.2, capsule shapes), restated against
oracle.refine_oracle's geometric and tri passes.  Whole passes:
tests/test_refinement.py of the reference (rest volume conserved, no orphaned
vertex, the mesh grows, growth only on refining passes), plus the invariants
of the deterministic selection (no tet holds two split edges, no hanging
vertex, independent of the tet order).
"""
import numpy as np
import pytest

from oracle import refine_oracle as ro
from tests.refine_cases import deformed, grid_mesh, hanging_edges, mesh_from

H_MIN = 0.1
D1 = 0.2
Q2 = np.array([(0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.3, 0.6, 0.0), (0.3, 0.2, 0.6), (0.3, 0.2, -0.6)],
              dtype=np.float32)
T2 = np.array([(0, 1, 2, 3), (0, 1, 2, 4)], dtype=np.int32)


def _dm_inv(q, tets):
    return ro.inverse3_f32(ro.edge_matrix(q, tets.astype(np.int64)))


def _tet_pass(q, tets, energy, distance=None, shape_id=None, shape_type=(ro.SHAPE_CAPSULE,), inv_mass=None,
              elastic_stats=(0.0, 0.0)):
    """geometric_scores with the reference test's defaults (_run_tet_pass,
    tests/test_refine_scoring.py:39-67): mu 1, weights 1, absolute density;
    returns {(a, b): score} over the registered (non-kinematic) edges."""
    q = np.asarray(q, dtype=np.float32)
    n = q.shape[0]
    et = ro.EdgeTable(tets, n)
    cfg = ro.RefineConfig(scoring="geometric", min_edge_length=H_MIN, contact_d1=D1)
    inv = np.ones(n, np.float32) if inv_mass is None else np.asarray(inv_mass, np.float32)
    dist = np.full(n, 1.0e8, np.float32) if distance is None else np.asarray(distance, np.float32)
    sid = np.full(n, -1) if shape_id is None else np.asarray(shape_id)
    mats = np.ones((tets.shape[0], 3), np.float32)
    score, elig = ro.geometric_scores(et, q, tets, inv, np.asarray(energy, np.float32), mats, _dm_inv(q, tets), dist,
                                      sid, np.asarray(shape_type), cfg, elastic_stats=elastic_stats)
    return et, score, {(int(et.slot_row[s]), int(et.col_idx[s])): float(score[s]) for s in np.nonzero(elig)[0]}


def test_scores_are_per_edge_maxima_not_sums():
    _, _, one = _tet_pass(Q2, T2, energy=[1.0, 0.0])
    _, _, both = _tet_pass(Q2, T2, energy=[1.0, 1.0])
    for e in [(0, 1), (0, 2), (1, 2)]:
        assert one[e] > 0.0
        assert both[e] == pytest.approx(one[e], rel=1e-5)
    assert one[(0, 4)] == 0.0 and one[(1, 4)] == 0.0 and one[(2, 4)] == 0.0


def test_longest_edge_of_tet_scores_highest_and_score_is_dimensionless():
    _, _, sc = _tet_pass(Q2, T2, energy=[1.0, 1.0])
    lengths = {e: np.linalg.norm(Q2[e[0]] - Q2[e[1]]) for e in sc}
    longest = max(lengths, key=lengths.get)
    assert longest == (0, 1)
    assert sc[longest] == max(sc.values())
    Dm = np.stack([Q2[1] - Q2[0], Q2[2] - Q2[0], Q2[3] - Q2[0]], axis=1).astype(np.float64)
    vol = abs(np.linalg.det(Dm)) / 6.0
    assert sc[longest] == pytest.approx((lengths[longest] / H_MIN) * 1.0 / vol, rel=1e-4)


def test_short_edges_are_registered_but_never_candidates():
    _, _, sc = _tet_pass(Q2 * 0.15, T2, energy=[1.0, 1.0])
    assert len(sc) == 9
    assert all(v == 0.0 for v in sc.values())


def test_fully_kinematic_edges_are_excluded():
    _, _, sc = _tet_pass(Q2, T2, energy=[1.0, 1.0], inv_mass=[0.0, 0.0, 1.0, 1.0, 1.0])
    assert (0, 1) not in sc
    assert (0, 2) in sc


def test_vertex_contact_counts_capsules_only():
    n = Q2.shape[0]
    dist = np.full(n, 1.0e8)
    dist[3] = 0.5 * D1
    sid = np.full(n, -1)
    sid[3] = 0
    _, _, capsule = _tet_pass(Q2, T2, energy=[0.0, 0.0], distance=dist, shape_id=sid,
                              shape_type=(ro.SHAPE_CAPSULE,))
    _, _, plane = _tet_pass(Q2, T2, energy=[0.0, 0.0], distance=dist, shape_id=sid, shape_type=(ro.SHAPE_PLANE,))
    touching = [(0, 3), (1, 3), (2, 3)]
    for e in touching:
        assert capsule[e] > 0.0
        assert plane[e] == 0.0
    for e in capsule:
        if e not in touching:
            assert capsule[e] == 0.0
    dist[3] = -0.5 * D1
    _, _, pen = _tet_pass(Q2, T2, energy=[0.0, 0.0], distance=dist, shape_id=sid)
    assert pen[(0, 3)] > capsule[(0, 3)]


def test_tri_contact_promotes_edge_nearest_closest_point():
    q = np.array([(0.0, 0.0, 0.0), (1.0, 0.0, 0.0), (0.5, np.sqrt(3) / 2, 0.0), (0.5, 0.3, 0.8)], dtype=np.float32)
    tets = np.array([(0, 1, 2, 3)], dtype=np.int32)
    et, score, before = _tet_pass(q, tets, energy=[0.0])
    assert all(v == 0.0 for v in before.values())
    tris = np.array([(0, 1, 2)], dtype=np.int32)
    cfg = ro.RefineConfig(scoring="geometric", min_edge_length=H_MIN, contact_d1=D1)
    inv = np.ones(4, np.float32)

    edges = np.nonzero(et.is_edge & (et.slot_row < et.col_idx))[0]

    def tri_pass(bary, d):
        s = ro.tri_scores(score, et, q, tris, inv, np.array([d], np.float32), np.array([bary], np.float32), cfg)
        return {(int(et.slot_row[k]), int(et.col_idx[k])): float(s[k]) for k in edges}

    sc = tri_pass((0.0, 0.5, 0.5), 0.5 * D1)
    assert sc[(1, 2)] > sc[(0, 1)] and sc[(1, 2)] > sc[(0, 2)]
    assert sc[(0, 1)] == pytest.approx(sc[(0, 2)], rel=1e-5)
    assert sc[(1, 2)] == pytest.approx((1.0 / H_MIN) * 1.0 * 0.5 * 1.0, rel=1e-4)
    assert sc[(0, 3)] == 0.0
    sc = tri_pass((1 / 3, 1 / 3, 1 / 3), 0.5 * D1)
    assert sc[(0, 1)] == pytest.approx(sc[(1, 2)], rel=1e-5)
    assert sc[(0, 1)] == pytest.approx(sc[(0, 2)], rel=1e-5)
    sc = tri_pass((0.0, 0.5, 0.5), 2.0 * D1)
    assert all(v == 0.0 for v in sc.values())
    sc_a = tri_pass((0.0, 0.5, 0.5), 0.5 * D1)
    sc_b = tri_pass((0.0, 0.5, 0.5), 0.0)
    assert sc_b[(1, 2)] == pytest.approx(2.0 * sc_a[(1, 2)], rel=1e-5)


def test_elastic_term_is_excess_over_mean_density():
    t = T2[0]
    Dm = np.stack([Q2[t[1]] - Q2[t[0]], Q2[t[2]] - Q2[t[0]], Q2[t[3]] - Q2[t[0]]], axis=1).astype(np.float64)
    vol = abs(np.linalg.det(Dm)) / 6.0
    rho = 1.0 / vol
    _, _, sc = _tet_pass(Q2, T2, energy=[1.0, 1.0], elastic_stats=(2.0 * rho, 2.0))
    assert all(v == 0.0 for v in sc.values())
    _, _, sc = _tet_pass(Q2, T2, energy=[1.0, 1.0], elastic_stats=(rho, 2.0))
    L = np.linalg.norm(Q2[0] - Q2[1])
    assert sc[(0, 1)] == pytest.approx(L / H_MIN, rel=1e-4)


def test_legacy_score_sums_over_tets_in_order():
    """populate_candidates (refinement.py:74-121): the shared edges of the two
    tets score (E_0 + E_1) L, the others E_t L; a midpoint inside a shape
    scores the penetration score."""
    et = ro.EdgeTable(T2, 5)
    cfg = ro.RefineConfig(scoring="legacy", tet_score_weight=1.0, vertex_score_weight=0.0)
    E = np.array([0.25, 2.0], np.float32)
    score, elig = ro.legacy_scores(et, Q2, np.ones(5, np.float32), E, np.zeros(5, np.float32), cfg)
    sc = {(int(et.slot_row[s]), int(et.col_idx[s])): float(score[s]) for s in np.nonzero(elig)[0]}
    L = lambda a, b: float(np.linalg.norm(Q2[a] - Q2[b]))
    assert sc[(0, 1)] == pytest.approx(2.25 * L(0, 1), rel=1e-6)
    assert sc[(0, 3)] == pytest.approx(0.25 * L(0, 3), rel=1e-6)
    assert sc[(1, 4)] == pytest.approx(2.0 * L(1, 4), rel=1e-6)
    pen, _ = ro.legacy_scores(et, Q2, np.ones(5, np.float32), E, np.zeros(5, np.float32), cfg,
                              midpoint_distance=lambda mid: np.where(mid[:, 2] > 0.2, -1.0, 1.0))
    top = {(int(et.slot_row[s]), int(et.col_idx[s])): float(pen[s]) for s in np.nonzero(elig)[0]}
    assert top[(0, 3)] == pytest.approx(1.0e6) and top[(0, 1)] == sc[(0, 1)]


def _passes(scoring, n_passes=6, refine_every=1, seed=0):
    mesh = grid_mesh()
    q = deformed(mesh.rest_q, seed=seed)
    cap_v, cap_t = 8 * mesh.rest_q.shape[0], 8 * mesh.tets.shape[0]
    cfg = (ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0, refine_every=refine_every)
           if scoring == "legacy" else
           ro.RefineConfig(scoring="geometric", threshold=1e-6, min_edge_length=0.05, refine_every=refine_every))
    out = []
    rng = np.random.default_rng(seed)
    for k in range(n_passes):
        E = rng.uniform(0.0, 1.0, mesh.tets.shape[0]).astype(np.float32)
        res = ro.refine_pass(mesh, q, np.zeros_like(q), cfg, tet_scores=E, max_particles=cap_v, max_tets=cap_t,
                             pass_counter=k)
        out.append((mesh, res))
        mesh, q = res.mesh, res.q
    return out


@pytest.mark.parametrize("scoring", ["legacy", "geometric"])
def test_refinement_conserves_volume_and_grows_mesh(scoring):
    """tests/test_refinement.py:81-122 on the oracle: no orphaned vertex, no
    inverted tet, rest volume conserved, and the mesh grows."""
    runs = _passes(scoring)
    v0 = ro.rest_volume_total(runs[0][0].rest_q, runs[0][0].tets)[0]
    for before, res in runs:
        m = res.mesh
        assert m.tets.max() < m.rest_q.shape[0] and m.tets.min() >= 0
        used = np.zeros(m.rest_q.shape[0], bool)
        used[m.tets.ravel()] = True
        assert used.all(), "orphaned vertex"
        vol, vmin = ro.rest_volume_total(m.rest_q, m.tets)
        assert vmin > -1e-9
        assert vol == pytest.approx(v0, abs=1e-6)
    assert runs[-1][1].mesh.tets.shape[0] > runs[0][0].tets.shape[0]


@pytest.mark.parametrize("scoring", ["legacy", "geometric"])
def test_selection_is_conflict_free_and_conforming(scoring):
    for before, res in _passes(scoring):
        et = ro.EdgeTable(before.tets, before.rest_q.shape[0])
        sel = res.state[et.tet_edge] == ro.SELECTED
        assert sel.sum(axis=1).max() <= 1, "a tet holds two split edges"
        if res.split_edges:
            s = np.nonzero(res.state == ro.SELECTED)[0]
            pairs = list(zip(et.slot_row[s].tolist(), et.col_idx[s].tolist()))
            assert hanging_edges(res.mesh.tets, pairs) == 0
            # every tet around a split edge split: T grows by the tets on split edges
            assert res.mesh.tets.shape[0] == before.tets.shape[0] + int(sel.any(axis=1).sum())
            # new vertices sit at the edge midpoints, in ascending edge order
            n0 = before.rest_q.shape[0]
            mid = (before.rest_q[et.slot_row[s]] + (before.rest_q[et.col_idx[s]] - before.rest_q[et.slot_row[s]])
                   * np.float32(0.5)).astype(np.float32)
            np.testing.assert_array_equal(res.mesh.rest_q[n0:], mid)
        assert ro.is_conforming(res.mesh.tets)


def test_masses_and_kinematic_vertices():
    """A splitting pass rebuilds the lumped masses from density * volume / 4:
    their sum is density times the rest volume; vertex 0 stays kinematic; new
    vertices are free."""
    for before, res in _passes("legacy", n_passes=3):
        m = res.mesh
        if res.split_edges == 0:
            continue
        vol = ro.rest_volume_total(m.rest_q, m.tets)[0]
        assert float(m.mass.astype(np.float64).sum()) == pytest.approx(1.0 * vol, rel=1e-5)
        assert m.inv_mass[0] == 0.0
        n0 = before.rest_q.shape[0]
        assert np.all(m.inv_mass[n0:] > 0.0)
        np.testing.assert_allclose(m.inv_mass[1:] * m.mass[1:], 1.0, rtol=1e-6)


def test_selection_does_not_depend_on_tet_order():
    mesh = grid_mesh(dims=(4, 3, 2))
    q = deformed(mesh.rest_q)
    T = mesh.tets.shape[0]
    E = np.random.default_rng(3).uniform(0.0, 1.0, T).astype(np.float32)
    cfg = ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0)
    perm = np.random.default_rng(4).permutation(T)
    shuffled = ro.Mesh(mesh.rest_q, mesh.tets[perm], mesh.poses[perm], mesh.materials[perm], mesh.stretch[perm],
                       mesh.lam[perm], mesh.mass, mesh.inv_mass, mesh.tris)
    a = ro.refine_pass(mesh, q, q, cfg, tet_scores=E, max_particles=10 ** 6, max_tets=10 ** 6)
    b = ro.refine_pass(shuffled, q, q, cfg, tet_scores=E[perm], max_particles=10 ** 6, max_tets=10 ** 6)
    assert a.split_edges == b.split_edges > 0
    np.testing.assert_array_equal(a.state, b.state)
    np.testing.assert_array_equal(a.q, b.q)
    sort = lambda t: np.array(sorted(map(tuple, np.sort(t, axis=1))))
    np.testing.assert_array_equal(sort(a.mesh.tets), sort(b.mesh.tets))


def test_refine_every_gates_passes():
    """tests/test_refinement.py:187-210: with refine_every 3 the mesh grows
    only on passes 0, 3, 6, ..."""
    grew = [k for k, (before, res) in enumerate(_passes("legacy", n_passes=9, refine_every=3))
            if res.mesh.tets.shape[0] > before.tets.shape[0]]
    assert grew and all(k % 3 == 0 for k in grew)


def test_capacity_overflow_drops_the_pass():
    mesh = grid_mesh()
    q = deformed(mesh.rest_q)
    E = np.ones(mesh.tets.shape[0], np.float32)
    cfg = ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0)
    full = ro.refine_pass(mesh, q, q, cfg, tet_scores=E, max_particles=10 ** 6, max_tets=10 ** 6)
    assert full.split_edges > 0
    tight = ro.refine_pass(mesh, q, q, cfg, tet_scores=E, max_particles=10 ** 6,
                           max_tets=full.mesh.tets.shape[0] - 1)
    assert tight.overflow and tight.split_edges == 0
    np.testing.assert_array_equal(tight.mesh.tets, mesh.tets)


def test_surface_tris_split_with_their_edges():
    mesh = grid_mesh()
    from oracle.contact_oracle import boundary_tris
    mesh.tris = np.asarray(boundary_tris(mesh.tets, mesh.rest_q), dtype=np.int32)
    q = deformed(mesh.rest_q)
    E = np.random.default_rng(5).uniform(0.0, 1.0, mesh.tets.shape[0]).astype(np.float32)
    cfg = ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0)
    res = ro.refine_pass(mesh, q, q, cfg, tet_scores=E, max_particles=10 ** 6, max_tets=10 ** 6, max_tris=10 ** 6)
    assert res.split_edges > 0
    # the refined surface is the boundary of the refined tets
    ref = np.asarray(boundary_tris(res.mesh.tets, res.mesh.rest_q), dtype=np.int32)
    canon = lambda t: sorted(map(tuple, np.sort(t, axis=1)))
    assert canon(res.mesh.tris) == canon(ref)
