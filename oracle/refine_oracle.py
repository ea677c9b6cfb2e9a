"""CPU oracle for adaptive refinement -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product: only ``tests/`` may import it.

It restates, in float32 numpy with the library's order of operations, one
pass of the reference's edge-bisection refinement ``refine()``
(src/mfem/refinement/refinement.py:914-1322):

============================================  ==========================================
stage                                         reference
============================================  ==========================================
legacy edge score (sum over incident tets of  refinement.py:74-121 (populate_candidates)
(E_t w_t + min vertex score w_v) L, midpoint
penetration override)
geometric edge score (per-edge max of         refinement.py:157-256
(L/h)(L/L_max)(w_e s_el + w_c s_c))
elastic density mean                          refinement.py:163-192
surface-tri contact term                      refinement.py:259-316
selection: each tet's best edge above the     refinement.py:319-557 (get_tet_candidate,
threshold, conflicts resolved over sweeps     remove_conflicting_candidates,
                                              finalize_nonconflicting_candidates,
                                              udpate_tet_candidate, invalidate_failed_candidates)
refine_every gate, pass counter               refinement.py:560-575
capacity guard (drop the whole pass)          refinement.py:578-604
new vertices at split_position on the edge    refinement.py:697-730
tets split into two children, DmInv, s,       refinement.py:733-824 (scatter_tets)
lambda, materials copied, lumped masses
surface tris split the same way               refinement.py:827-911
============================================  ==========================================

Where the reference leaves the outcome to thread scheduling, this restatement
(and the CUDA path it checks) fixes one deterministic rule:

* Selection.  An edge is a candidate when it is not between two kinematic
  vertices and scores above the threshold.  Edges are ranked by score, ties
  by the smaller (min vertex, max vertex) key.  Each sweep, every tet picks
  its best still-available candidate (a tet that holds a selected edge keeps
  it); an available candidate that every tet containing it picked becomes
  selected, and the other edges of those tets become unavailable.  So no tet
  holds two selected edges and every tet around a selected edge splits (the
  reference's pending / finalize flags reach the same invariant through
  races, and can drop an edge some tets already split on).
* Numbering.  New vertices are numbered in ascending edge key order after
  the old ones; the reference numbers them by the tet that wins a hash
  insert.  A new vertex sits at q_lo + (q_hi - q_lo) t with lo < hi.
* Masses.  On a pass that splits, every vertex's lumped mass is rebuilt as
  the sum of density * volume / 4 over its tets in ascending (old tet,
  child) order, and a vertex that was not kinematic gets inv_mass = 1/mass;
  kinematic vertices stay kinematic.  A pass that splits nothing leaves the
  mesh untouched.  (The reference zeroes and re-accumulates
  model.particle_mass with float atomics on every call, splitting or not,
  and never updates particle_inv_mass.)
* Scores.  Legacy scores add their per-tet terms in ascending tet order
  (the reference adds with float atomics).

No reference test pins a whole refine pass: the reference's own tests check
scoring known answers (tests/test_refine_scoring.py, restated in
tests/test_oracle_refine.py) and properties of whole runs (rest volume
conserved, no orphaned vertex, growth only on refining steps:
tests/test_refinement.py), which the tests apply to this restatement and to
the CUDA path.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import mfem_oracle as mo

f32 = np.float32

# local vertex pairs (i, j), j < i, in the reference's loop order
# (`for i in range(4): for j in range(i)`, refinement.py:113-114)
TET_PAIRS = ((1, 0), (2, 0), (2, 1), (3, 0), (3, 1), (3, 2))
TRI_PAIRS = ((1, 0), (2, 0), (2, 1))

AVAILABLE, SELECTED, UNAVAILABLE = 1, 2, 3

SHAPE_PLANE, SHAPE_CAPSULE = 0, 1


@dataclass
class RefineConfig:
    scoring: str = "legacy"              # "legacy" or "geometric"
    threshold: float = 10.1              # min_refine_score (legacy) / refine_geometric_threshold
    tet_score_weight: float = 0.0        # refinement.py:64-66 defaults
    vertex_score_weight: float = 0.1
    penetrating_edge_score: float = 1.0e6
    min_edge_length: float = 0.1
    contact_d1: float = 0.1
    elastic_weight: float = 1.0
    vertex_contact_weight: float = 1.0
    tri_contact_weight: float = 1.0
    split_position: float = 0.5
    density: float = 1.0
    conflict_iterations: int = 5
    refine_every: int = 1


@dataclass
class Mesh:
    """One body's refinable state (host arrays)."""
    rest_q: np.ndarray        # [n, 3] f32
    tets: np.ndarray          # [T, 4] i32
    poses: np.ndarray         # [T, 3, 3] f32 DmInv
    materials: np.ndarray     # [T, 3] f32
    stretch: np.ndarray       # [T, 6] f32
    lam: np.ndarray           # [T, 6] f32
    mass: np.ndarray          # [n] f32
    inv_mass: np.ndarray      # [n] f32
    tris: np.ndarray          # [m, 3] i32


@dataclass
class RefineResult:
    mesh: Mesh
    q: np.ndarray
    qd: np.ndarray
    score: np.ndarray          # [nnzb] edge scores (upper slots)
    state: np.ndarray          # [nnzb] edge states after the selection
    split_edges: int
    overflow: bool
    refining: bool


# ---------------------------------------------------------------------------
# edge table: the upper off-diagonal slots of the exact vertex adjacency
# ---------------------------------------------------------------------------


class EdgeTable:
    def __init__(self, tets, n):
        tets = np.asarray(tets, dtype=np.int64)
        self.row_ptr, self.col_idx = mo.bsr_sparsity(tets, n)
        self.nnzb = int(self.col_idx.shape[0])
        self.slot_row = np.repeat(np.arange(n, dtype=np.int64), np.diff(self.row_ptr))
        slots = mo.tet_slot_map(tets, self.row_ptr, self.col_idx).astype(np.int64)
        T = tets.shape[0]
        # [T, 6] slot of each tet edge (lower vertex's row) in TET_PAIRS order
        self.tet_edge = np.empty((T, 6), dtype=np.int64)
        for p, (i, j) in enumerate(TET_PAIRS):
            lo_i = tets[:, i] < tets[:, j]
            self.tet_edge[:, p] = np.where(lo_i, slots[:, i * 4 + j], slots[:, j * 4 + i])
        self.is_edge = np.zeros(self.nnzb, dtype=bool)
        self.is_edge[self.tet_edge.ravel()] = True
        # tets of each edge, ascending: (slot, tet) pairs sorted by slot, stably
        flat_slot = self.tet_edge.ravel()
        flat_tet = np.repeat(np.arange(T, dtype=np.int64), 6)
        order = np.argsort(flat_slot, kind="stable")
        self.et_slot = flat_slot[order]
        self.et_tet = flat_tet[order]
        self.et_pair = np.tile(np.arange(6), T)[order]
        self.edge_start = np.searchsorted(self.et_slot, np.arange(self.nnzb + 1))
        # tets of each vertex, ascending (tet, corner)
        flat_v = tets.ravel()
        vorder = np.argsort(flat_v, kind="stable")
        self.vt_vertex = flat_v[vorder]
        self.vt_tet = vorder // 4
        self.vt_corner = vorder % 4
        self.vert_start = np.searchsorted(self.vt_vertex, np.arange(n + 1))


def _seg_sum_f32(start, values, n_seg):
    """Sequential float32 sum of each segment [start[s], start[s+1])."""
    out = np.zeros(n_seg, dtype=f32)
    lens = np.diff(start)
    if lens.size == 0:
        return out
    for k in range(int(lens.max()) if lens.size else 0):
        m = lens > k
        out[m] = (out[m] + values[start[:-1][m] + k]).astype(f32)
    return out


def _length(a, b):
    d = (b - a).astype(f32)
    return np.sqrt(((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]).astype(f32) + d[..., 2] * d[..., 2]).astype(f32))


def det3_f32(M):
    """Cofactor expansion along the first row, float32, in the library's order."""
    M = M.astype(f32)
    c0 = (M[..., 1, 1] * M[..., 2, 2] - M[..., 1, 2] * M[..., 2, 1]).astype(f32)
    c1 = (M[..., 1, 2] * M[..., 2, 0] - M[..., 1, 0] * M[..., 2, 2]).astype(f32)
    c2 = (M[..., 1, 0] * M[..., 2, 1] - M[..., 1, 1] * M[..., 2, 0]).astype(f32)
    return ((M[..., 0, 0] * c0 + M[..., 0, 1] * c1).astype(f32) + M[..., 0, 2] * c2).astype(f32)


def inverse3_f32(M):
    """Adjugate over determinant, float32, in the library's order."""
    M = M.astype(f32)
    a, b, c = M[..., 0, 0], M[..., 0, 1], M[..., 0, 2]
    d, e, f = M[..., 1, 0], M[..., 1, 1], M[..., 1, 2]
    g, h, i = M[..., 2, 0], M[..., 2, 1], M[..., 2, 2]
    A = (e * i - f * h).astype(f32)
    B = (f * g - d * i).astype(f32)
    C = (d * h - e * g).astype(f32)
    det = ((a * A + b * B).astype(f32) + c * C).astype(f32)
    inv_det = (f32(1.0) / det).astype(f32)
    out = np.empty(M.shape, dtype=f32)
    out[..., 0, 0] = A * inv_det
    out[..., 0, 1] = (c * h - b * i).astype(f32) * inv_det
    out[..., 0, 2] = (b * f - c * e).astype(f32) * inv_det
    out[..., 1, 0] = B * inv_det
    out[..., 1, 1] = (a * i - c * g).astype(f32) * inv_det
    out[..., 1, 2] = (c * d - a * f).astype(f32) * inv_det
    out[..., 2, 0] = C * inv_det
    out[..., 2, 1] = (b * g - a * h).astype(f32) * inv_det
    out[..., 2, 2] = (a * e - b * d).astype(f32) * inv_det
    return out


def edge_matrix(x, tet_rows):
    """Dm = [x1 - x0, x2 - x0, x3 - x0] (columns), float32."""
    xe = x[tet_rows].astype(f32)
    return np.stack([(xe[:, 1] - xe[:, 0]).astype(f32), (xe[:, 2] - xe[:, 0]).astype(f32),
                     (xe[:, 3] - xe[:, 0]).astype(f32)], axis=2)


# ---------------------------------------------------------------------------
# scores
# ---------------------------------------------------------------------------


def tet_energy(energy, stretch, materials, poses):
    """Per-tet elastic energy in s, rounded to float32 (the tet_scores the
    reference's solver passes, solver.py:958, 475)."""
    return mo.elastic_energy_only(energy, stretch.astype(np.float64), materials.astype(np.float64),
                                  poses.astype(np.float64)).astype(f32)


def eligible_edges(et: EdgeTable, inv_mass):
    a = et.slot_row
    b = et.col_idx.astype(np.int64)
    return et.is_edge & (a < b) & ~((inv_mass[a] == 0.0) & (inv_mass[b] == 0.0))


def legacy_scores(et: EdgeTable, q, inv_mass, tet_scores, vertex_scores, cfg: RefineConfig, midpoint_distance=None):
    """Per-edge sum over the incident tets, ascending, of
    (E_t w_t + min(vs_a, vs_b) w_v) L; an edge whose midpoint is inside a
    shape scores the penetration score (refinement.py:74-121)."""
    elig = eligible_edges(et, inv_mass)
    a = et.slot_row
    b = et.col_idx.astype(np.int64)
    L = _length(q[a], q[b])
    vmin = np.minimum(vertex_scores[a], vertex_scores[b]).astype(f32)
    vterm = (vmin * f32(cfg.vertex_score_weight)).astype(f32)
    tterm = (tet_scores[et.et_tet].astype(f32) * f32(cfg.tet_score_weight)).astype(f32)
    terms = ((tterm + vterm[et.et_slot]).astype(f32) * L[et.et_slot]).astype(f32)
    score = _seg_sum_f32(et.edge_start, terms, et.nnzb)
    if midpoint_distance is not None:
        mid = (f32(0.5) * (q[a] + q[b]).astype(f32)).astype(f32)
        pen = midpoint_distance(mid) < 0.0
        score = np.where(pen, np.maximum(f32(0.0), f32(cfg.penetrating_edge_score)), score).astype(f32)
    return np.where(elig, score, f32(0.0)).astype(f32), elig


def tet_density(tet_scores, materials, poses):
    """Strain-energy density over mu (refinement.py:163-176)."""
    vol = np.abs((f32(1.0) / (f32(6.0) * det3_f32(poses)).astype(f32)).astype(f32))
    mu = materials[:, 0].astype(f32)
    ok = (mu > 0.0) & (vol > 0.0)
    dens = (np.maximum(tet_scores.astype(f32), f32(0.0)) / (vol * mu).astype(f32)).astype(f32)
    return np.where(ok, dens, f32(0.0)).astype(f32)


def geometric_scores(et: EdgeTable, q, tets, inv_mass, tet_scores, materials, poses, distance, shape_id,
                     shape_type, cfg: RefineConfig, elastic_stats=None):
    """Per-edge max over the incident tets of (L/h)(L/L_max)(w_e s_el + w_c s_c),
    edges shorter than 2h excluded (refinement.py:195-256).  elastic_stats
    = (sum of densities, count) as the reference kernel takes them; None:
    the mesh's own (elastic_density_stats, refinement.py:179-192)."""
    elig = eligible_edges(et, inv_mass)
    dens = tet_density(tet_scores, materials, poses)
    if elastic_stats is None:
        total = float(np.sum(dens.astype(np.float64)))
        count = float(tets.shape[0])
    else:
        total, count = float(elastic_stats[0]), float(elastic_stats[1])
    if count > 0.0 and total > 0.0:
        mean = f32(total / count)
        s_el = np.maximum((dens / mean).astype(f32) - f32(1.0), f32(0.0)).astype(f32)
    else:
        s_el = dens
    tv = tets.astype(np.int64)
    lmax = np.zeros(tets.shape[0], dtype=f32)
    for i, j in TET_PAIRS:
        lmax = np.maximum(lmax, _length(q[tv[:, i]], q[tv[:, j]]))
    lmax = np.maximum(lmax, f32(1.0e-20))
    a = et.slot_row
    b = et.col_idx.astype(np.int64)
    L = _length(q[a], q[b])
    h = f32(cfg.min_edge_length)
    d1 = f32(cfg.contact_d1)

    def prox(v):
        sid = shape_id[v]
        ok = sid >= 0
        cap = np.zeros(v.shape, dtype=bool)
        cap[ok] = shape_type[sid[ok]] == SHAPE_CAPSULE
        p = np.maximum(((d1 - distance[v].astype(f32)).astype(f32) / d1).astype(f32), f32(0.0))
        return np.where(cap, p, f32(0.0)).astype(f32)

    s_c = np.maximum(prox(a), prox(b)).astype(f32)
    t = et.et_tet
    s = et.et_slot
    val = ((L[s] / h).astype(f32) * (L[s] / lmax[t]).astype(f32)).astype(f32)
    val = (val * ((f32(cfg.elastic_weight) * s_el[t]).astype(f32)
                  + (f32(cfg.vertex_contact_weight) * s_c[s]).astype(f32)).astype(f32)).astype(f32)
    val = np.where(L[s] >= f32(2.0) * h, np.maximum(val, f32(0.0)), f32(0.0)).astype(f32)
    score = np.zeros(et.nnzb, dtype=f32)
    np.maximum.at(score, s, val)
    return np.where(elig, score, f32(0.0)).astype(f32), elig


def tri_edge_slot(et: EdgeTable, u, v):
    lo = np.minimum(u, v).astype(np.int64)
    hi = np.maximum(u, v).astype(np.int64)
    key_all = et.slot_row * (et.row_ptr.shape[0] - 1) + et.col_idx.astype(np.int64)
    pos = np.searchsorted(key_all, lo * (et.row_ptr.shape[0] - 1) + hi)
    assert np.all(et.col_idx[pos] == hi)
    return pos


def tri_scores(score, et: EdgeTable, q, tris, inv_mass, tri_distance, tri_bary, cfg: RefineConfig):
    """Raises the scores of the edges of surface tris inside the barrier
    range, the edge nearest the closest point most (refinement.py:259-316)."""
    score = score.copy()
    d1 = f32(cfg.contact_d1)
    h = f32(cfg.min_edge_length)
    tr = tris.astype(np.int64)
    live = tri_distance.astype(f32) < d1
    prox = np.maximum(((d1 - tri_distance.astype(f32)).astype(f32) / d1).astype(f32), f32(0.0))
    lmax = np.full(tris.shape[0], f32(1.0e-20), dtype=f32)
    for k in range(3):
        i = (k + 1) % 3
        lmax = np.maximum(lmax, _length(q[tr[:, i]], q[tr[:, k]]))
    for k in range(3):
        i, j = (k + 1) % 3, (k + 2) % 3
        u, v = tr[:, i], tr[:, j]
        L = _length(q[u], q[v])
        ok = live & ~((inv_mass[u] == 0.0) & (inv_mass[v] == 0.0)) & (L >= f32(2.0) * h)
        w = (f32(1.0) - tri_bary[:, k].astype(f32)).astype(f32)
        val = ((L / h).astype(f32) * (L / lmax).astype(f32)).astype(f32)
        val = (((val * f32(cfg.tri_contact_weight)).astype(f32) * prox).astype(f32) * w).astype(f32)
        slot = tri_edge_slot(et, u, v)
        np.maximum.at(score, slot[ok], np.maximum(val[ok], f32(0.0)))
    return score


# ---------------------------------------------------------------------------
# selection
# ---------------------------------------------------------------------------


def select_edges(et: EdgeTable, score, elig, threshold, sweeps):
    """Deterministic conflict-free selection (see the module docstring)."""
    cand_ok = elig & (score > f32(threshold))
    state = np.where(cand_ok, AVAILABLE, 0).astype(np.int8)
    T = et.tet_edge.shape[0]
    cand = np.full(T, -1, dtype=np.int64)
    te = et.tet_edge
    for _ in range(sweeps):
        st = state[te]
        sc = score[te]
        held = st == SELECTED
        has_held = held.any(axis=1)
        avail = st == AVAILABLE
        # best available: highest score, then smallest slot
        key_sc = np.where(avail, sc, -np.inf)
        best_sc = key_sc.max(axis=1)
        tie = avail & (key_sc == best_sc[:, None])
        slot_or_big = np.where(tie, te, np.iinfo(np.int64).max)
        best = slot_or_big.min(axis=1)
        best = np.where(avail.any(axis=1), best, -1)
        held_slot = np.where(held, te, -1).max(axis=1)
        cand = np.where(has_held, held_slot, best)
        # an available candidate some tet did not pick is blocked
        blocked = np.zeros(et.nnzb, dtype=bool)
        other = avail & (te != cand[:, None])
        blocked[te[other]] = True
        newly = (state == AVAILABLE) & ~blocked
        state[newly] = SELECTED
        # tets whose pick was selected lose their other edges
        picked = cand >= 0
        picked[picked] = state[cand[picked]] == SELECTED
        rows = np.nonzero(picked)[0]
        if rows.size:
            others = te[rows][te[rows] != cand[rows][:, None]]
            state[others] = np.where(state[others] == SELECTED, SELECTED, UNAVAILABLE)
    split = np.zeros(T, dtype=bool)
    split_slot = np.full(T, -1, dtype=np.int64)
    st = state[te]
    held = st == SELECTED
    split = held.any(axis=1)
    split_slot[split] = np.where(held, te, -1).max(axis=1)[split]
    return state, split, split_slot


# ---------------------------------------------------------------------------
# the pass
# ---------------------------------------------------------------------------


def refine_pass(mesh: Mesh, q, qd, cfg: RefineConfig, energy="arap", tet_scores=None, vertex_scores=None,
                midpoint_distance=None, distance=None, shape_id=None, shape_type=None, tri_distance=None,
                tri_bary=None, max_particles=None, max_tets=None, max_tris=None, pass_counter=None):
    """One refine() call on `mesh` at positions q (velocities qd)."""
    n = mesh.rest_q.shape[0]
    T = mesh.tets.shape[0]
    m = mesh.tris.shape[0]
    q = np.asarray(q, dtype=f32)
    qd = np.asarray(qd, dtype=f32)
    et = EdgeTable(mesh.tets, n)
    if tet_scores is None:
        tet_scores = tet_energy(energy, mesh.stretch, mesh.materials, mesh.poses)
    tet_scores = np.asarray(tet_scores, dtype=f32)
    if cfg.scoring == "legacy":
        vs = np.zeros(n, dtype=f32) if vertex_scores is None else np.asarray(vertex_scores, dtype=f32)
        score, elig = legacy_scores(et, q, mesh.inv_mass, tet_scores, vs, cfg, midpoint_distance)
    else:
        dist = np.full(n, 1.0e8, dtype=f32) if distance is None else np.asarray(distance, dtype=f32)
        sid = np.full(n, -1, dtype=np.int64) if shape_id is None else np.asarray(shape_id, dtype=np.int64)
        stype = np.zeros(0, dtype=np.int64) if shape_type is None else np.asarray(shape_type, dtype=np.int64)
        score, elig = geometric_scores(et, q, mesh.tets, mesh.inv_mass, tet_scores, mesh.materials, mesh.poses,
                                       dist, sid, stype, cfg)
        if tri_distance is not None and m > 0:
            score = tri_scores(score, et, q, mesh.tris, mesh.inv_mass, np.asarray(tri_distance, dtype=f32),
                               np.asarray(tri_bary, dtype=f32), cfg)
    refining = True
    if pass_counter is not None and cfg.refine_every > 1:
        refining = pass_counter % cfg.refine_every == 0
    if refining:
        state, split, split_slot = select_edges(et, score, elig, cfg.threshold, cfg.conflict_iterations)
    else:
        state = np.zeros(et.nnzb, dtype=np.int8)
        split = np.zeros(T, dtype=bool)
        split_slot = np.full(T, -1, dtype=np.int64)
    selected = state == SELECTED
    n_new_v = int(selected.sum())
    T_new = T + int(split.sum())
    tri_split_slot = np.full(m, -1, dtype=np.int64)
    if m > 0:
        tr = mesh.tris.astype(np.int64)
        for i, j in TRI_PAIRS:
            s = tri_edge_slot(et, tr[:, i], tr[:, j])
            hit = selected[s]
            tri_split_slot = np.where(hit, s, tri_split_slot)
    m_new = m + int((tri_split_slot >= 0).sum())
    cap_v = n if max_particles is None else max_particles
    cap_t = T if max_tets is None else max_tets
    cap_m = m if max_tris is None else max_tris
    overflow = bool(n_new_v > 0 and (T_new > cap_t or n + n_new_v > cap_v or m_new > cap_m))
    if overflow or n_new_v == 0:
        return RefineResult(mesh, q.copy(), qd.copy(), score, state, 0, overflow, refining)

    # new vertices, ascending edge key
    new_index = np.full(et.nnzb, -1, dtype=np.int64)
    new_index[selected] = n + np.arange(n_new_v)
    sel = np.nonzero(selected)[0]
    a = et.slot_row[sel]
    b = et.col_idx[sel].astype(np.int64)
    t = f32(cfg.split_position)

    def interp(arr):
        return (arr[a] + ((arr[b] - arr[a]).astype(f32) * t).astype(f32)).astype(f32)

    q_out = np.concatenate([q, interp(q)])
    qd_out = np.concatenate([qd, interp(qd)])
    rest_out = np.concatenate([mesh.rest_q.astype(f32), interp(mesh.rest_q.astype(f32))])

    # tets: children at the exclusive scan of 1 + split
    tet_map = np.concatenate([[0], np.cumsum(1 + split.astype(np.int64))])
    tets_out = np.zeros((T_new, 4), dtype=np.int32)
    poses_out = np.zeros((T_new, 3, 3), dtype=f32)
    mat_out = np.zeros((T_new, 3), dtype=f32)
    s_out = np.zeros((T_new, 6), dtype=f32)
    l_out = np.zeros((T_new, 6), dtype=f32)
    tmass = np.zeros(T_new, dtype=f32)
    dens = f32(cfg.density)
    keep = ~split
    dst = tet_map[:-1][keep]
    tets_out[dst] = mesh.tets[keep]
    poses_out[dst] = mesh.poses[keep]
    tmass[dst] = (dens / (f32(6.0) * det3_f32(mesh.poses[keep])).astype(f32)).astype(f32)
    rows = np.nonzero(split)[0]
    tv = mesh.tets[rows].astype(np.int64)
    ss = split_slot[rows]
    lo = et.slot_row[ss]
    hi = et.col_idx[ss].astype(np.int64)
    # the pair (i, j), j < i, of the split edge in the tet (refinement.py:787-793)
    pi = np.zeros(rows.size, dtype=np.int64)
    pj = np.zeros(rows.size, dtype=np.int64)
    for i, j in TET_PAIRS:
        hit = ((tv[:, i] == lo) & (tv[:, j] == hi)) | ((tv[:, i] == hi) & (tv[:, j] == lo))
        pi = np.where(hit, i, pi)
        pj = np.where(hit, j, pj)
    nv = new_index[ss]
    for c in range(2):
        child = tv.copy()
        repl = pi if c == 0 else pj
        child[np.arange(rows.size), repl] = nv
        dstc = tet_map[rows] + c
        tets_out[dstc] = child.astype(np.int32)
        Dm = edge_matrix(rest_out, child)
        det = det3_f32(Dm)
        vol = (det / f32(6.0)).astype(f32)
        tmass[dstc] = (vol * dens).astype(f32)
        poses_out[dstc] = inverse3_f32(Dm)
    src = np.repeat(np.arange(T), 1 + split.astype(np.int64))
    mat_out[:] = mesh.materials[src]
    s_out[:] = mesh.stretch[src]
    l_out[:] = mesh.lam[src]

    # masses in ascending (old tet, child) order
    n_tot = n + n_new_v
    mass = np.zeros(n_tot, dtype=f32)
    quarter = f32(4.0)
    # old vertices: per incident old tet, the unsplit tet or the children that keep the vertex
    vt_t = et.vt_tet
    vt_c = et.vt_corner
    contrib = np.zeros((vt_t.size, 2), dtype=f32)
    has = np.zeros((vt_t.size, 2), dtype=bool)
    sp = split[vt_t]
    base = tet_map[vt_t]
    contrib[~sp, 0] = (tmass[base[~sp]] / quarter).astype(f32)
    has[~sp, 0] = True
    if sp.any():
        idx = np.nonzero(sp)[0]
        # position of the split tet's row in `rows`
        row_of = np.full(T, -1, dtype=np.int64)
        row_of[rows] = np.arange(rows.size)
        r = row_of[vt_t[idx]]
        for c in range(2):
            repl = (pi if c == 0 else pj)[r]
            keeps = repl != vt_c[idx]
            contrib[idx[keeps], c] = (tmass[base[idx[keeps]] + c] / quarter).astype(f32)
            has[idx[keeps], c] = True
    flat_vals = contrib.reshape(-1)
    flat_has = has.reshape(-1)
    # per vertex: segments of the vertex's entries, (tet, child) ascending
    starts = et.vert_start
    seg_vals = np.zeros((vt_t.size, 2), dtype=f32)
    seg_vals[:] = np.where(has, contrib, f32(0.0))
    vals = seg_vals.reshape(-1)
    mass[:n] = _seg_sum_f32(2 * starts, vals, n)
    del flat_vals, flat_has
    # new vertices: both children of every old tet on the edge
    e_lo = et.edge_start[sel]
    e_hi = et.edge_start[sel + 1]
    ev = np.zeros(0, dtype=f32)
    estart = [0]
    parts = []
    for k in range(sel.size):
        ts = et.et_tet[e_lo[k]:e_hi[k]]
        parts.append(np.stack([(tmass[tet_map[ts]] / quarter).astype(f32),
                               (tmass[tet_map[ts] + 1] / quarter).astype(f32)], axis=1).reshape(-1))
        estart.append(estart[-1] + parts[-1].size)
    if parts:
        ev = np.concatenate(parts)
    mass[n:] = _seg_sum_f32(np.asarray(estart, dtype=np.int64), ev, sel.size)
    inv_out = np.zeros(n_tot, dtype=f32)
    free = np.ones(n_tot, dtype=bool)
    free[:n] = mesh.inv_mass != 0.0
    ok = free & (mass > 0.0)
    inv_out[ok] = (f32(1.0) / mass[ok]).astype(f32)

    # tris
    tris_out = mesh.tris.copy()
    if m > 0:
        tsplit = tri_split_slot >= 0
        tri_map = np.concatenate([[0], np.cumsum(1 + tsplit.astype(np.int64))])
        tris_out = np.zeros((m_new, 3), dtype=np.int32)
        tris_out[tri_map[:-1][~tsplit]] = mesh.tris[~tsplit]
        trows = np.nonzero(tsplit)[0]
        tt = mesh.tris[trows].astype(np.int64)
        ts = tri_split_slot[trows]
        lo = et.slot_row[ts]
        hi = et.col_idx[ts].astype(np.int64)
        pi3 = np.zeros(trows.size, dtype=np.int64)
        pj3 = np.zeros(trows.size, dtype=np.int64)
        for i, j in TRI_PAIRS:
            hit = ((tt[:, i] == lo) & (tt[:, j] == hi)) | ((tt[:, i] == hi) & (tt[:, j] == lo))
            pi3 = np.where(hit, i, pi3)
            pj3 = np.where(hit, j, pj3)
        for c in range(2):
            child = tt.copy()
            child[np.arange(trows.size), pi3 if c == 0 else pj3] = new_index[ts]
            tris_out[tri_map[trows] + c] = child.astype(np.int32)

    out = Mesh(rest_out, tets_out, poses_out, mat_out, s_out, l_out, mass, inv_out, tris_out)
    return RefineResult(out, q_out, qd_out, score, state, n_new_v, False, refining)


# ---------------------------------------------------------------------------
# properties the reference's tests check (tests/test_refinement.py)
# ---------------------------------------------------------------------------


def rest_volume_total(rest_q, tets):
    """Sum of signed rest volumes in float64 (the reference test's
    _rest_volume_total); also returns the smallest volume."""
    x = np.asarray(rest_q, dtype=np.float64)[np.asarray(tets, dtype=np.int64)]
    Dm = np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], axis=2)
    v = np.linalg.det(Dm) / 6.0
    return float(v.sum()), float(v.min()) if v.size else 0.0


def is_conforming(tets):
    """Every face is shared by at most two tets and no tet edge passes
    through a vertex of the mesh: for every tet, each of its faces either
    lies on one other tet or on none (a hanging vertex would leave a face
    covered by two smaller faces)."""
    tets = np.sort(np.asarray(tets, dtype=np.int64), axis=1)
    faces = np.concatenate([tets[:, [1, 2, 3]], tets[:, [0, 2, 3]], tets[:, [0, 1, 3]], tets[:, [0, 1, 2]]])
    _, counts = np.unique(faces, axis=0, return_counts=True)
    return bool(np.all(counts <= 2))
