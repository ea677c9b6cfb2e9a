"""Adaptive refinement on the GPU (mfem_refine through the C ABI, and
RefinementSolver with enable_refinement) against the CPU oracle.

Topology (tets, tris, which edges split, new-vertex numbering) must match the
oracle exactly; new positions, velocities and rest positions too (same
operations, round-to-nearest); DmInv, masses and inverse masses within 1e-6
relative.  Whole runs are held to the reference's own properties
(tests/test_refinement.py): rest volume conserved within 1e-6, no orphaned
vertex, the mesh grows, growth only on refining steps, finite states.
"""
import ctypes

import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib
from mfem_gb300.refinement_model import soft_grid
from oracle import contact_oracle as co
from oracle import refine_oracle as ro
from tests.refine_cases import beam_mesh, deformed, grid_mesh, hanging_edges

pytestmark = pytest.mark.gpu

DEV = torch.device("cuda:0")
LIB = None


def lib():
    global LIB
    if LIB is None:
        LIB = _lib.load()
    return LIB


def _t(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=DEV).contiguous()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class DevicePass:
    """A plan of `mesh` and the capacity buffers of one mfem_refine call."""

    def __init__(self, mesh: ro.Mesh, energy="arap", caps=(4, 4, 4), shapes=None, tris=None):
        L = lib()
        self.mesh = mesh
        n, T = mesh.rest_q.shape[0], mesh.tets.shape[0]
        cfg = _lib.default_config()
        cfg.energy = _lib.ENERGY[energy]
        cfg.line_search = 0
        plan = ctypes.c_void_p()
        P = lambda a: np.ascontiguousarray(a).ctypes.data_as(ctypes.c_void_p)
        self._keep = [np.ascontiguousarray(a) for a in (mesh.tets, mesh.poses, mesh.materials, mesh.rest_q,
                                                        mesh.mass, mesh.inv_mass)]
        g = np.array([0.0, -9.81, 0.0], np.float32)
        rc = L.mfem_plan_create(ctypes.byref(cfg), n, T, *[P(a) for a in self._keep], P(g), 0, ctypes.byref(plan))
        assert rc == 0, L.mfem_plan_last_error(None).decode()
        self.plan = plan
        self.m = 0
        if shapes is not None:
            ccfg = _lib.MfemContactConfig()
            L.mfem_contact_config_default(ctypes.byref(ccfg))
            ccfg.d1 = 0.2
            ccfg.d0 = 0.02
            tr = np.zeros((0, 3), np.int32) if tris is None else np.ascontiguousarray(tris, np.int32)
            S = len(shapes)
            arrs = [np.array([s["type"] for s in shapes], np.int32),
                    np.array([s["pose"] for s in shapes], np.float32),
                    np.array([s["scale"] for s in shapes], np.float32), np.full(S, -1, np.int32),
                    np.zeros(S, np.float32)]
            self._keep += arrs + [tr]
            rc = L.mfem_plan_set_contact(plan, ctypes.byref(ccfg), S, *[P(a) for a in arrs], 0, tr.shape[0], P(tr))
            assert rc == 0, L.mfem_plan_last_error(plan).decode()
            self.m = tr.shape[0]
        for which, arr in ((0, mesh.stretch), (1, mesh.lam)):
            src = _t(arr)
            assert L.mfem_plan_copy_in(plan, which, _ptr(src), src.numel() * 4, None) == 0
        torch.cuda.synchronize()
        self.cap_v, self.cap_t, self.cap_m = n * caps[0], T * caps[1], max(self.m * caps[2], 1)
        z = lambda shape, dt=torch.float32: torch.zeros(shape, dtype=dt, device=DEV)
        self.out = dict(tets=z((self.cap_t, 4), torch.int32), poses=z((self.cap_t, 9)), materials=z((self.cap_t, 3)),
                        stretch=z((self.cap_t, 6)), lam=z((self.cap_t, 6)), rest=z((self.cap_v, 3)),
                        mass=z(self.cap_v), inv_mass=z(self.cap_v), tris=z((self.cap_m, 3), torch.int32),
                        counts=z(8, torch.int32))
        om = _lib.MfemRefineMesh()
        om.max_particles, om.max_tets, om.max_tris = self.cap_v, self.cap_t, self.cap_m
        for field, key in (("tet_indices", "tets"), ("tet_poses", "poses"), ("tet_materials", "materials"),
                           ("tet_stretch", "stretch"), ("tet_lambda", "lam"), ("rest_q", "rest"),
                           ("particle_mass", "mass"), ("particle_inv_mass", "inv_mass"), ("tri_indices", "tris"),
                           ("counts", "counts")):
            setattr(om, field, self.out[key].data_ptr())
        self.om = om

    def run(self, q, qd, rcfg: ro.RefineConfig, tet_scores=None, vertex_scores=None, distance=None, shape_id=None,
            pass_counter=None):
        L = lib()
        c = _lib.MfemRefineConfig()
        L.mfem_refine_config_default(ctypes.byref(c))
        c.scoring = _lib.REFINE_SCORING[rcfg.scoring]
        for f in ("threshold", "tet_score_weight", "vertex_score_weight", "penetrating_edge_score",
                  "min_edge_length", "contact_d1", "elastic_weight", "vertex_contact_weight", "tri_contact_weight",
                  "split_position", "density"):
            setattr(c, f, float(getattr(rcfg, f)))
        c.conflict_iterations = rcfg.conflict_iterations
        c.refine_every = rcfg.refine_every
        n = self.mesh.rest_q.shape[0]
        self.q = torch.zeros((self.cap_v, 3), dtype=torch.float32, device=DEV)
        self.qd = torch.zeros_like(self.q)
        self.q[:n] = _t(q)
        self.qd[:n] = _t(qd)
        keep = []
        inp = _lib.MfemRefineInputs()
        if tet_scores is not None:
            keep.append(_t(tet_scores))
            inp.tet_scores = keep[-1].data_ptr()
        if vertex_scores is not None:
            keep.append(_t(vertex_scores))
            inp.vertex_scores = keep[-1].data_ptr()
        if distance is not None:
            keep.append(_t(distance))
            inp.particle_distance = keep[-1].data_ptr()
            keep.append(_t(shape_id, torch.int32))
            inp.particle_shape_id = keep[-1].data_ptr()
        pc = None
        if pass_counter is not None:
            pc = _t(np.array([pass_counter], np.int32), torch.int32)
        rc = L.mfem_refine(self.plan, ctypes.byref(c), ctypes.byref(inp), _ptr(self.q), _ptr(self.qd), _ptr(pc),
                           ctypes.byref(self.om), None)
        assert rc == 0, L.mfem_plan_last_error(self.plan).decode()
        torch.cuda.synchronize()
        counts = self.out["counts"].cpu().numpy()
        n2, T2, m2 = int(counts[0]), int(counts[1]), int(counts[2])
        o = {k: v.cpu().numpy() for k, v in self.out.items()}
        res = dict(counts=counts, tets=o["tets"][:T2], poses=o["poses"][:T2].reshape(-1, 3, 3),
                   materials=o["materials"][:T2], stretch=o["stretch"][:T2], lam=o["lam"][:T2], rest=o["rest"][:n2],
                   mass=o["mass"][:n2], inv_mass=o["inv_mass"][:n2], tris=o["tris"][:m2],
                   q=self.q[:n2].cpu().numpy(), qd=self.qd[:n2].cpu().numpy())
        if pc is not None:
            res["pass_counter"] = int(pc.cpu().item())
        return res

    def close(self):
        lib().mfem_plan_destroy(self.plan)


def _compare(dev, res: ro.RefineResult):
    m = res.mesh
    assert int(dev["counts"][3]) == res.split_edges
    assert bool(dev["counts"][4]) == res.overflow
    np.testing.assert_array_equal(dev["tets"], m.tets)
    np.testing.assert_array_equal(dev["tris"], m.tris)
    np.testing.assert_array_equal(dev["q"], res.q)
    np.testing.assert_array_equal(dev["qd"], res.qd)
    np.testing.assert_array_equal(dev["rest"], m.rest_q)
    np.testing.assert_array_equal(dev["stretch"], m.stretch)
    np.testing.assert_array_equal(dev["lam"], m.lam)
    np.testing.assert_array_equal(dev["materials"], m.materials)
    np.testing.assert_allclose(dev["poses"], m.poses, rtol=1e-6, atol=1e-6 * np.abs(m.poses).max())
    np.testing.assert_allclose(dev["mass"], m.mass, rtol=1e-6)
    np.testing.assert_allclose(dev["inv_mass"], m.inv_mass, rtol=1e-6)


@pytest.mark.parametrize("scoring", ["legacy", "geometric"])
def test_pass_matches_oracle_on_the_reference_grid(scoring):
    mesh = grid_mesh()
    q = deformed(mesh.rest_q)
    qd = deformed(np.zeros_like(mesh.rest_q), seed=7, amp=0.1)
    E = np.random.default_rng(2).uniform(0.0, 1.0, mesh.tets.shape[0]).astype(np.float32)
    cfg = (ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0, density=1.0)
           if scoring == "legacy" else
           ro.RefineConfig(scoring="geometric", threshold=1e-6, min_edge_length=0.05, density=1.0))
    dp = DevicePass(mesh)
    try:
        for k in range(3):
            dev = dp.run(q, qd, cfg, tet_scores=E)
            ref = ro.refine_pass(mesh, q, qd, cfg, tet_scores=E, max_particles=dp.cap_v, max_tets=dp.cap_t)
            assert ref.split_edges > 0
            _compare(dev, ref)
    finally:
        dp.close()


def test_pass_matches_oracle_on_nh_beam():
    """The 64 x 16 x 16 Neo-Hookean beam (98,304 tets): a legacy pass with
    random tet scores splits thousands of edges, exactly as the oracle."""
    mesh, _ = beam_mesh("nh_beam")
    q = deformed(mesh.rest_q, amp=1e-3)
    E = np.random.default_rng(11).lognormal(0.0, 1.0, mesh.tets.shape[0]).astype(np.float32)
    cfg = ro.RefineConfig(scoring="legacy", threshold=4.0e-2, tet_score_weight=1.0, density=1000.0)
    dp = DevicePass(mesh, energy="neohookean", caps=(2, 2, 1))
    try:
        dev = dp.run(q, np.zeros_like(q), cfg, tet_scores=E)
        ref = ro.refine_pass(mesh, q, np.zeros_like(q), cfg, tet_scores=E, max_particles=dp.cap_v,
                             max_tets=dp.cap_t)
        assert ref.split_edges > 1000
        _compare(dev, ref)
        vol0 = ro.rest_volume_total(mesh.rest_q, mesh.tets)[0]
        assert ro.rest_volume_total(dev["rest"], dev["tets"])[0] == pytest.approx(vol0, rel=1e-9)
    finally:
        dp.close()


def test_energies_computed_on_the_device():
    """tet_scores left to the library: the elastic energy of the plan's s,
    which must select the same edges as the oracle's energies."""
    mesh = grid_mesh(dims=(4, 3, 2), seed=3)
    mesh.stretch = (mesh.stretch + np.random.default_rng(9).normal(0, 0.05, mesh.stretch.shape)).astype(np.float32)
    q = deformed(mesh.rest_q)
    cfg = ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0)
    dp = DevicePass(mesh)
    try:
        dev = dp.run(q, np.zeros_like(q), cfg)
        ref = ro.refine_pass(mesh, q, np.zeros_like(q), cfg, energy="arap", max_particles=dp.cap_v,
                             max_tets=dp.cap_t)
        assert ref.split_edges > 0
        np.testing.assert_array_equal(dev["tets"], ref.mesh.tets)
        np.testing.assert_array_equal(dev["q"], ref.q)
    finally:
        dp.close()


def _capsule(pos, radius=0.1, half=0.5):
    # capsule axis along world y: rotate local +Z to +Y (quaternion about x by -90 degrees)
    s = np.sqrt(0.5)
    return dict(type=co.SHAPE_CAPSULE, pose=[pos[0], pos[1], pos[2], -s, 0.0, 0.0, s], scale=[radius, half, 0.0])


def test_geometric_contact_scores_match_oracle():
    """Geometric scores with the capsule term, the distances and shapes given
    as inputs (float32, from the oracle's SDFs): exact agreement; then the
    same pass with the library's own distances selects edges near the tool."""
    mesh = grid_mesh()
    q = mesh.rest_q.copy()
    shape = _capsule((0.3, 0.2, 0.5))
    shapes = [shape, dict(type=co.SHAPE_PLANE, pose=[0, -1.0, 0, 0, 0, 0, 1], scale=[0, 0, 0])]
    cshapes = [dict(type=s["type"], transform=np.array(s["pose"], np.float64),
                    scale=np.array(s["scale"], np.float64), body=-1) for s in shapes]
    d, _, sid = co.vertex_distances(q, cshapes, np.zeros((0, 7)))
    d = d.astype(np.float32)
    cfg = ro.RefineConfig(scoring="geometric", threshold=0.5, min_edge_length=0.05, contact_d1=0.2,
                          elastic_weight=0.0)
    dp = DevicePass(mesh, shapes=shapes)
    try:
        E = np.zeros(mesh.tets.shape[0], np.float32)
        dev = dp.run(q, np.zeros_like(q), cfg, tet_scores=E, distance=d, shape_id=sid)
        ref = ro.refine_pass(mesh, q, np.zeros_like(q), cfg, tet_scores=E, distance=d, shape_id=sid,
                             shape_type=[s["type"] for s in shapes], max_particles=dp.cap_v, max_tets=dp.cap_t)
        assert ref.split_edges > 0
        _compare(dev, ref)
        own = dp.run(q, np.zeros_like(q), cfg, tet_scores=E)
        assert int(own["counts"][3]) > 0
        new = own["rest"][mesh.rest_q.shape[0]:]
        dn, _, _ = co.vertex_distances(new, cshapes[:1], np.zeros((0, 7)))
        assert np.all(dn < 0.4)
    finally:
        dp.close()


def test_pass_counter_gates_on_the_device():
    mesh = grid_mesh()
    q = deformed(mesh.rest_q)
    E = np.ones(mesh.tets.shape[0], np.float32)
    cfg = ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0, refine_every=3)
    dp = DevicePass(mesh)
    try:
        for c in range(5):
            dev = dp.run(q, np.zeros_like(q), cfg, tet_scores=E, pass_counter=c)
            assert dev["pass_counter"] == c + 1
            assert int(dev["counts"][5]) == (1 if c % 3 == 0 else 0)
            assert (int(dev["counts"][3]) > 0) == (c % 3 == 0)
            if c % 3:
                np.testing.assert_array_equal(dev["tets"], mesh.tets)
                np.testing.assert_array_equal(dev["mass"], mesh.mass)
    finally:
        dp.close()


def test_capacity_overflow_drops_the_pass():
    mesh = grid_mesh()
    q = deformed(mesh.rest_q)
    E = np.ones(mesh.tets.shape[0], np.float32)
    cfg = ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0)
    dp = DevicePass(mesh, caps=(4, 1, 1))
    try:
        dev = dp.run(q, np.zeros_like(q), cfg, tet_scores=E)
        assert int(dev["counts"][4]) == 1 and int(dev["counts"][3]) == 0
        np.testing.assert_array_equal(dev["tets"], mesh.tets)
        np.testing.assert_array_equal(dev["rest"], mesh.rest_q)
    finally:
        dp.close()


def test_contact_tris_split_with_their_edges():
    mesh = grid_mesh()
    tris = co.boundary_tris(mesh.tets, mesh.rest_q)
    mesh.tris = np.asarray(tris, np.int32)
    q = deformed(mesh.rest_q)
    E = np.random.default_rng(5).uniform(0.0, 1.0, mesh.tets.shape[0]).astype(np.float32)
    cfg = ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0, vertex_score_weight=0.0)
    # a plane far below the body (z = -5, normal +z): contact on, nothing penetrates
    shapes = [dict(type=co.SHAPE_PLANE, pose=[0, 0, -5.0, 0, 0, 0, 1], scale=[0, 0, 0])]
    dp = DevicePass(mesh, shapes=shapes, tris=tris, caps=(4, 4, 4))
    try:
        dev = dp.run(q, np.zeros_like(q), cfg, tet_scores=E)
        ref = ro.refine_pass(mesh, q, np.zeros_like(q), cfg, tet_scores=E, max_particles=dp.cap_v,
                             max_tets=dp.cap_t, max_tris=dp.cap_m,
                             midpoint_distance=lambda mid: mid[:, 2] + 5.0)
        assert ref.split_edges > 0
        _compare(dev, ref)
    finally:
        dp.close()


# -- whole runs through RefinementSolver (tests/test_refinement.py) -------------


def _grid_model(device=DEV):
    x, tets, mats = soft_grid(3, 2, 2, 0.2, 0.2, 0.2, 10.0, 1.0, 0.0)
    mesh = grid_mesh()
    inv = mesh.inv_mass.copy()
    model = Model(x, np.zeros_like(x), mesh.mass, inv, tets, mesh.poses, mats, np.array([0.0, -9.81, 0.0]),
                  device=device)
    return model.pad_particles(4 * x.shape[0]), tets.shape[0]


SCORING = {
    "legacy": dict(refine_tet_score_weight=1.0),
    "geometric": dict(refine_scoring="geometric", refine_geometric_threshold=1.0e-6, refine_min_edge_length=0.05),
}


@pytest.mark.parametrize("scoring", sorted(SCORING))
def test_refinement_conserves_volume_and_grows_mesh(scoring):
    model, T0 = _grid_model()
    solver = MixedFEMSolver(model, iterations=8, max_tets=4 * T0, max_particles=model.particle_count,
                            enable_refinement=True, refine_every_n_steps=3, min_refine_score=1.0e-6,
                            **SCORING[scoring])
    s0, s1 = model.state(), model.state()
    mesh0 = solver.refined_mesh()
    vol0 = ro.rest_volume_total(mesh0["rest"], mesh0["tets"])[0]
    n0, t0 = solver.active_particle_count, solver.active_tet_count
    grew_on = []
    for i in range(60):
        before = solver.active_tet_count
        solver.step(s0, s1, None, None, 1.0 / 240.0)
        s0, s1 = s1, s0
        if solver.active_tet_count > before:
            grew_on.append(i)
        n = solver.active_particle_count
        q = s0.particle_q[:n].cpu().numpy()
        assert np.isfinite(q).all() and np.isfinite(s0.particle_qd[:n].cpu().numpy()).all()
        mesh = solver.refined_mesh()
        assert mesh["tets"].max() < n and mesh["tets"].min() >= 0
        vol, vmin = ro.rest_volume_total(mesh["rest"], mesh["tets"])
        assert vmin > -1e-9
        assert vol == pytest.approx(vol0, abs=1e-6)
    assert solver.active_tet_count > t0 and solver.active_particle_count > n0
    assert grew_on and all(i % 3 == 0 for i in grew_on), grew_on
    assert ro.is_conforming(solver.refined_mesh()["tets"])


def test_refined_step_matches_a_plan_of_the_refined_mesh():
    """After a splitting pass the step runs on a plan of the refined mesh: the
    same step from a fresh solver built on that mesh (s, lambda carried) gives
    the same positions."""
    model, T0 = _grid_model()
    solver = MixedFEMSolver(model, iterations=8, max_tets=4 * T0, enable_refinement=True, refine_every_n_steps=1,
                            min_refine_score=1.0e-6, refine_tet_score_weight=1.0, line_search=False)
    s0, s1 = model.state(), model.state()
    for _ in range(60):
        solver.step(s0, s1, None, None, 1.0 / 240.0)
        s0, s1 = s1, s0
        if solver.active_tet_count > T0:
            break
    assert solver.active_tet_count > T0
    mesh = solver.refined_mesh()
    n = solver.active_particle_count
    # one more step on the refined mesh, refinement off from here on
    solver.refine_every_n_steps = 10 ** 9
    solver._refine_pass = 1
    start_q, start_qd = s0.particle_q.clone(), s0.particle_qd.clone()
    solver.step(s0, s1, None, None, 1.0 / 240.0)
    plain = Model(mesh["rest"], np.zeros_like(mesh["rest"]), mesh["mass"], mesh["inv_mass"], mesh["tets"],
                  mesh["poses"], mesh["materials"], np.array([0.0, -9.81, 0.0]), device=DEV)
    other = MixedFEMSolver(plain, iterations=8, line_search=False)
    other.write_buffer("tet_stretch", torch.as_tensor(mesh["tet_stretch"]).reshape(-1))
    other.write_buffer("tet_lambda", torch.as_tensor(mesh["tet_lambda"]).reshape(-1))
    a = plain.state()
    a.particle_q.copy_(start_q[:n])
    a.particle_qd.copy_(start_qd[:n])
    b = plain.state()
    other.step(a, b, None, None, 1.0 / 240.0)
    np.testing.assert_array_equal(b.particle_q.cpu().numpy(), s1.particle_q[:n].cpu().numpy())


def test_contact_driven_refinement_through_the_solver():
    """Geometric scoring driven by contact only (elastic weight 0): the
    cantilever pressed by a descending capsule tool onto a ground plane, with
    surface tris in the tri barrier.  Edges split only near the tool, on
    refining steps; the plan's contact tris stay the boundary of the refined
    tets; rest volume conserved; the trajectory stays finite."""
    from tests.test_gpu_contact import PARAMS, PLANE_POSE, tool_pose
    from mfem_gb300 import beams
    mesh = beams.build_beam("cantilever")
    tris = co.boundary_tris(mesh.tet_indices, mesh.rest_q.astype(np.float64))
    base = Model.from_beam(mesh, device=DEV)
    base.add_body(tool_pose(0)[0])
    base.add_shape_plane(PLANE_POSE)
    base.add_shape_capsule(0.03, 0.15, body=0)
    base.set_tri_indices(tris)
    model = base.pad_particles(4 * mesh.n)
    solver = MixedFEMSolver(model, iterations=8, line_search=False, max_tets=4 * mesh.T, enable_refinement=True,
                            refine_every_n_steps=2, refine_scoring="geometric", refine_geometric_threshold=0.2,
                            refine_min_edge_length=0.03, refine_elastic_weight=0.0, refine_density=1000.0,
                            **PARAMS)
    vol0 = ro.rest_volume_total(mesh.rest_q, mesh.tet_indices)[0]
    A, B = model.state(), model.state()
    grew_on = []
    for k in range(8):
        before = solver.active_tet_count
        B.body_q.copy_(torch.as_tensor(tool_pose(k), device=DEV))
        A.body_q.copy_(B.body_q)
        solver.step(A, B, None, None, mesh.spec.dt)
        A, B = B, A
        if solver.active_tet_count > before:
            grew_on.append(k)
        n = solver.active_particle_count
        assert np.isfinite(A.particle_q[:n].cpu().numpy()).all()
    assert grew_on and all(k % 2 == 0 for k in grew_on), grew_on
    m = solver.refined_mesh()
    n = solver.active_particle_count
    assert m["tets"].max() < n
    vol, vmin = ro.rest_volume_total(m["rest"], m["tets"])
    assert vmin > 0.0 and vol == pytest.approx(vol0, rel=1e-6)
    assert ro.is_conforming(m["tets"])
    new_rest = m["rest"][mesh.n:n]
    assert new_rest.shape[0] > 0 and np.all(np.abs(new_rest[:, 0] - 0.85) < 0.25), new_rest[:, 0]
    canon = lambda t: sorted(map(tuple, np.sort(np.asarray(t), axis=1)))
    assert canon(m["tris"]) == canon(co.boundary_tris(m["tets"], m["rest"].astype(np.float64)))
