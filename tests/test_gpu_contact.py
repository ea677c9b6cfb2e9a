"""GPU parity of contact against rigid shapes (src/mfem/refinement/contact.py)
with the CPU contact oracle.

Scene: the 10x2x2 ARAP cantilever (pinned at x = 0) pressed down at its free
end by a capsule tool on a kinematic body that descends 2 mm per step, onto a
ground plane 3 cm below the beam, with friction against both (mu 0.1 tool,
0.3 ground); surface tris take part in the tri barrier.

Tolerances (float32 kernels against the float64 oracle): per-vertex contact
blocks, gradients and energies 1e-4 of each quantity's largest magnitude;
per-tri distance 1e-5 absolute, weights and normals 1e-4; assembled blocks
and rhs 1e-5 of their scale; positions along a trajectory 1e-5 relative to
the largest position (the bar of the plain step).
"""
import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib, beams
from oracle import contact_oracle as C
from oracle import mfem_oracle as O

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
PARAMS = dict(contact_d0=1e-3, contact_d1=2e-2, contact_stiffness=1e3, friction_mu=[0.3, 0.1], friction_eps_v=1e-2)


def close(a, b, rtol, atol=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    err = np.abs(a - b).max()
    assert err <= rtol * scale + atol, f"max err {err:.3e} vs scale {scale:.3e} (rtol {rtol})"


def qaa(axis, deg):
    axis = np.asarray(axis, dtype=np.float64)
    axis /= np.linalg.norm(axis)
    h = np.radians(deg) / 2.0
    return (*(np.sin(h) * axis), np.cos(h))


PLANE_POSE = (0.0, -0.03, 0.0, *qaa((1.0, 0.0, 0.0), -90.0))


def tool_pose(k):
    return np.array([[0.85, 0.245 - 0.002 * k, 0.1, 0.0, 0.0, 0.0, 1.0]], dtype=np.float32)


def scene(line_search=False, iterations=8, use_cuda_graph=True, shapes=True, **extra):
    mesh = beams.build_beam("cantilever")
    tris = C.boundary_tris(mesh.tet_indices, mesh.rest_q.astype(np.float64))
    model = Model.from_beam(mesh, device=DEV)
    if shapes:
        model.add_body(tool_pose(0)[0])
        model.add_shape_plane(PLANE_POSE)
        model.add_shape_capsule(0.03, 0.15, body=0)
        model.set_tri_indices(tris)
    solver = MixedFEMSolver(model, iterations=iterations, line_search=line_search, use_cuda_graph=use_cuda_graph,
                            **(PARAMS if shapes else {}), **extra)
    oshapes = [dict(type=C.SHAPE_PLANE, transform=PLANE_POSE, scale=[0, 0, 0], body=-1),
               dict(type=C.SHAPE_CAPSULE, transform=[0, 0, 0, 0, 0, 0, 1], scale=[0.03, 0.15, 0.0], body=0)]
    co = C.ContactOracle(oshapes, d0=PARAMS["contact_d0"], d1=PARAMS["contact_d1"],
                         stiffness=PARAMS["contact_stiffness"], friction_mu=PARAMS["friction_mu"],
                         friction_eps_v=PARAMS["friction_eps_v"], tris=tris)
    return mesh, model, solver, co


def test_contact_terms_and_assembly_match_oracle():
    mesh, model, solver, co = scene()
    dt = mesh.spec.dt
    rng = np.random.default_rng(3)
    # start of step: the beam bent down onto the plane and the tool
    x_start = mesh.rest_q.astype(np.float64).copy()
    x_start[:, 1] -= 0.024 * (x_start[:, 0] ** 2)
    x = x_start + rng.normal(0, 1e-3, x_start.shape)
    x_start32, x32 = x_start.astype(np.float32), x.astype(np.float32)
    body_q = tool_pose(12)
    solver.set_body_poses(torch.as_tensor(body_q, device=DEV))
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=DEV)
    solver.predict(t(x_start32), torch.zeros_like(t(x_start32)), dt)
    xg = t(x32)
    solver.update_system(xg)
    solver.assemble(xg, dt)
    torch.cuda.synchronize()
    co.begin_step(x_start32.astype(np.float64), body_q.astype(np.float64))
    assert (co.force_lagged > 0).sum() >= 5, "the scene must have frictional contacts"
    np.testing.assert_allclose(solver.read_buffer("friction_force").cpu().numpy(), co.force_lagged,
                               rtol=2e-4, atol=1e-3 * co.force_lagged.max())
    Ev, gv, Hv = co.vertex_terms(x32.astype(np.float64), body_q.astype(np.float64), dt)
    Et, gt, _ = co.tri_terms(x32.astype(np.float64), body_q.astype(np.float64))
    assert (Ev > 0).sum() >= 5 and (Et > 0).sum() >= 2, "the scene must touch the plane and the tool"
    n = mesh.n
    close(solver.read_buffer("contact_block").cpu().numpy().reshape(n, 3, 3), Hv, 1e-4)
    close(solver.read_buffer("contact_gradient").cpu().numpy().reshape(n, 3), gv + gt, 1e-4)
    close(solver.read_buffer("contact_energy").cpu().numpy(), Ev, 1e-4)
    rec = solver.contact_tris()
    act = Et > 0
    close(rec[act, 1], Et[act], 1e-4)
    for tri in np.flatnonzero(act):
        i0, i1, i2 = co.tris[tri]
        d, w, nv, sid = C.tri_capsule_contact(x32[i0].astype(float), x32[i1].astype(float), x32[i2].astype(float),
                                              co.shapes, body_q.astype(np.float64))
        assert abs(rec[tri, 0] - d) <= 1e-5 and rec[tri, 10] == sid
        np.testing.assert_allclose(rec[tri, 7:10], w, atol=1e-4)
        np.testing.assert_allclose(rec[tri, 4:7], nv, atol=1e-4)
    # the assembled system carries the contact blocks and gradients
    ref = O.OracleSolver(mesh, dtype=np.float64, contact=co)
    ref.body_q = body_q.astype(np.float64)
    ref.s = solver.tet_stretch.cpu().numpy().astype(np.float64)
    el = ref.element_terms(x32.astype(np.float64))
    x_tilde = solver.read_buffer("x_tilde").cpu().numpy().reshape(n, 3).astype(np.float64)
    blocks, g, _ = ref.assemble(x32.astype(np.float64), x_tilde, dt, el)
    close(solver.read_buffer("h_values").cpu().numpy().reshape(-1, 3, 3), blocks, 1e-5)
    close(solver.read_buffer("rhs").cpu().numpy().reshape(n, 3), g, 1e-5)


def _tri_mesh_model(verts, capsule_pose):
    """One tet whose face (0, 1, 2) is the contact tri, and one capsule on a
    body at `capsule_pose` (radius 0.1, half height 0.5, D0 0.05, D1 0.2,
    stiffness 10: the reference's tests/test_tri_contact.py:23-27)."""
    v = np.asarray(list(verts) + [(0.0, 0.0, 1.0)], dtype=np.float32)
    tets = np.array([[0, 1, 2, 3]], dtype=np.int32)
    Dm = np.stack([v[1] - v[0], v[2] - v[0], v[3] - v[0]], axis=1).astype(np.float64)
    model = Model(v, np.zeros_like(v), np.ones(4), np.ones(4), tets, np.linalg.inv(Dm)[None].astype(np.float32),
                  np.array([[1.0, 1.0, 0.0]]), np.zeros(3), device=DEV)
    model.add_body(capsule_pose)
    model.add_shape_capsule(0.1, 0.5, body=0)
    model.set_tri_indices([[0, 1, 2]])
    solver = MixedFEMSolver(model, iterations=1, line_search=False, contact_d0=0.05, contact_d1=0.2,
                            contact_stiffness=10.0)
    x = torch.as_tensor(v, device=DEV)
    solver.predict(x, torch.zeros_like(x), 1.0 / 60.0)
    solver.update_system(x)
    solver.assemble(x, 1.0 / 60.0)
    torch.cuda.synchronize()
    return solver, v


BIG_TRI = [(-3.0, -3.0, 0.0), (3.0, -3.0, 0.0), (0.0, 3.0, 0.0)]


def test_tri_contact_known_answers():
    """tests/test_tri_contact.py:194-216 through the GPU kernels."""
    gap = 0.08
    solver, _ = _tri_mesh_model(BIG_TRI, (0.0, -1.0, gap + 0.1 + 0.5, 0.0, 0.0, 0.0, 1.0))
    rec = solver.contact_tris()[0]
    assert rec[0] == pytest.approx(gap, abs=1e-5)
    np.testing.assert_allclose(rec[4:7], [0.0, 0.0, -1.0], atol=1e-5)
    assert rec[1] > 0.0 and rec[7:10].sum() == pytest.approx(1.0, abs=1e-6)
    g = solver.read_buffer("contact_gradient").cpu().numpy().reshape(4, 3)[:3]
    assert (g[:, 2] > 0.0).all()
    total = g.sum(axis=0)
    assert np.abs(total[:2]).max() < 1e-4 * abs(total[2])
    e_touch = solver.contact_tris()[0][1]
    solver2, _ = _tri_mesh_model(BIG_TRI, (0.0, -1.0, 0.0, 0.0, 0.0, 0.0, 1.0))
    rec2 = solver2.contact_tris()[0]
    assert rec2[0] == pytest.approx(-0.1, abs=1e-6)
    assert rec2[1] > e_touch > 0.0


@pytest.mark.parametrize("pos,rot", [
    ((0.3, -0.8, 0.08 + 0.1 + 0.5), (0.1, 0.05, 0.0, 0.9937)),
    ((0.4, -3.3, 0.1), tuple(C.quat_mul(qaa((0.0, 0.0, 1.0), 15.0), qaa((0.0, 1.0, 0.0), 90.0)))),
])
def test_tri_contact_gradient_matches_oracle(pos, rot):
    """The reference's finite-difference cases (tests/test_tri_contact.py:
    253-277): the GPU's scattered tri gradient against the oracle's, which
    the CPU tests pin to finite differences."""
    rot = tuple(np.asarray(rot, dtype=np.float64) / np.linalg.norm(rot))
    solver, v = _tri_mesh_model(BIG_TRI, (*pos, *rot))
    shapes = [dict(type=C.SHAPE_CAPSULE, transform=[0, 0, 0, 0, 0, 0, 1], scale=[0.1, 0.5, 0.0], body=0)]
    co = C.ContactOracle(shapes, d0=0.05, d1=0.2, stiffness=10.0, tris=[[0, 1, 2]])
    body_q = np.array([[*pos, *rot]])
    E, gt, _ = co.tri_terms(v.astype(np.float64), body_q)
    Ev, gv, _ = co.vertex_terms(v.astype(np.float64), body_q, 1.0 / 60.0)
    rec = solver.contact_tris()[0]
    assert rec[1] == pytest.approx(E[0], rel=1e-4)
    close(solver.read_buffer("contact_gradient").cpu().numpy().reshape(4, 3), gt + gv, 1e-4)


@pytest.mark.parametrize("line_search,steps", [(False, 20), (True, 8)])
def test_contact_trajectory_matches_oracle(line_search, steps):
    mesh, model, solver, co = scene(line_search=line_search)
    ref = O.OracleSolver(mesh, dtype=np.float64, contact=co, line_search=line_search)
    A, B = model.state(), model.state()
    q, qd = mesh.q0.astype(np.float64), mesh.qd0.astype(np.float64)
    for k in range(steps):
        B.body_q.copy_(torch.as_tensor(tool_pose(k), device=DEV))
        solver.step(A, B, None, None, mesh.spec.dt)
        ref.body_q = tool_pose(k).astype(np.float64)
        q, qd = ref.step(q, qd, mesh.spec.dt)
        A, B = B, A
        assert all(st["status"] == 0 for st in solver.solve_stats())
        close(A.particle_q.cpu().numpy(), q, 1e-5)
    assert q[:, 1].min() < -0.015  # the tool pushed the tip onto the plane


@pytest.mark.parametrize("pc", ["fsai", "learned"])
def test_contact_trajectory_with_factor_preconditioner(pc):
    """Contact blocks enter H before the factor is built from it."""
    mesh, model, solver, co = scene(preconditioner=pc)
    ref = O.OracleSolver(mesh, dtype=np.float64, contact=co)
    A, B = model.state(), model.state()
    q, qd = mesh.q0.astype(np.float64), mesh.qd0.astype(np.float64)
    for k in range(12):
        B.body_q.copy_(torch.as_tensor(tool_pose(k), device=DEV))
        solver.step(A, B, None, None, mesh.spec.dt)
        ref.body_q = tool_pose(k).astype(np.float64)
        q, qd = ref.step(q, qd, mesh.spec.dt)
        A, B = B, A
        assert all(st["status"] == 0 for st in solver.solve_stats())
        close(A.particle_q.cpu().numpy(), q, 1e-5)


@pytest.mark.parametrize("pc", ["block_jacobi", "fsai"])
def test_contact_trajectory_with_mixed_precision(pc):
    """fp16 blocks with contact: the contact blocks enter H before its 16-bit
    copy is made, and the refined solve keeps the trajectory on the oracle."""
    mesh, model, solver, co = scene(preconditioner=pc, solver_precision="fp16")
    ref = O.OracleSolver(mesh, dtype=np.float64, contact=co)
    A, B = model.state(), model.state()
    q, qd = mesh.q0.astype(np.float64), mesh.qd0.astype(np.float64)
    for k in range(12):
        B.body_q.copy_(torch.as_tensor(tool_pose(k), device=DEV))
        solver.step(A, B, None, None, mesh.spec.dt)
        ref.body_q = tool_pose(k).astype(np.float64)
        q, qd = ref.step(q, qd, mesh.spec.dt)
        A, B = B, A
        assert all(st["status"] == 0 for st in solver.mixed_stats())
        close(A.particle_q.cpu().numpy(), q, 1e-5)


def test_graph_and_eager_agree_bitwise_with_contact():
    runs = []
    for graph in (True, False):
        mesh, model, solver, _ = scene(line_search=True, use_cuda_graph=graph)
        A, B = model.state(), model.state()
        for k in range(4):
            B.body_q.copy_(torch.as_tensor(tool_pose(k), device=DEV))
            solver.step(A, B, None, None, mesh.spec.dt)
            A, B = B, A
        runs.append(A.particle_q.clone())
    assert torch.equal(runs[0], runs[1])


def test_far_shapes_change_nothing():
    """Shapes out of reach (d > d1 everywhere) leave the step bit-identical
    to a solver without contact."""
    mesh = beams.build_beam("cantilever")
    plain = MixedFEMSolver(Model.from_beam(mesh, device=DEV), iterations=4, line_search=True)
    model = Model.from_beam(mesh, device=DEV)
    model.add_shape_plane((0.0, -5.0, 0.0, *qaa((1.0, 0.0, 0.0), -90.0)))
    model.add_shape_capsule(0.03, 0.15, pose=(5.0, 5.0, 5.0, 0.0, 0.0, 0.0, 1.0))
    model.set_tri_indices(C.boundary_tris(mesh.tet_indices, mesh.rest_q.astype(np.float64)))
    far = MixedFEMSolver(model, iterations=4, line_search=True, friction_mu=0.5)
    outs = []
    for solver, m in ((plain, plain.model), (far, model)):
        A, B = m.state(), m.state()
        for _ in range(3):
            solver.step(A, B, None, None, mesh.spec.dt)
            A, B = B, A
        outs.append(A.particle_q.clone())
    assert torch.equal(outs[0], outs[1])


def test_set_contact_rejects_bad_input():
    mesh = beams.build_beam("cantilever", cells=(2, 1, 1))
    for bad in ("tri", "body", "dist"):
        model = Model.from_beam(mesh, device=DEV)
        model.add_shape_capsule(0.03, 0.15, body=0 if bad == "body" else -1)
        kw = dict(contact_d0=0.2, contact_d1=0.1) if bad == "dist" else {}
        if bad == "tri":
            model.set_tri_indices([[0, 1, mesh.n - 1]])  # vertices 0 and n-1 share no tet
        with pytest.raises(_lib.MfemError):
            MixedFEMSolver(model, iterations=1, **kw)
