"""GPU edge cases: the solver's status reporting and degenerate inputs.

Failures are made on the host side (a NaN in the input, an iteration cap of
1, a singular block, a mesh with a vertex in no tet); no test faults, traps
or hangs the GPU.
"""
import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, beams, _lib
from oracle import mfem_oracle as O

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _solver(mesh, **kw):
    model = Model.from_beam(mesh, device=DEV)
    kw.setdefault("energy", mesh.spec.energy)
    return model, MixedFEMSolver(model, iterations=kw.pop("iterations", 2),
                                  line_search=kw.pop("line_search", False), **kw)


def test_iteration_cap_reports_maxiter_and_continues():
    mesh = beams.build_beam("cantilever")
    model, solver = _solver(mesh, cg_max_iterations=1)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, mesh.spec.dt)
    stats = solver.solve_stats()
    assert [s["status"] for s in stats] == [_lib.MFEM_MAXITER] * 2
    assert [s["iterations"] for s in stats] == [1, 1]
    assert torch.isfinite(s1.particle_q).all()


def test_nonfinite_input_reports_nonfinite():
    mesh = beams.build_beam("cantilever")
    model, solver = _solver(mesh)
    s0, s1 = model.state(), model.state()
    s0.particle_q[5, 1] = float("nan")
    solver.step(s0, s1, None, None, mesh.spec.dt)
    stats = solver.solve_stats()
    assert stats[0]["status"] == _lib.MFEM_NONFINITE


def test_zero_iterations_is_free_flight_prediction_copy():
    mesh = beams.build_beam("cantilever")
    model, solver = _solver(mesh, iterations=0)
    s0, s1 = model.state(), model.state()
    s0.particle_qd.fill_(0.25)
    solver.step(s0, s1, None, None, mesh.spec.dt)
    torch.cuda.synchronize()
    assert torch.equal(s1.particle_q, s0.particle_q)
    assert torch.all(s1.particle_qd == 0)


def test_isolated_vertex_falls_freely():
    """A vertex in no tet still owns a diagonal block (mass / dt^2): it follows
    the predictor x~ = x + v dt + g dt^2 / 2 exactly as the oracle does."""
    mesh = beams.build_beam("cantilever", cells=(2, 1, 1))
    n = mesh.n
    extra = np.array([[5.0, 5.0, 5.0]], dtype=np.float32)
    model = Model(np.concatenate([mesh.rest_q, extra]), np.zeros((n + 1, 3), np.float32),
                  np.concatenate([mesh.particle_mass, [2.0]]), np.concatenate([mesh.particle_inv_mass, [0.5]]),
                  mesh.tet_indices, mesh.tet_poses, mesh.tet_materials, mesh.gravity, device=DEV)
    solver = MixedFEMSolver(model, iterations=3, line_search=False)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, mesh.spec.dt)
    assert all(s["status"] == 0 for s in solver.solve_stats())
    dt = mesh.spec.dt
    expect = extra[0] + np.array([0.0, -9.81, 0.0]) * dt * dt / 2
    np.testing.assert_allclose(s1.particle_q[-1].cpu().numpy(), expect, rtol=1e-6, atol=1e-7)


def test_mesh_without_tets():
    q = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]], dtype=np.float32)
    model = Model(q, np.zeros_like(q), np.ones(2, np.float32), np.array([0.0, 1.0], np.float32),
                  np.zeros((0, 4), np.int32), np.zeros((0, 3, 3), np.float32), np.zeros((0, 3), np.float32),
                  np.array([0.0, -9.81, 0.0], np.float32), device=DEV)
    solver = MixedFEMSolver(model, iterations=2, line_search=False)
    s0, s1 = model.state(), model.state()
    solver.step(s0, s1, None, None, 0.01)
    assert all(s["status"] == 0 for s in solver.solve_stats())
    out = s1.particle_q.cpu().numpy()
    assert out[1, 1] < 0.0                   # free vertex falls
    assert abs(out[0, 1]) < abs(out[1, 1])   # attached vertex is held by the penalty spring


def test_unpreconditioned_cg_converges_to_same_answer():
    mesh = beams.build_beam("cantilever")
    outs = []
    for pre in (True, False):
        model, solver = _solver(mesh, iterations=2, preconditioner=pre, cg_max_iterations=5000)
        s0, s1 = model.state(), model.state()
        solver.step(s0, s1, None, None, mesh.spec.dt)
        assert all(s["status"] == 0 for s in solver.solve_stats())
        outs.append(s1.particle_q.cpu().numpy())
    assert np.abs(outs[0] - outs[1]).max() <= 1e-5 * np.abs(outs[0]).max()


def test_bad_arguments_raise():
    mesh = beams.build_beam("cantilever")
    model, solver = _solver(mesh)
    s0 = model.state()
    bad = torch.zeros((mesh.n, 3), dtype=torch.float64, device=DEV)
    with pytest.raises(ValueError):
        solver.step(s0, type(s0)(bad, s0.particle_qd), None, None, 0.01)
    with pytest.raises(_lib.MfemError):
        solver.step(s0, model.state(), None, None, -1.0)
    with pytest.raises(ValueError, match="max_tets"):
        MixedFEMSolver(model, iterations=2, enable_refinement=True)
    with pytest.raises(ValueError, match="refine_scoring"):
        MixedFEMSolver(model, iterations=2, enable_refinement=True, max_tets=model.tet_count,
                       refine_scoring="nearest")
    with pytest.raises(_lib.MfemError):
        MixedFEMSolver(model, iterations=2, line_search_max_iterations=-1)
    with pytest.raises(ValueError):
        MixedFEMSolver(model, iterations=2, energy="stvk")


def test_checkpoint_round_trip(tmp_path):
    mesh = beams.build_beam("cantilever")
    model, solver = _solver(mesh, iterations=8)
    s0, s1 = model.state(), model.state()
    for _ in range(3):
        solver.step(s0, s1, None, None, mesh.spec.dt)
        s0, s1 = s1, s0
    solver.save_state(str(tmp_path / "ck.npz"), s0)
    solver.step(s0, s1, None, None, mesh.spec.dt)
    expect = s1.particle_q.cpu().numpy()
    model2, solver2 = _solver(mesh, iterations=8)
    r0, r1 = model2.state(), model2.state()
    solver2.load_state(str(tmp_path / "ck.npz"), r0)
    solver2.step(r0, r1, None, None, mesh.spec.dt)
    np.testing.assert_array_equal(r1.particle_q.cpu().numpy(), expect)
