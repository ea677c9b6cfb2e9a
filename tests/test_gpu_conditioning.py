"""Nearly singular stretch Hessians (strongly stretched Neo-Hookean tets).

The reference evaluates lambda = -H_l (g_l - G dx) and ds = -H_s^-1 (SYM
lambda + g_s) with g_l = c + SYM H_s^-1 g_s.  With H_l = INV_SYM H_s INV_SYM
and u = c - G dx these are exactly lambda = -(H_l u + INV_SYM g_s) and
ds = INV_SYM u, which the library evaluates: in the reference's order fp32
rounding is amplified by cond(H_s), above 1e4 for such tets, and the
Neo-Hookean beam at 32x8x8 cells then left the float64 oracle's trajectory
at step 20 and diverged at step 23.
"""
import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib, beams

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
INV_SYM = np.array([1.0, 1.0, 1.0, 0.5, 0.5, 0.5])


def test_local_solve_is_the_cancellation_free_form():
    mesh = beams.build_beam("nh_beam", cells=(16, 4, 4))
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=8, energy="neohookean", line_search=False)
    A, B = model.state(), model.state()
    for _ in range(3):
        solver.step(A, B, None, None, mesh.spec.dt)
        A, B = B, A
    q = A.particle_q.clone()
    x = q.clone()
    solver.predict(q, A.particle_qd, mesh.spec.dt)
    solver.update_system(x)
    solver.assemble(x, mesh.spec.dt)
    solver.global_solve(0)
    T = mesh.T
    s0 = solver.tet_stretch.cpu().numpy().astype(np.float64)
    c = solver.read_buffer("constraint").cpu().numpy().astype(np.float64).reshape(6, T).T
    G = solver.read_buffer("grad_constraint").cpu().numpy().astype(np.float64).reshape(72, T).T.reshape(T, 6, 12)
    gs = solver.read_buffer("grad_s").cpu().numpy().astype(np.float64).reshape(6, T).T
    iu = np.triu_indices(6)
    Hl = np.zeros((T, 6, 6))
    Hl[:, iu[0], iu[1]] = solver.read_buffer("h_lambda").cpu().numpy().astype(np.float64).reshape(21, T).T
    Hl = Hl + np.triu(Hl, 1).transpose(0, 2, 1)
    dx = solver.read_buffer("dx").cpu().numpy().astype(np.float64).reshape(-1, 3)
    solver.local_solve(x)
    torch.cuda.synchronize()
    s1 = solver.tet_stretch.cpu().numpy().astype(np.float64)
    lam = solver.tet_lambda.cpu().numpy().astype(np.float64)
    u = c - np.einsum("tij,tj->ti", G, dx[mesh.tet_indices].reshape(T, 12))
    ds_ref = INV_SYM * u
    lam_ref = -(np.einsum("tij,tj->ti", Hl, u) + INV_SYM * gs)
    assert np.abs((s1 - s0) - ds_ref).max() <= 1e-5 * np.abs(ds_ref).max() + 1e-7
    assert np.abs(lam - lam_ref).max() <= 1e-5 * np.abs(lam_ref).max()


def test_beam_stays_on_its_trajectory_past_step_20():
    """32x8x8 cells: all solves converge and the beam stays bounded through
    step 24 (it diverged at step 23 when lambda and ds went through H_s^-1)."""
    mesh = beams.build_beam("nh_beam", cells=(32, 8, 8))
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=8, energy="neohookean", line_search=False)
    A, B = model.state(), model.state()
    A.particle_q.copy_(torch.as_tensor(mesh.q0, device=DEV))
    extent = float(np.abs(mesh.q0).max())
    for step in range(25):
        solver.step(A, B, None, None, mesh.spec.dt)
        A, B = B, A
        st = solver.solve_stats()
        assert all(s["status"] == _lib.MFEM_OK for s in st), (step, st)
        q = A.particle_q
        assert bool(torch.isfinite(q).all()) and float(q.abs().max()) < 1.1 * extent, step


@pytest.mark.parametrize("line_search", [False, True])
def test_full_beam_fifty_steps_converge(line_search):
    """The nh_beam workload's whole 50-step run (64x16x16 cells): every solve
    converges and the beam stays bounded, with the plain update and with the
    reference's default line search."""
    mesh = beams.build_beam("nh_beam")
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=mesh.spec.iterations, energy=mesh.spec.energy,
                            line_search=line_search)
    A, B = model.state(), model.state()
    A.particle_q.copy_(torch.as_tensor(mesh.q0, device=DEV))
    extent = float(np.abs(mesh.q0).max())
    for step in range(50):
        solver.step(A, B, None, None, mesh.spec.dt)
        A, B = B, A
        assert all(s["status"] == _lib.MFEM_OK for s in solver.solve_stats()), step
        if line_search:
            assert all(e["status"] == _lib.MFEM_OK for e in solver.line_search_stats()), step
    q = A.particle_q
    assert bool(torch.isfinite(q).all()) and float(q.abs().max()) < 1.1 * extent
