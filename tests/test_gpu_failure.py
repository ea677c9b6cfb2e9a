"""The timeout path, driven from the host (mfem_plan_inject_timeout): the
plan's sticky error flag is set as a bounded wait that gave up would set it,
so no kernel waits, spins or faults.  The persistent kernels of the next
step leave at their first check, the stats call reports MFEM_TIMEOUT and
re-arms every grid barrier of the plan, and the plan then steps normally.
"""
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib, beams
from mfem_gb300.batched import BatchedSolver

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def run_steps(solver, mesh, s0, s1, n):
    for _ in range(n):
        solver.step(s0, s1, None, None, mesh.spec.dt)
        s0, s1 = s1, s0
    return s0, s1


@pytest.mark.parametrize("kw", [dict(), dict(preconditioner="fsai"), dict(solver_precision="fp16"),
                                dict(solver_precision="fp32_refined"), dict(line_search=True)],
                         ids=["single_reduction", "factor", "mixed_fp16", "mixed_fp32", "line_search"])
def test_injected_timeout_is_reported_and_the_plan_recovers(kw):
    mesh = beams.build_beam("nh_beam", cells=(16, 4, 4))
    kw = dict(kw)
    kw.setdefault("line_search", False)
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=mesh.spec.iterations, energy=mesh.spec.energy, **kw)
    s0, s1 = model.state(), model.state()
    s0, s1 = run_steps(solver, mesh, s0, s1, 1)
    assert all(st["status"] == _lib.MFEM_OK for st in solver.solve_stats())
    q_before = s0.particle_q.clone()

    solver.inject_timeout()
    solver.step(s0, s1, None, None, mesh.spec.dt)
    with pytest.raises(_lib.MfemError) as err:
        solver.solve_stats()
    assert err.value.code == _lib.MFEM_TIMEOUT
    # the re-armed plan steps on from the state before the failed step
    s1.particle_q.copy_(q_before)
    s1, s0 = run_steps(solver, mesh, s1, s0, 2)
    assert all(st["status"] == _lib.MFEM_OK for st in solver.solve_stats())
    assert torch.isfinite(s1.particle_q).all()


def test_injected_timeout_in_a_batch_is_reported_and_the_batch_recovers():
    """Bodies in one persistent launch, each group of CTAs on its own
    barrier counter: the per-body stats call reports the timeout and re-arms
    every body's counter."""
    batch = beams.batched_bodies(6, seed=3, nx=(2, 7), nyz=(1, 3))
    bs = BatchedSolver(batch, device=DEV)
    A, B = bs.state(), bs.model.state()
    bs.step(A, B)
    assert (bs.body_stats()["status"] == _lib.MFEM_OK).all()
    q_before = B.particle_q.clone()
    bs.solver.inject_timeout()
    bs.step(B, A)
    with pytest.raises(_lib.MfemError) as err:
        bs.body_stats()
    assert err.value.code == _lib.MFEM_TIMEOUT
    A.particle_q.copy_(q_before)
    for _ in range(2):
        bs.step(A, B)
        A, B = B, A
    assert (bs.body_stats()["status"] == _lib.MFEM_OK).all()
    assert torch.isfinite(A.particle_q).all()
