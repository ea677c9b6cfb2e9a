"""GPU parity of the backtracking line search (src/mfem/line_search.py:76-163,
src/mfem/refinement/solver.py:803-928) against the CPU oracle.

Tolerances (float32 kernels against the float64 oracle): local-solve lambda
and ds 3e-4 of each quantity's largest magnitude (lambda = -H_l (g_l - G dx)
cancels; the plain ARAP local solve meets 1e-4).  With the GPU's own lambda
and ds fed to the oracle: merit f0 and trial merit f1 1e-5 relative (float32
c; a float32 SVD at the float32-rounded trial point), slope t 1e-5 relative,
and the same decisions.  Along a trajectory: the first-iteration merit 1e-4
relative (it carries the float32 lambda) and positions 1e-5 relative to the
largest position (the bar of the plain step).  Decisions are compared where
the Armijo margin is far above float32 resolution (the first Newton
iteration of a step); later in a step the merit changes by about 1e-8, the
size of the threshold, and the reference's own float32 decisions there
depend on rounding.
"""
import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, beams
from oracle import mfem_oracle as O

pytestmark = pytest.mark.gpu

DEV = "cuda:0"


def close(a, b, rtol):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(np.abs(b).max(), 1e-30)
    err = np.abs(a - b).max()
    assert err <= rtol * scale, f"max err {err:.3e} vs scale {scale:.3e} (rtol {rtol})"


def make(name, cells=None, **kw):
    mesh = beams.build_beam(name, cells=cells)
    model = Model.from_beam(mesh, device=DEV)
    kw.setdefault("energy", mesh.spec.energy)
    solver = MixedFEMSolver(model, iterations=kw.pop("iterations", mesh.spec.iterations), **kw)
    return mesh, model, solver


def test_line_search_is_the_default():
    _, _, solver = make("cantilever")
    assert solver.line_search and solver.config.line_search == 1
    assert solver.config.line_search_max_iterations == 20
    assert solver.config.line_search_c == pytest.approx(0.01)


@pytest.mark.parametrize("name,cells", [("cantilever", None), ("nh_beam", (8, 2, 2))])
def test_line_search_stage_matches_oracle(name, cells):
    """One Newton iteration stage by stage after three steps: lambda, ds,
    f0, t, the decision and the updated x, s against the oracle run on the
    GPU's own x, s, x~ and dx."""
    mesh, model, solver = make(name, cells)
    dt = mesh.spec.dt
    A, B = model.state(), model.state()
    for _ in range(3):
        solver.step(A, B, None, None, dt)
        A, B = B, A
    q = A.particle_q.clone()
    qd = A.particle_qd.clone()
    x = q.clone()
    solver.predict(q, qd, dt)
    solver.update_system(x)
    solver.assemble(x, dt)
    solver.global_solve(0)
    torch.cuda.synchronize()
    T = mesh.T
    s_before = solver.tet_stretch.cpu().numpy().astype(np.float64)
    x_tilde = solver.read_buffer("x_tilde").cpu().numpy().reshape(-1, 3).astype(np.float64)
    dx = solver.read_buffer("dx").cpu().numpy().reshape(-1, 3).astype(np.float64)
    x_np = x.cpu().numpy().astype(np.float64)
    solver.local_solve(x)
    torch.cuda.synchronize()
    st = solver.line_search_stats()[0]
    lam = solver.tet_lambda.cpu().numpy()
    ds = solver.read_buffer("stretch_direction").cpu().numpy().reshape(6, T).T

    ref = O.OracleSolver(mesh, dtype=np.float64, line_search=True)
    ref.s = s_before.copy()
    el = ref.element_terms(x_np)
    lam_ref, ds_ref = ref.local_solve(el, dx)
    close(lam, lam_ref, 3e-4)
    close(ds, ds_ref, 3e-4)
    # the search itself, on the GPU's lambda and ds
    ref.lmbda = lam.astype(np.float64)
    x_ref, s_ref = ref.line_search_update(x_np, x_tilde, dt, el, dx, ds.astype(np.float64))
    r = ref.last_line_search[0]
    assert st["status"] == 0
    assert st["f0"] == pytest.approx(r.f0, rel=1e-5)
    assert st["t"] == pytest.approx(r.t, rel=1e-5)
    assert st["accepted"] == r.accepted and st["evaluations"] == r.evaluations and st["alpha"] == r.alpha
    # f1 is an fp32 sum over every tet of terms that partly cancel (Psi(s)
    # - lambda . c); it agrees to about 1e-5 of its value
    assert st["f1"] == pytest.approx(r.f1, rel=3e-5)
    close(x.cpu().numpy(), x_ref, 1e-6)
    close(solver.tet_stretch.cpu().numpy(), s_ref, 2e-6)


@pytest.mark.parametrize("name,cells,steps", [("cantilever", None, 100), ("nh_beam", (16, 4, 4), 5)])
def test_line_search_trajectory_matches_oracle(name, cells, steps):
    mesh, model, solver = make(name, cells)
    dt = mesh.spec.dt
    ref = O.OracleSolver(mesh, dtype=np.float64, line_search=True)
    A, B = model.state(), model.state()
    A.particle_q.copy_(torch.as_tensor(mesh.q0, device=DEV))
    q_ref, qd_ref = mesh.q0.astype(np.float64), mesh.qd0.astype(np.float64)
    for k in range(steps):
        solver.step(A, B, None, None, dt)
        A, B = B, A
        q_ref, qd_ref = ref.step(q_ref, qd_ref, dt)
        st = solver.line_search_stats()
        assert all(e["status"] == 0 for e in st)
        # the first Newton iteration takes the full step on both sides
        assert st[0]["accepted"] and st[0]["alpha"] == 1.0 and st[0]["evaluations"] == 1
        r0 = ref.last_line_search[0]
        assert r0.accepted and r0.alpha == 1.0 and r0.evaluations == 1
        assert st[0]["f0"] == pytest.approx(r0.f0, rel=1e-4)
        close(A.particle_q.cpu().numpy(), q_ref, 1e-5)


@pytest.mark.parametrize("pc", ["fsai", "learned"])
def test_line_search_with_factor_preconditioner(pc):
    mesh, model, solver = make("nh_beam", (16, 4, 4), preconditioner=pc)
    dt = mesh.spec.dt
    ref = O.OracleSolver(mesh, dtype=np.float64, line_search=True)
    A, B = model.state(), model.state()
    A.particle_q.copy_(torch.as_tensor(mesh.q0, device=DEV))
    q_ref, qd_ref = mesh.q0.astype(np.float64), mesh.qd0.astype(np.float64)
    for k in range(4):
        solver.step(A, B, None, None, dt)
        A, B = B, A
        q_ref, qd_ref = ref.step(q_ref, qd_ref, dt)
        assert all(e["status"] == 0 for e in solver.line_search_stats())
        assert all(s["status"] == 0 for s in solver.solve_stats())
        close(A.particle_q.cpu().numpy(), q_ref, 1e-5)


def test_iteration_cap_leaves_state_unchanged():
    """line_search_max_iterations=1: the counter after the first trial is
    already at the cap, so nothing is ever written and x stays at q_in."""
    mesh, model, solver = make("cantilever", iterations=3, line_search_max_iterations=1)
    A, B = model.state(), model.state()
    s0 = solver.tet_stretch.clone()
    solver.step(A, B, None, None, mesh.spec.dt)
    torch.cuda.synchronize()
    assert torch.equal(B.particle_q, A.particle_q)
    assert torch.count_nonzero(B.particle_qd) == 0
    assert torch.equal(solver.tet_stretch, s0)
    for e in solver.line_search_stats():
        assert not e["accepted"] and e["evaluations"] in (1, 2) and e["status"] == 0


def test_graph_and_eager_agree_bitwise():
    runs = []
    for graph in (True, False):
        mesh, model, solver = make("nh_beam", (16, 4, 4), use_cuda_graph=graph)
        A, B = model.state(), model.state()
        stats = []
        for _ in range(4):
            solver.step(A, B, None, None, mesh.spec.dt)
            A, B = B, A
            stats.append(solver.line_search_stats())
        runs.append((A.particle_q.clone(), solver.tet_stretch.clone(), stats))
    assert torch.equal(runs[0][0], runs[1][0])
    assert torch.equal(runs[0][1], runs[1][1])
    assert runs[0][2] == runs[1][2]


def test_plain_update_records_no_line_search():
    mesh, model, solver = make("cantilever", iterations=2, line_search=False)
    A, B = model.state(), model.state()
    solver.step(A, B, None, None, mesh.spec.dt)
    assert all(e["evaluations"] == 0 for e in solver.line_search_stats())
