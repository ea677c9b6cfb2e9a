"""The oracle's backtracking line search (src/mfem/line_search.py:76-163,
src/mfem/refinement/solver.py:803-928) on the CPU.

No reference test exercises the line search, so these tests pin the
restatement to the reference's source: the trial counter semantics of its
device loop on scripted merit values, the merit function against finite
differences, and the slope sign the reference uses.
"""
import numpy as np
import pytest

from mfem_gb300 import beams
from oracle import mfem_oracle as O


def _scripted(values):
    calls = []

    def f(alpha):
        calls.append(alpha)
        return values[len(calls) - 1]

    return f, calls


def test_first_trial_accepted():
    f, calls = _scripted([0.5])
    r = O.backtracking(f, 1.0, 0.1, 1.0, 0.5, 1e-8, 20)
    assert calls == [1.0] and r.accepted and r.alpha == 1.0 and r.evaluations == 1


def test_backtracks_until_sufficient_decrease():
    # f0 = 1, t = 1: trial j needs 1 - f1 + 1e-8 >= 0.5^j
    f, calls = _scripted([1.5, 1.2, 0.7])
    r = O.backtracking(f, 1.0, 1.0, 1.0, 0.5, 1e-8, 20)
    assert calls == [1.0, 0.5, 0.25]
    assert r.accepted and r.alpha == 0.25 and r.evaluations == 3


def test_counter_semantics_at_the_iteration_cap():
    # never a sufficient decrease: trials j = 0..max_iterations, nothing written
    f, calls = _scripted([2.0] * 10)
    r = O.backtracking(f, 1.0, 1.0, 1.0, 0.5, 1e-8, 3)
    assert calls == [1.0, 0.5, 0.25, 0.125] and r.evaluations == 4 and not r.accepted
    # a decrease found on the last counted trial (j = max_iterations - 1) is not written
    f, calls = _scripted([2.0, 2.0, 0.0])
    r = O.backtracking(f, 1.0, 1.0, 1.0, 0.5, 1e-8, 3)
    assert r.evaluations == 3 and not r.accepted
    # ... one trial earlier it is
    f, calls = _scripted([2.0, 0.0])
    r = O.backtracking(f, 1.0, 1.0, 1.0, 0.5, 1e-8, 3)
    assert r.evaluations == 2 and r.accepted and r.alpha == 0.5
    # max_iterations 0 and 1: one (or two) trials, never written
    for cap in (0, 1):
        f, _ = _scripted([0.0, 0.0])
        assert not O.backtracking(f, 1.0, 1.0, 1.0, 0.5, 1e-8, cap).accepted


def test_negative_slope_accepts_small_increases():
    # t < 0 (the reference's slope sign, late Newton iterations): an increase
    # below threshold + alpha |t| passes
    f, _ = _scripted([1.0 + 5e-9])
    assert O.backtracking(f, 1.0, -1e-9, 1.0, 0.5, 1e-8, 20).accepted
    r = O.backtracking(lambda alpha: 1.0 + 1e-7, 1.0, -1e-9, 1.0, 0.5, 1e-8, 20)
    assert r.evaluations == 21 and not r.accepted


def _mid_step(name, cells):
    """A beam after 3 plain steps, mid-way through one Newton iteration:
    element terms, PCG direction and local-solve lambda/ds."""
    mesh = beams.build_beam(name, cells=cells)
    S = O.OracleSolver(mesh, dtype=np.float64)
    q, qd = mesh.q0.astype(np.float64), mesh.qd0.astype(np.float64)
    for _ in range(3):
        q, qd = S.step(q, qd, mesh.spec.dt)
    dt = mesh.spec.dt
    x_tilde = S.predictor(q, qd, dt)
    x = q.copy()
    el = S.element_terms(x)
    blocks, g, _ = S.assemble(x, x_tilde, dt, el)
    Minv = O.block_jacobi_inverse(S.diag_blocks(blocks), S.singular_threshold)
    dx, _ = O.pcg(S.bsr_apply(blocks), g, x_tilde - x, Minv, 1e-10, 2000)
    lam, ds = S.local_solve(el, dx)
    S.lmbda = lam
    return S, x, x_tilde, dt, el, dx, ds


@pytest.fixture(scope="module")
def mid_step():
    return _mid_step("cantilever", None)


def test_merit_directional_derivative():
    """Neo-Hookean (whose energy value and g_s agree): d/da f(x + a dx, s + a
    ds) at 0 is (g_x + G^T lambda) . dx + (g_s + SYM lambda) . ds; the
    reference's slope uses g_x - G^T lambda instead."""
    S, x, x_tilde, dt, el, dx, ds = _mid_step("nh_beam", (8, 2, 2))
    s0 = S.s.copy()
    h = 1e-6
    fp = S.objective(x + h * dx, s0 + h * ds, x_tilde, dt)
    fm = S.objective(x - h * dx, s0 - h * ds, x_tilde, dt)
    fd = (fp - fm) / (2 * h)
    gx = S.kinetic_gradient(x, x_tilde, dt)
    GtL = np.zeros_like(x)
    contrib = np.einsum("tik,ti->tk", el["G"], S.lmbda).reshape(S.T, 4, 3)
    np.add.at(GtL, S.tets.ravel(), contrib.reshape(-1, 3))
    gs = el["g_s"] + O.SYM_DIAG * S.lmbda
    true_slope = np.sum((gx + GtL) * dx) + np.sum(gs * ds)
    ref_slope = np.sum((gx - GtL) * dx) + np.sum(gs * ds)
    assert abs(fd - true_slope) <= 1e-6 * abs(fd)
    assert abs(ref_slope - true_slope) > 0.1 * abs(true_slope)


def test_line_search_update_uses_reference_slope(mid_step):
    S, x, x_tilde, dt, el, dx, ds = mid_step
    s0 = S.s.copy()
    S.line_search = True
    S.last_line_search = []
    x1, s1 = S.line_search_update(x, x_tilde, dt, el, dx, ds)
    S.s = s0
    r = S.last_line_search[0]
    gx = S.kinetic_gradient(x, x_tilde, dt)
    GtL = np.zeros_like(x)
    contrib = np.einsum("tik,ti->tk", el["G"], S.lmbda).reshape(S.T, 4, 3)
    np.add.at(GtL, S.tets.ravel(), contrib.reshape(-1, 3))
    m = np.sum((gx - GtL) * dx) + np.sum((el["g_s"] + O.SYM_DIAG * S.lmbda) * ds)
    assert r.t == pytest.approx(-0.01 * m, rel=1e-12)
    assert r.f0 == pytest.approx(S.objective(x, s0, x_tilde, dt), rel=1e-12)
    if r.accepted:
        np.testing.assert_array_equal(x1, x + r.alpha * dx)
        np.testing.assert_array_equal(s1, s0 + r.alpha * ds)


def test_objective_attachment_form(mid_step):
    """k |x - p|^2 / 2 equals the reference's x.(Q x / 2 + b) + c with Q = k I,
    b = -k p, c = k p.p / 2 (boundary_condition.py:62-71)."""
    S, x, x_tilde, dt, el, dx, ds = mid_step
    k = S.hess_attach[:, None]
    p = S.pin_target
    ref = np.sum(x * (0.5 * k * x - k * p)) + 0.5 * np.sum(k * p * p)
    ours = np.sum(0.5 * S.hess_attach * np.sum((x - p) ** 2, axis=1))
    assert ours == pytest.approx(ref, rel=1e-9, abs=1e-12)


def test_oracle_step_with_line_search_stays_close_to_plain():
    """On the cantilever, the line search accepts the full Newton step in the
    first iteration of every step and the trajectory stays within 1e-4 of the
    plain one."""
    mesh = beams.build_beam("cantilever")
    A = O.OracleSolver(mesh, dtype=np.float64)
    B = O.OracleSolver(mesh, dtype=np.float64, line_search=True)
    qa, qda = mesh.q0.astype(np.float64), mesh.qd0.astype(np.float64)
    qb, qdb = qa.copy(), qda.copy()
    for _ in range(10):
        qa, qda = A.step(qa, qda, mesh.spec.dt)
        qb, qdb = B.step(qb, qdb, mesh.spec.dt)
        first = B.last_line_search[0]
        assert first.accepted and first.alpha == 1.0 and first.evaluations == 1
        assert len(B.last_line_search) == B.iterations
    assert np.abs(qa - qb).max() <= 1e-4 * np.abs(qa).max()
