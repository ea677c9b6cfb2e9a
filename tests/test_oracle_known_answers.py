"""Pins the CPU oracle to the reference's own known-answer tests.

Each test restates one reference test (file:line cited) with the same inputs
and the same assertion, run on the oracle instead of Warp, plus a tighter
float64 check where the reference's tolerance was set for float32 finite
differences.  The inputs come from tests/golden/known_answers.npz, rebuilt by
tests/golden/make_golden.py from the seeds and literals of those tests.
"""
import os

import numpy as np
import pytest

from oracle import mfem_oracle as O

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "known_answers.npz"))


def test_golden_file_matches_its_generator():
    from tests.golden import make_golden
    fresh = make_golden.known_answers()
    for k, v in fresh.items():
        np.testing.assert_array_equal(GOLDEN[k], v, err_msg=k)


def test_constraint_is_rotation_invariant():
    """tests/test_kernels.py:59-99 -- a rest tet rotated 12 deg about z with
    s = (1,1,1,0,0,0) has constraint 0 (abs 1e-5), in float32."""
    pos = GOLDEN["rot_pos"].astype(np.float32)
    dminv = GOLDEN["rot_dminv"].astype(np.float32)
    s = np.array([[1.0, 1.0, 1.0, 0.0, 0.0, 0.0]], dtype=np.float32)
    c, _ = O.compute_constraints(pos, np.array([[0, 1, 2, 3]]), dminv, s)
    assert c.dtype == np.float32
    np.testing.assert_allclose(c, 0.0, atol=1e-5)


def _fd_jacobian(fun, x0, h):
    x0 = np.asarray(x0, dtype=np.float64)
    f0 = fun(x0)
    J = np.zeros((f0.size, x0.size))
    for i in range(x0.size):
        xp = x0.copy().ravel()
        xm = x0.copy().ravel()
        xp[i] += h
        xm[i] -= h
        J[:, i] = (fun(xp.reshape(x0.shape)).ravel() - fun(xm.reshape(x0.shape)).ravel()) / (2 * h)
    return J


def _dense_legacy_gradient(G, tets, n):
    """The legacy evaluate_constraint_gradient_dx BSR (+SYM dS/dx, the
    negative of the refinement kernel's G) densified like tests/utils.py:441-466."""
    T = tets.shape[0]
    D = np.zeros((6 * T, 3 * n))
    for t in range(T):
        for k in range(4):
            D[6 * t:6 * t + 6, 3 * tets[t, k]:3 * tets[t, k] + 3] += -G[t][:, 3 * k:3 * k + 3]
    return D


@pytest.mark.parametrize("kind,tol", [("tet", 5e-2), ("cube", 1e-2)])
@pytest.mark.parametrize("i", range(5))
def test_constraint_gradient_matches_finite_differences(kind, tol, i):
    """tests/test_kernels.py:139-218 (single tet, abs 5e-2) and 221-298
    (unit-cube Delaunay tets, abs 1e-2): dc/dx against finite differences,
    for I and four I + 0.3 N(0,1) deformations (default_rng(42))."""
    pos = GOLDEN[f"{kind}{i}_pos"]
    tets = GOLDEN[f"{kind}{i}_tets"]
    dminv = GOLDEN[f"{kind}{i}_dminv"]
    s = GOLDEN[f"{kind}{i}_s"]
    n = pos.shape[0]
    _, G = O.compute_constraints(pos, tets, dminv, s)
    np.testing.assert_allclose(G, GOLDEN[f"{kind}{i}_G"], rtol=1e-12, atol=1e-12)
    analytic = _dense_legacy_gradient(G, tets, n)

    def c_of(x):
        c, _ = O.compute_constraints(x.reshape(n, 3), tets, dminv, s)
        return c.ravel()

    fd = _fd_jacobian(c_of, pos, 1e-6)
    assert analytic == pytest.approx(fd, abs=tol)          # the reference's bar
    np.testing.assert_allclose(analytic, fd, atol=1e-6)    # float64 central differences


@pytest.mark.parametrize("i", range(5))
def test_stretch_gradient_matches_finite_differences(i):
    """tests/test_functions.py:112-149: the 6x9 stretch gradient against
    finite differences of sym6(S(F)) by the row-major entries of F (abs 2e-2)."""
    pos = GOLDEN[f"tet{i}_pos"]
    dminv = GOLDEN[f"tet{i}_dminv"]
    F = O.deformation_gradient(pos, np.array([[0, 1, 2, 3]]), dminv)
    U, sig, V = O.rotational_svd(F)
    J = O.stretch_gradient(F, U, sig, V)[0]

    def s_of(f):
        Fm = f.reshape(1, 3, 3)
        U_, s_, V_ = O.rotational_svd(Fm)
        return O.mat33_to_sym6(O.stretch_component(U_, s_, V_)).ravel()

    fd = _fd_jacobian(s_of, F[0], 1e-6)
    assert J.shape == (6, 9)
    assert J == pytest.approx(fd, abs=2e-2)
    np.testing.assert_allclose(J, fd, atol=1e-6)


def _psd(name):
    A = GOLDEN[name].astype(np.float32)
    fixed, inv = O.psd_fix(A[None])
    return A, fixed[0], inv[0]


@pytest.mark.parametrize("name,dim", [("A3_pd", 3), ("A6_pd", 6)])
def test_psd_fix_keeps_pd_input(name, dim):
    """tests/numerical/test_psd_fix.py:257-263, 281-287."""
    A, mat, inv = _psd(name)
    np.testing.assert_allclose(mat, A, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(mat @ inv, np.eye(dim), atol=2e-5)


@pytest.mark.parametrize("name,dim", [("A3_non_pd", 3), ("A6_non_pd", 6)])
def test_psd_fix_repairs_indefinite_input(name, dim):
    """tests/numerical/test_psd_fix.py:265-277, 289-301."""
    A, mat, inv = _psd(name)
    assert np.all(np.linalg.eigvalsh(mat) > 0)
    np.testing.assert_allclose(mat, mat.T, atol=1e-6)
    np.testing.assert_allclose(inv, inv.T, atol=1e-6)
    np.testing.assert_allclose(mat @ inv, np.eye(dim), atol=1e-4)
    f64, i64 = GOLDEN[name + "_fixed"], GOLDEN[name + "_inv"]
    np.testing.assert_allclose(mat, f64, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(inv, i64, rtol=1e-4, atol=1e-4)
