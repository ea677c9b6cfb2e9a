"""CPU checks of the oracle's step-level behaviour and of the beam workloads.

The reference ships no test of the assembly, the PCG or a whole step, so
these check the oracle against the mathematics itself: the assembled matrix
equals the dense sum of element Hessians, the local solve satisfies the
linearised constraint, the PCG meets its stopping rule, float32 tracks
float64, and the committed trajectory is reproduced.
"""
import os

import numpy as np
import pytest

from mfem_gb300 import beams
from oracle import mfem_oracle as O


@pytest.mark.parametrize("name,T,n,nnzb", [
    ("cantilever", 240, 99, 951),
    ("nh_beam", 98_304, 18_785, 262_177),
])
def test_beam_sizes(name, T, n, nnzb):
    """Mesh sizes of the workloads: 6 tets per hex cell, exact sparsity."""
    m = beams.build_beam(name)
    assert (m.T, m.n) == (T, n)
    rp, ci = O.bsr_sparsity(m.tet_indices, m.n)
    assert ci.shape[0] == nnzb
    assert np.bincount(m.tet_indices.ravel()).max() == 24
    vol = 1.0 / (6.0 * np.linalg.det(m.tet_poses.astype(np.float64)))
    assert np.all(vol > 0)
    np.testing.assert_allclose(vol.sum(), np.prod(m.spec.extent), rtol=1e-6)


def test_beam_materials_and_pins():
    m = beams.build_beam("nh_beam")
    mu, lam = m.tet_materials[:, 0], m.tet_materials[:, 1]
    E = mu * 2 * (1 + 0.45)
    assert E.min() >= 1e4 * (1 - 1e-5) and E.max() <= 1e6 * (1 + 1e-5)
    np.testing.assert_allclose(lam / mu, 2 * 0.45 / (1 - 2 * 0.45), rtol=1e-5)
    pinned = m.particle_inv_mass == 0
    assert pinned.sum() == 17 * 17
    assert np.all(m.rest_q[pinned, 0] == 0)
    assert np.all(m.q0[pinned] == m.rest_q[pinned])
    free = ~pinned
    d = (m.q0 - m.rest_q)[free]
    assert 0.8e-3 < d.std() < 1.2e-3
    np.testing.assert_allclose(m.particle_mass.sum(), 1000.0 * 2.0 * 0.5 * 0.5, rtol=1e-5)


def test_slot_map_is_consistent():
    m = beams.build_beam("cantilever")
    rp, ci = O.bsr_sparsity(m.tet_indices, m.n)
    slots = O.tet_slot_map(m.tet_indices, rp, ci)
    for e in range(m.T):
        for k in range(4):
            for l in range(4):
                s = slots[e, 4 * k + l]
                r = m.tet_indices[e, k]
                assert rp[r] <= s < rp[r + 1]
                assert ci[s] == m.tet_indices[e, l]
    assert np.all(np.diff(ci[rp[5]:rp[6]]) > 0)


def _deformed_solver(energy):
    m = beams.build_beam("cantilever")
    S = O.OracleSolver(m, energy=energy, dtype=np.float64)
    rng = np.random.default_rng(7)
    x = m.q0.astype(np.float64) + rng.normal(0, 0.01, m.q0.shape)
    S.s = S.s + rng.normal(0, 0.02, S.s.shape)
    return m, S, x


@pytest.mark.parametrize("energy", ["arap", "neohookean"])
def test_assembly_equals_dense_sum(energy):
    m, S, x = _deformed_solver(energy)
    dt = m.spec.dt
    xt = x + 0.001
    el = S.element_terms(x)
    blocks, g, Hs = S.assemble(x, xt, dt, el)
    H = np.zeros((3 * m.n, 3 * m.n))
    for e in range(m.T):
        Ke = el["G"][e].T @ el["H_l"][e] @ el["G"][e]
        idx = (3 * m.tet_indices[e][:, None] + np.arange(3)).ravel()
        H[np.ix_(idx, idx)] += Ke
    diag = (S.hess_mass + S.hess_attach) / dt ** 2
    H += np.diag(np.repeat(diag, 3))
    np.testing.assert_allclose(Hs.toarray(), H, rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(H, H.T, atol=1e-9 * np.abs(H).max())
    assert np.linalg.eigvalsh(H).min() > 0
    # blocks in slot order reproduce H
    rp, ci = S.row_ptr, S.col_idx
    for r in range(0, m.n, 7):
        for k in range(rp[r], rp[r + 1]):
            c = ci[k]
            np.testing.assert_allclose(blocks[k], H[3 * r:3 * r + 3, 3 * c:3 * c + 3], atol=1e-9)


@pytest.mark.parametrize("energy", ["arap", "neohookean"])
def test_local_solve_satisfies_linearised_constraint(energy):
    """c - G dx - SYM ds = 0 and g_s + H_s ds + SYM lambda = 0 after the local
    solve (the Newton system behind src/mfem/refinement/kernels.py:252-283)."""
    m, S, x = _deformed_solver(energy)
    el = S.element_terms(x)
    dx = np.random.default_rng(3).normal(0, 1e-3, x.shape)
    lam, ds = S.local_solve(el, dx)
    dxe = dx[S.tets].reshape(m.T, 12)
    SYM = O.SYM_DIAG
    r1 = el["c"] - np.einsum("tij,tj->ti", el["G"], dxe) - SYM * ds
    r2 = el["g_s"] + np.einsum("tij,tj->ti", el["H_s"], ds) + SYM * lam
    assert np.abs(r1).max() < 1e-10
    assert np.abs(r2).max() < 1e-8 * max(1.0, np.abs(el["g_s"]).max())


def test_pcg_meets_stopping_rule():
    m, S, x = _deformed_solver("neohookean")
    el = S.element_terms(x)
    xt = x + 0.001
    blocks, g, Hs = S.assemble(x, xt, m.spec.dt, el)
    Minv = O.block_jacobi_inverse(S.diag_blocks(blocks), 1e-20)
    dx, res = O.pcg(S.bsr_apply(blocks), g, xt - x, Minv, 1e-6, 1000)
    assert res.converged
    true_r = np.linalg.norm(g.ravel() - Hs @ dx.ravel())
    assert true_r <= 1.01e-6 * np.linalg.norm(g)
    dx_direct = np.linalg.solve(Hs.toarray(), g.ravel())
    assert np.abs(dx.ravel() - dx_direct).max() < 1e-4 * np.abs(dx_direct).max()
    _, res1 = O.pcg(S.bsr_apply(blocks), g, xt - x, Minv, 1e-6, 1)
    assert res1.iterations == 1 and not res1.converged


def test_block_jacobi_singular_fallback():
    blocks = np.stack([np.eye(3) * 2.0, np.zeros((3, 3)), np.diag([1.0, 1e-30, 1.0])])
    inv = O.block_jacobi_inverse(blocks, 1e-20)
    np.testing.assert_allclose(inv[0], np.eye(3) / 2)
    np.testing.assert_array_equal(inv[1], np.eye(3))
    np.testing.assert_array_equal(inv[2], np.eye(3))


def test_float32_tracks_float64_and_golden_trajectory():
    """The oracle reproduces its committed float64 trajectory (first 10 steps),
    and float32 stays within 1e-6 relative of float64."""
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "cantilever_fp64.npz"))
    m = beams.build_beam("cantilever")
    A = O.OracleSolver(m, dtype=np.float64)
    B = O.OracleSolver(m, dtype=np.float32)
    qa, va, qb, vb = m.q0, m.qd0, m.q0, m.qd0
    for k in range(10):
        qa, va = A.step(qa, va, m.spec.dt)
        qb, vb = B.step(qb, vb, m.spec.dt)
        np.testing.assert_allclose(qa, gold["q"][k], rtol=0, atol=1e-12)
        assert [r.iterations for r in A.last_pcg] == list(gold["pcg_iterations"][k])
        assert np.abs(qb - qa).max() <= 1e-6 * np.abs(qa).max()


def test_initial_stretch_is_identity_at_rest():
    m = beams.build_beam("nh_beam", cells=(4, 2, 2))
    s = O.precompute_tet_stretch(m.rest_q.astype(np.float64), m.tet_indices, m.tet_poses.astype(np.float64))
    np.testing.assert_allclose(s, np.tile([1, 1, 1, 0, 0, 0], (m.T, 1)), atol=1e-6)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_bsr_apply_equals_dense_product(dtype):
    """The oracle's block-sparse product (warp.sparse.bsr_mv) against the
    dense matrix of the same blocks."""
    mesh = beams.build_beam("cantilever")
    S = O.OracleSolver(mesh, dtype=dtype)
    n, rp, ci = S.n, S.row_ptr, S.col_idx
    rng = np.random.default_rng(5)
    blocks = rng.standard_normal((ci.shape[0], 3, 3)).astype(dtype)
    v = rng.standard_normal((n, 3)).astype(dtype)
    D = np.zeros((3 * n, 3 * n))
    rows = np.repeat(np.arange(n), np.diff(rp))
    for k in range(ci.shape[0]):
        D[3 * rows[k]:3 * rows[k] + 3, 3 * ci[k]:3 * ci[k] + 3] = blocks[k]
    got = S.bsr_apply(blocks)(v)
    assert got.dtype == dtype and got.shape == (n, 3)
    tol = 1e-12 if dtype == np.float64 else 1e-5
    np.testing.assert_allclose(got.ravel(), D @ v.astype(np.float64).ravel(), rtol=tol, atol=tol * np.abs(D).max())
