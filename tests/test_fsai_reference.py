"""The float64 FSAI the GPU tests compare against (tests/test_gpu_fsai.py),
checked on CPU: on a small SPD block matrix with a tet-mesh pattern,
* G is lower block-triangular on the pattern and diag(G H G^T) = I;
* M = G^T G equals the textbook FSAI M (Kolotilina & Yeremin 1993: block
  row i = D X_i^T with X_i = H[P,P]^-1 E and D^T D = X_ii^-1 ... written
  here as C^-1 X^T with X_ii = C C^T), the two differing by a 3x3
  orthogonal factor per row."""
import numpy as np
import scipy.sparse as sp

from mfem_gb300 import beams
from fsai_reference import fsai_numpy, lower_pattern


def spd_system(seed=0):
    mesh = beams.build_beam("cantilever", cells=(4, 2, 2))
    t = mesh.tet_indices.astype(np.int64)
    n = mesh.n
    edges = {(int(a), int(b)) for tet in t for a in tet for b in tet}
    rows = sorted(edges)
    rp = np.zeros(n + 1, dtype=np.int64)
    for r, _ in rows:
        rp[r + 1] += 1
    rp = np.cumsum(rp)
    ci = np.array([c for _, c in rows])
    rng = np.random.default_rng(seed)
    B = rng.normal(size=(3 * n, 3 * n)) * 0.05
    # SPD with the block pattern: A = S + S^T masked, then shifted
    mask = np.zeros((3 * n, 3 * n), dtype=bool)
    for r, c in rows:
        mask[3 * r:3 * r + 3, 3 * c:3 * c + 3] = True
    A = np.where(mask, B + B.T, 0.0)
    A += (np.abs(A).sum(1).max() + 1.0) * np.eye(3 * n)
    vals = np.stack([A[3 * r:3 * r + 3, 3 * c:3 * c + 3] for r, c in rows])
    return n, rp, ci, vals, A


def textbook_fsai_M(n, rp, ci, A):
    lrow, lcol, _ = lower_pattern(rp, ci)
    G = np.zeros((3 * n, 3 * n))
    for i in range(n):
        P = lcol[lrow[i]:lrow[i + 1]]
        idx = np.concatenate([np.arange(3 * p, 3 * p + 3) for p in P])
        X = np.linalg.solve(A[np.ix_(idx, idx)], np.eye(len(idx))[:, -3:])
        C = np.linalg.cholesky(X[-3:])
        G[3 * i:3 * i + 3, idx] = np.linalg.solve(C, X.T)
    return G.T @ G


def test_fsai_reference_properties():
    n, rp, ci, vals, A = spd_system()
    Gb, fallback = fsai_numpy(rp, ci, vals)
    assert not fallback
    lrow, lcol, _ = lower_pattern(rp, ci)
    assert np.all(lcol <= np.repeat(np.arange(n), np.diff(lrow)))
    G = sp.bsr_matrix((Gb, lcol, lrow), shape=(3 * n, 3 * n)).toarray()
    D = G @ A @ G.T
    for i in range(n):
        np.testing.assert_allclose(D[3 * i:3 * i + 3, 3 * i:3 * i + 3], np.eye(3), atol=1e-10)
    np.testing.assert_allclose(G.T @ G, textbook_fsai_M(n, rp, ci, A), rtol=1e-9, atol=1e-12)
