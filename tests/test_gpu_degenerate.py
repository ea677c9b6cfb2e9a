"""Near-degenerate, flattened and inverted tets: the float64 polar path.

Tets with det F < 1e-3 take the polar decomposition F = U diag(sig) V^T and
the stretch derivative dS/dF in float64 (the element stage's second pass).
dS/dF carries 1 / max(sig_i + sig_j, 1e-8) (the reference's clamp,
src/mfem/refinement/utils.py:112-114), and float32 loses singular values
below about 2e-4 |F| in F^T F.  A soup of separate tets, each deformed by
F = R1 diag(sig) R2^T with chosen singular values (flattened, nearly
coplanar, inverted with the sign on the smallest singular value as the
reference's rotational_svd, utils.py:47-67, and ordinary tets in the same
warps), goes through the element stage.  On the tets with det F < 1e-3,
S (from c = SYM (S - s)), c and G must match the float64 oracle within 1e-6
of each tet's largest entry; the ordinary tets keep the float32 path and the
parity tests' 2e-5.  (On the host, the float32 path misses G by 1e-2 on the
tets collapsing towards a line; the float64 path is within 6e-8 on all.)
"""
import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver
from oracle import mfem_oracle as O

pytestmark = pytest.mark.gpu
DEV = "cuda:0"

SIGMAS = [
    (1.2, 0.9, 1.0e-4),      # flattened
    (1.0, 1.0, 3.0e-6),      # nearly coplanar
    (1.0, 0.8, 9.0e-4),      # just below the threshold
    (1.1, 0.8, -0.3),        # inverted
    (1.0, 0.5, -1.0e-3),     # inverted, nearly flat
    (0.9, 0.7, -0.05),       # inverted
    (1.0, 2.0e-3, 1.0e-4),   # collapsing towards a line
    (1.3, 1.1, 0.9),         # ordinary (float32 path)
    (0.8, 0.7, 0.6),         # ordinary
]


def random_rotation(rng):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    if np.linalg.det(q) < 0:
        q[:, 0] = -q[:, 0]
    return q


def degenerate_soup(reps=48, seed=21):
    """Separate tets (4 vertices each) at rest and deformed; every SIGMAS
    row `reps` times with random rotations, shuffled."""
    rng = np.random.default_rng(seed)
    base = 0.1 * np.array([[0.0, 0.0, 0.0], [1.0, 0.1, 0.0], [0.2, 1.0, 0.1], [0.1, 0.2, 1.0]])
    rows = [sig for sig in SIGMAS for _ in range(reps)]
    rng.shuffle(rows)
    rest, cur = [], []
    for k, sig in enumerate(rows):
        R0 = random_rotation(rng)
        X = base @ R0.T + rng.normal(0, 0.5, 3)
        F = random_rotation(rng) @ np.diag(sig) @ random_rotation(rng).T
        rest.append(X)
        cur.append((X - X[0]) @ F.T + X[0] + rng.normal(0, 0.1, 3))
    rest = np.concatenate(rest).astype(np.float32)
    cur = np.concatenate(cur).astype(np.float32)
    tets = np.arange(4 * len(rows), dtype=np.int32).reshape(-1, 4)
    xe = rest[tets].astype(np.float64)
    Dm = np.linalg.inv(np.stack([xe[:, 1] - xe[:, 0], xe[:, 2] - xe[:, 0], xe[:, 3] - xe[:, 0]], axis=-1))
    return rest, cur, tets, Dm.astype(np.float32), np.array(rows)


def per_tet_close(a, b, rtol, what):
    a = a.reshape(len(a), -1).astype(np.float64)
    b = b.reshape(len(b), -1).astype(np.float64)
    scale = np.maximum(np.abs(b).max(axis=1), 1e-30)
    err = np.abs(a - b).max(axis=1) / scale
    worst = int(np.argmax(err))
    assert err[worst] <= rtol, f"{what}: tet {worst} relative error {err[worst]:.3e}"
    return float(err.max())


def test_degenerate_tets_match_fp64_oracle():
    rest, cur, tets, Dm, rows = degenerate_soup()
    n, T = len(rest), len(tets)
    mats = np.tile(np.array([[3.5e4, 1.4e5, 0.0]], np.float32), (T, 1))
    model = Model(rest, np.zeros_like(rest), np.ones(n, np.float32), np.ones(n, np.float32), tets, Dm, mats,
                  np.zeros(3, np.float32), device=DEV)
    solver = MixedFEMSolver(model, iterations=1, energy="neohookean", line_search=False)
    s = solver.tet_stretch.cpu().numpy().reshape(T, 6)
    solver.update_system(torch.as_tensor(cur, device=DEV))
    torch.cuda.synchronize()
    c = solver.read_buffer("constraint").cpu().numpy().reshape(6, T).T
    G = np.transpose(solver.read_buffer("grad_constraint").cpu().numpy().reshape(6, 12, T), (2, 0, 1))
    c_ref, G_ref = O.compute_constraints(cur.astype(np.float64), tets, Dm.astype(np.float64), s.astype(np.float64))
    sym = O.SYM_DIAG
    S = c / sym + s
    S_ref = c_ref / sym + s
    F = O.deformation_gradient(cur.astype(np.float64), tets, Dm.astype(np.float64))
    detF = np.linalg.det(F)
    deg = detF < 1e-3
    assert deg.sum() >= 6 * 48 and (detF < 0).sum() >= 3 * 48  # the cases reach the fp64 path
    per_tet_close(S[deg], S_ref[deg], 1e-6, "S (det F < 1e-3)")
    per_tet_close(c[deg], c_ref[deg], 1e-6, "c (det F < 1e-3)")
    g_err = per_tet_close(G[deg], G_ref[deg], 1e-6, "G (det F < 1e-3)")
    per_tet_close(S[~deg], S_ref[~deg], 2e-5, "S")
    per_tet_close(G[~deg], G_ref[~deg], 2e-5, "G")
    print(f"worst relative G error {g_err:.2e} over {deg.sum()} tets below det 1e-3")


def test_degenerate_tets_step_is_finite():
    """A step of the soup with its degenerate tets: finite positions and
    every PCG outcome reported (no breakdown into non-finite values)."""
    rest, cur, tets, Dm, _ = degenerate_soup(reps=8, seed=5)
    n, T = len(rest), len(tets)
    mats = np.tile(np.array([[3.5e4, 1.4e5, 0.0]], np.float32), (T, 1))
    model = Model(rest, np.zeros_like(rest), np.full(n, 0.05, np.float32), np.full(n, 20.0, np.float32), tets,
                  Dm, mats, np.array([0.0, -9.81, 0.0], np.float32), device=DEV)
    solver = MixedFEMSolver(model, iterations=4, energy="neohookean", line_search=False)
    s0, s1 = model.state(), model.state()
    s0.particle_q.copy_(torch.as_tensor(cur, device=DEV))
    solver.step(s0, s1, None, None, 1.0 / 60.0)
    q = s1.particle_q.cpu().numpy()
    assert np.isfinite(q).all()
    assert all(st["status"] in (0, 1) for st in solver.solve_stats())
