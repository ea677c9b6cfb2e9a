"""CPU oracle for warp-mfem's global step -- TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.

It restates, in batched numpy (float64 or float32), the reference's
``RefinementSolver.step`` with refinement, contact and shell off, with the
line search on or off:

=========================================  =====================================================
stage                                      reference (warp-mfem, paths within the project)
=========================================  =====================================================
rotation-variant SVD, polar stretch        src/mfem/refinement/utils.py:46-72
dR/dF, dS/dF, dF/dx                        src/mfem/refinement/utils.py:75-177
constraint c and Jacobian G                src/mfem/refinement/kernels.py:131-169
ARAP energy / gradient / Hessian in s      src/mfem/refinement/elastic_energy.py:106-197
Neo-Hookean energy / gradient / Hessian    src/mfem/refinement/elastic_energy.py:255-346
det / grad / Hessian of det on sym6        src/mfem/utils.py:56-97
GMW81 modified Cholesky, PSD fix           src/mfem/numerical/gmw81.py:18-86, psd_fix.py:105-191
H_lambda, g_lambda, H_lambda G             src/mfem/refinement/kernels.py:188-249
mass / attachment / kinetic gradient       src/mfem/refinement/kernels.py:7-30, 172-185;
                                           src/mfem/boundary_condition.py:10-83;
                                           src/mfem/refinement/solver.py:320-393, 930-947
predictor x~                               src/mfem/refinement/kernels.py:77-91
assembly H = sum G^T H_l G + (M+Q)/dt^2,   src/mfem/refinement/solver.py:641-743
         g = sum G^T H_l g_l - g_x
block-Jacobi preconditioner                src/mfem/refinement/kernels.py:32-53; solver.py:581-609
PCG (warm start dx = x~ - x)               src/mfem/refinement/solver.py:220-235, 529-532
local solve for lambda and ds              src/mfem/refinement/kernels.py:252-283
update and velocity                        src/mfem/refinement/solver.py:555-577; kernels.py:351-363
line search (merit function, Armijo)       src/mfem/line_search.py:76-163; refinement/solver.py:803-928;
                                           kernels.py:285-348; elastic_energy.py:155-176, 287-311;
                                           boundary_condition.py:62-71
initial stretch s = S(F_rest), lambda = 0  src/mfem/refinement/additional_state.py:146-189
=========================================  =====================================================

Third-party arithmetic that the reference takes from warp-lang 1.15.0 (not part
of the reference tree) is restated from its published definition:

* ``wp.svd3`` -> ``numpy.linalg.svd`` (singular values descending) followed by
  the reference's own reflection fix, which puts the sign on the smallest one.
* ``warp.optim.linear.cg`` with a block-Jacobi ``M`` -> textbook preconditioned
  CG, stopped when ``||r||_2 <= tol * ||b||_2`` (checked before every
  iteration, so a warm start that already satisfies it costs no iteration).
  Warp's exact stopping test is not pinned by any reference test.
* ``warp.sparse`` assembly -> exact vertex-adjacency CSR with ascending
  columns; the sum of the element blocks is exact in float64.

Pinning: the element math is checked against the reference's own known-answer
tests (rotation invariance of c, finite-difference Jacobians of c and of the
stretch, the PSD-fix matrices: tests/test_kernels.py, tests/test_functions.py,
tests/numerical/test_psd_fix.py).  The reference ships no test of the
assembly, the PCG or a whole step and cannot be run here (warp-lang / newton are
absent), so at step level the oracle's parity with the reference is UNPINNED:
it follows the reference's code line by line, nothing more.  The same holds
for the line search, which no reference test exercises.  It keeps the
reference's slope sign: the x-gradient is g_x - G^T lambda with G = dC_dX =
-dc/dx (kernels.py:159, solver.py:905), which is not the merit function's
x-gradient g_x + G^T lambda.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SYM_DIAG = np.array([1.0, 1.0, 1.0, 2.0, 2.0, 2.0])
INV_SYM_DIAG = np.array([1.0, 1.0, 1.0, 0.5, 0.5, 0.5])
_E6 = np.array([1.0, 1.0, 1.0, 0.0, 0.0, 0.0])

# ---------------------------------------------------------------------------
# sym6 helpers: order (xx, yy, zz, xy, xz, yz)  (src/mfem/refinement/utils.py:7-20)
# ---------------------------------------------------------------------------


def sym6_to_mat33(s):
    s = np.asarray(s)
    M = np.empty(s.shape[:-1] + (3, 3), dtype=s.dtype)
    M[..., 0, 0] = s[..., 0]
    M[..., 1, 1] = s[..., 1]
    M[..., 2, 2] = s[..., 2]
    M[..., 0, 1] = M[..., 1, 0] = s[..., 3]
    M[..., 0, 2] = M[..., 2, 0] = s[..., 4]
    M[..., 1, 2] = M[..., 2, 1] = s[..., 5]
    return M


def mat33_to_sym6(M):
    return np.stack([M[..., 0, 0], M[..., 1, 1], M[..., 2, 2],
                     M[..., 0, 1], M[..., 0, 2], M[..., 1, 2]], axis=-1)


def flatten_cols(M):
    """vec9 of the columns of M (src/mfem/refinement/utils.py:22-28)."""
    return np.swapaxes(M, -1, -2).reshape(M.shape[:-2] + (9,))


def unflatten_cols(v):
    """matrix_from_cols(v[0:3], v[3:6], v[6:9]) (src/mfem/refinement/utils.py:30-32)."""
    return np.swapaxes(v.reshape(v.shape[:-1] + (3, 3)), -1, -2)


# ---------------------------------------------------------------------------
# Polar decomposition and its derivatives
# ---------------------------------------------------------------------------


def rotational_svd(F):
    """U, sigma, V with the reference's reflection fix
    (src/mfem/refinement/utils.py:46-67): sign of det(U) det(V) moves onto
    sigma[2] (the smallest singular value) and the matching column of U or V."""
    U, sig, Vt = np.linalg.svd(F)
    V = np.swapaxes(Vt, -1, -2).copy()
    U = U.copy()
    sig = sig.copy()
    det_u = np.linalg.det(U)
    det_v = np.linalg.det(V)
    flipped = (det_u * det_v).astype(F.dtype)
    sig[..., 2] *= flipped
    mu_ = (det_u < 0) & (det_v >= 0)
    mv_ = (det_v < 0) & (det_u >= 0)
    U[mu_, :, 2] *= flipped[mu_, None]
    V[mv_, :, 2] *= flipped[mv_, None]
    return U, sig, V


def stretch_component(U, sig, V):
    """S = V diag(sigma) V^T (src/mfem/refinement/utils.py:70-72)."""
    return np.einsum("...ik,...k,...jk->...ij", V, sig, V)


_TWISTS = np.array([
    [[0.0, -1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 0.0]],   # about z
    [[0.0, 0.0, 0.0], [0.0, 0.0, 1.0], [0.0, -1.0, 0.0]],   # about x
    [[0.0, 0.0, 1.0], [0.0, 0.0, 0.0], [-1.0, 0.0, 0.0]],   # about y
])


def rotation_gradient(U, sig, V):
    """9x9 dR/dF (column-major vec9 on both sides), src/mfem/refinement/utils.py:93-121."""
    dt = U.dtype
    Tw = _TWISTS.astype(dt)
    inv_sqrt2 = dt.type(1.0) / np.sqrt(dt.type(2.0))
    t = [flatten_cols(inv_sqrt2 * (U @ Tw[k] @ np.swapaxes(V, -1, -2))) for k in range(3)]
    s0, s1, s2 = sig[..., 0], sig[..., 1], sig[..., 2]
    floor = dt.type(1.0e-8)
    s01 = np.maximum(s0 + s1, floor)
    s12 = np.maximum(s1 + s2, floor)
    s02 = np.maximum(s0 + s2, floor)
    two = dt.type(2.0)
    return ((two / s01)[..., None, None] * np.einsum("...i,...j->...ij", t[0], t[0])
            + (two / s12)[..., None, None] * np.einsum("...i,...j->...ij", t[1], t[1])
            + (two / s02)[..., None, None] * np.einsum("...i,...j->...ij", t[2], t[2]))


def stretch_gradient(F, U, sig, V):
    """6x9 dS/dF; column i*3+j is F[i, j] (row-major), src/mfem/refinement/utils.py:75-90."""
    dR = rotation_gradient(U, sig, V)
    R = U @ np.swapaxes(V, -1, -2)
    FT = np.swapaxes(F, -1, -2)
    grad = np.zeros(F.shape[:-2] + (6, 9), dtype=F.dtype)
    for i in range(3):
        for j in range(3):
            M = FT @ unflatten_cols(dR[..., :, j * 3 + i])
            M[..., j, :] += R[..., i, :]
            grad[..., :, i * 3 + j] = mat33_to_sym6(M)
    return grad


def dF_dx(DmInv):
    """9x12 dF/dx; row i*3+j is F[i, j], column 3k+a is vertex k component a
    (src/mfem/refinement/utils.py:123-177)."""
    B = np.concatenate([-DmInv.sum(axis=-2, keepdims=True), DmInv], axis=-2)  # [.., 4, 3]
    D = np.zeros(DmInv.shape[:-2] + (9, 12), dtype=DmInv.dtype)
    for i in range(3):
        for j in range(3):
            for k in range(4):
                D[..., i * 3 + j, 3 * k + i] = B[..., k, j]
    return D


def deformation_gradient(x, tets, DmInv):
    """F = [x1-x0, x2-x0, x3-x0] (columns) * DmInv (src/mfem/refinement/kernels.py:145-156)."""
    xe = x[tets]
    Ds = np.stack([xe[:, 1] - xe[:, 0], xe[:, 2] - xe[:, 0], xe[:, 3] - xe[:, 0]], axis=-1)
    return Ds @ DmInv


def compute_constraints(x, tets, DmInv, s):
    """c = SYM (sym6(S(F)) - s) and G = -(SYM dS/dF dF/dx) as a [T, 6, 12]
    matrix whose 6x3 column blocks are the reference's mat63 blocks
    (src/mfem/refinement/kernels.py:131-169)."""
    dt = x.dtype
    F = deformation_gradient(x, tets, DmInv)
    U, sig, V = rotational_svd(F)
    sF = mat33_to_sym6(stretch_component(U, sig, V))
    J = stretch_gradient(F, U, sig, V)
    D = dF_dx(DmInv)
    SYM = SYM_DIAG.astype(dt)
    G = -(SYM[:, None] * (J @ D))
    c = SYM * (sF - s)
    return c, G


def precompute_tet_stretch(x, tets, DmInv):
    """Initial s = sym6(S(F)) (src/mfem/refinement/kernels.py:55-75)."""
    F = deformation_gradient(x, tets, DmInv)
    U, sig, V = rotational_svd(F)
    return mat33_to_sym6(stretch_component(U, sig, V))


# ---------------------------------------------------------------------------
# Energies in stretch space
# ---------------------------------------------------------------------------


def rest_volume(DmInv):
    """vol = 1 / (6 det DmInv) (src/mfem/refinement/elastic_energy.py:143-145)."""
    return 1.0 / (6.0 * np.linalg.det(DmInv))


def det_sym6(s):
    return (s[..., 0] * s[..., 1] * s[..., 2] + 2.0 * s[..., 3] * s[..., 4] * s[..., 5]) - (
        s[..., 1] * s[..., 4] * s[..., 4] + s[..., 0] * s[..., 5] * s[..., 5]
        + s[..., 2] * s[..., 3] * s[..., 3])


def grad_det_sym6(s):
    return np.stack([
        s[..., 1] * s[..., 2] - s[..., 5] * s[..., 5],
        s[..., 0] * s[..., 2] - s[..., 4] * s[..., 4],
        s[..., 0] * s[..., 1] - s[..., 3] * s[..., 3],
        2.0 * (s[..., 4] * s[..., 5] - s[..., 2] * s[..., 3]),
        2.0 * (s[..., 3] * s[..., 5] - s[..., 1] * s[..., 4]),
        2.0 * (s[..., 3] * s[..., 4] - s[..., 0] * s[..., 5]),
    ], axis=-1)


def hess_det_sym6(s):
    """src/mfem/utils.py:85-97 (row-major 6x6)."""
    z = np.zeros_like(s[..., 0])
    s0, s1, s2, s3, s4, s5 = (s[..., i] for i in range(6))
    rows = [
        [z, s2, s1, z, z, -2.0 * s5],
        [s2, z, s0, z, -2.0 * s4, z],
        [s1, s0, z, -2.0 * s3, z, z],
        [z, z, -2.0 * s3, -2.0 * s2, 2.0 * s5, 2.0 * s4],
        [z, -2.0 * s4, z, 2.0 * s5, -2.0 * s1, 2.0 * s3],
        [-2.0 * s5, z, z, 2.0 * s4, 2.0 * s3, -2.0 * s0],
    ]
    return np.stack([np.stack(r, axis=-1) for r in rows], axis=-2)


def arap_energy(s, materials, DmInv):
    """Energy, gradient, Hessian and inverse Hessian in s for ARAP
    (src/mfem/refinement/elastic_energy.py:106-197).  The energy keeps the
    reference's second invariant s0s1+s1s2+s2s0+2(...) (lines 110-112); only
    the line search reads it."""
    dt = s.dtype
    mu = materials[:, 0]
    vol = rest_volume(DmInv)
    I1 = s[:, 0] + s[:, 1] + s[:, 2]
    I2 = s[:, 0] * s[:, 1] + s[:, 1] * s[:, 2] + s[:, 2] * s[:, 0] + 2.0 * (
        s[:, 3] ** 2 + s[:, 4] ** 2 + s[:, 5] ** 2)
    SYM = SYM_DIAG.astype(dt)
    energy = vol * (mu * (I2 + 3.0 - 2.0 * I1) / 2.0)
    grad = vol[:, None] * (mu[:, None] * (2.0 * SYM * s - 2.0 * _E6.astype(dt)) / 2.0)
    H = (mu * vol)[:, None, None] * np.diag(SYM)
    Hinv = (1.0 / (mu * vol))[:, None, None] * np.diag(INV_SYM_DIAG.astype(dt))
    return energy, grad, H, Hinv


def neohookean_energy(s, materials, DmInv):
    """src/mfem/refinement/elastic_energy.py:255-346: energy and gradient, and
    the Hessian vol (mu SYM + lam gJ gJ^T + (lam (J-1) - mu) hJ) made positive
    definite by psd_fix_6."""
    dt = s.dtype
    mu = materials[:, 0]
    lam = materials[:, 1]
    vol = rest_volume(DmInv)
    SYM = SYM_DIAG.astype(dt)
    I2 = s[:, 0] ** 2 + s[:, 1] ** 2 + s[:, 2] ** 2 + 2.0 * (s[:, 3] ** 2 + s[:, 4] ** 2 + s[:, 5] ** 2)
    J = det_sym6(s)
    gJ = grad_det_sym6(s)
    hJ = hess_det_sym6(s)
    energy = vol * (mu * (I2 - 3.0) / 2.0 - mu * (J - 1.0) + lam / 2.0 * (J - 1.0) * (J - 1.0))
    grad = vol[:, None] * (mu[:, None] * SYM * s + (lam * (J - 1.0) - mu)[:, None] * gJ)
    hess = vol[:, None, None] * (
        mu[:, None, None] * np.diag(SYM)
        + lam[:, None, None] * np.einsum("ti,tj->tij", gJ, gJ)
        + (lam * (J - 1.0) - mu)[:, None, None] * hJ)
    H, Hinv = psd_fix(hess)
    return energy, grad, H, Hinv


# ---------------------------------------------------------------------------
# GMW81 modified Cholesky and the PSD fix (src/mfem/numerical/gmw81.py:18-86,
# src/mfem/numerical/psd_fix.py:105-191).  The constants are the reference's
# float32 ones in every precision.
# ---------------------------------------------------------------------------


def gmw81(A):
    A = np.array(A, copy=True)
    dt = A.dtype
    dim = A.shape[-1]
    eps = dt.type(1.19e-7)
    delta = np.sqrt(eps)
    gamma = np.zeros(A.shape[:-2], dtype=dt)
    xi = np.zeros(A.shape[:-2], dtype=dt)
    for i in range(dim):
        gamma = np.maximum(gamma, np.abs(A[..., i, i]))
        for j in range(i + 1, dim):
            xi = np.maximum(xi, np.abs(A[..., i, j]))
    beta2 = np.maximum(gamma, np.maximum(xi / np.sqrt(dt.type(dim * dim - 1)), eps))
    for j in range(dim):
        for i in range(j + 1, dim):
            c_ij = A[..., j, i].copy()
            for k in range(j):
                c_ij = c_ij - A[..., k, k] * A[..., k, k] * A[..., i, k] * A[..., j, k]
            A[..., i, j] = c_ij
        theta = np.zeros(A.shape[:-2], dtype=dt)
        for i in range(j + 1, dim):
            theta = np.maximum(theta, np.abs(A[..., i, j]))
        c_jj = A[..., j, j]
        d_j = np.maximum(delta, np.maximum(np.abs(c_jj), theta * theta / beta2))
        A[..., j, j] = np.sqrt(d_j)
        for i in range(j + 1, dim):
            c_ij = A[..., i, j].copy()
            A[..., i, j] = c_ij / d_j
            A[..., i, i] = A[..., i, i] - c_ij * c_ij / d_j
    for j in range(dim):
        sqrt_dj = A[..., j, j].copy()
        for i in range(j + 1, dim):
            A[..., i, j] = A[..., i, j] * sqrt_dj
        for i in range(j):
            A[..., i, j] = 0.0
    return A


def _psd_fix_from_L(L):
    L = np.array(L, copy=True)
    dim = L.shape[-1]
    fixed = np.zeros_like(L)
    for i in range(dim):
        for j in range(i + 1):
            acc = np.zeros(L.shape[:-2], dtype=L.dtype)
            for k in range(j + 1):
                acc = acc + L[..., i, k] * L[..., j, k]
            fixed[..., i, j] = acc
            fixed[..., j, i] = acc
    for k in range(dim):
        L[..., k, k] = 1.0 / L[..., k, k]
        for i in range(k + 1, dim):
            acc = np.zeros(L.shape[:-2], dtype=L.dtype)
            for j in range(k, i):
                acc = acc + L[..., i, j] * L[..., j, k]
            L[..., i, k] = -acc / L[..., i, i]
    inv = np.zeros_like(L)
    for i in range(dim):
        for j in range(i + 1):
            acc = np.zeros(L.shape[:-2], dtype=L.dtype)
            for k in range(i, dim):
                acc = acc + L[..., k, i] * L[..., k, j]
            inv[..., i, j] = acc
            inv[..., j, i] = acc
    return fixed, inv


def psd_fix(A):
    """(A + E, (A + E)^-1) for symmetric A (any trailing dim)."""
    return _psd_fix_from_L(gmw81(A))


# ---------------------------------------------------------------------------
# Sparsity and element -> slot maps (the symbolic half of the assembly)
# ---------------------------------------------------------------------------


def bsr_sparsity(tets, n):
    """Exact vertex-adjacency sparsity of H (diagonal included), columns
    ascending: returns (row_ptr [n+1], col_idx [nnzb]) as int32."""
    tets = np.asarray(tets, dtype=np.int64)
    rows = np.repeat(tets, 4, axis=1).ravel()
    cols = np.tile(tets, (1, 4)).ravel()
    keys = np.unique(np.concatenate([rows * n + cols, np.arange(n, dtype=np.int64) * (n + 1)]))
    r = keys // n
    c = keys % n
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(row_ptr, r + 1, 1)
    return np.cumsum(row_ptr).astype(np.int32), c.astype(np.int32)


def tet_slot_map(tets, row_ptr, col_idx):
    """[T, 16] int32: slot of block (tets[e, k], tets[e, l]) at index k*4+l."""
    tets = np.asarray(tets, dtype=np.int64)
    T = tets.shape[0]
    out = np.empty((T, 16), dtype=np.int32)
    for k in range(4):
        for l in range(4):
            r = tets[:, k]
            c = tets[:, l]
            pos = _vectorised_slot(row_ptr, col_idx, r, c)
            assert np.all(col_idx[pos] == c)
            out[:, k * 4 + l] = pos
    return out


def _vectorised_slot(row_ptr, col_idx, r, c):
    n = row_ptr.shape[0] - 1
    key_all = np.repeat(np.arange(n, dtype=np.int64), np.diff(row_ptr)) * n + col_idx.astype(np.int64)
    return np.searchsorted(key_all, r * n + c)


# ---------------------------------------------------------------------------
# The step
# ---------------------------------------------------------------------------


@dataclass
class PCGResult:
    iterations: int
    residual_norm: float
    rhs_norm: float
    converged: bool


def block_jacobi_inverse(diag_blocks, singular_threshold):
    """Inverse of every 3x3 diagonal block, identity where |det| < threshold
    (src/mfem/refinement/kernels.py:32-53)."""
    det = np.linalg.det(diag_blocks)
    out = np.broadcast_to(np.eye(3, dtype=diag_blocks.dtype), diag_blocks.shape).copy()
    ok = np.abs(det) >= singular_threshold
    out[ok] = np.linalg.inv(diag_blocks[ok])
    return out


def pcg(apply_A, b, x0, Minv_blocks, tol, maxiter):
    """Block-Jacobi PCG on [n, 3] vectors; stops when ||r|| <= tol ||b||."""
    import scipy.sparse as sp
    dt = b.dtype
    n = Minv_blocks.shape[0]
    M = sp.bsr_matrix((Minv_blocks, np.arange(n), np.arange(n + 1)), shape=(3 * n, 3 * n))

    def precond(v):
        return (M @ v.reshape(-1)).reshape(n, 3)
    x = x0.copy()
    r = b - apply_A(x)
    z = precond(r)
    p = z.copy()
    rz = np.sum(r * z, dtype=dt)
    b_norm = math.sqrt(float(np.sum(b * b, dtype=dt)))
    target = tol * b_norm
    it = 0
    r_norm = math.sqrt(float(np.sum(r * r, dtype=dt)))
    while r_norm > target and it < maxiter:
        Ap = apply_A(p)
        pAp = np.sum(p * Ap, dtype=dt)
        alpha = rz / pAp
        x = x + alpha * p
        r = r - alpha * Ap
        z = precond(r)
        rz_new = np.sum(r * z, dtype=dt)
        beta = rz_new / rz
        rz = rz_new
        p = z + beta * p
        it += 1
        r_norm = math.sqrt(float(np.sum(r * r, dtype=dt)))
    return x, PCGResult(it, r_norm, b_norm, r_norm <= target)


def elastic_energy_only(energy, s, materials, DmInv):
    """Per-tet elastic energy in s (the *_energy_only kernels,
    src/mfem/refinement/elastic_energy.py:155-176, 287-311)."""
    if energy == "arap":
        return arap_energy(s, materials, DmInv)[0]
    mu = materials[:, 0]
    lam = materials[:, 1]
    vol = rest_volume(DmInv)
    I2 = s[:, 0] ** 2 + s[:, 1] ** 2 + s[:, 2] ** 2 + 2.0 * (s[:, 3] ** 2 + s[:, 4] ** 2 + s[:, 5] ** 2)
    J = det_sym6(s)
    return vol * (mu * (I2 - 3.0) / 2.0 - mu * (J - 1.0) + lam / 2.0 * (J - 1.0) * (J - 1.0))


@dataclass
class LineSearchResult:
    accepted: bool
    alpha: float
    evaluations: int
    f0: float
    f1: float
    t: float


def backtracking(f, f0, t, alpha0, tau, threshold, max_iterations) -> LineSearchResult:
    """The device loop of src/mfem/line_search.py:76-163 on the host.
    f(alpha) is the merit at the trial alpha.  Trial j uses alpha0 tau^j; the
    loop goes on while (f0 - f1) + threshold < alpha t and the counter (j
    before the trial) is below max_iterations (_condition_kernel, :44-63),
    so it runs at most max_iterations + 1 trials.  The last trial is written
    only if the counter after it is below max_iterations
    (_iteration_condition and capture_if, :66-72, 148-161)."""
    alpha = alpha0
    j = 0
    while True:
        f1 = f(alpha)
        more = ((f0 - f1) + threshold < alpha * t) and j < max_iterations
        j += 1
        if not more:
            break
        alpha = alpha * tau
    return LineSearchResult(j < max_iterations, float(alpha), j, float(f0), float(f1), float(t))


class OracleSolver:
    """The reference's step on the CPU.  ``dtype`` float64 is the accuracy
    judge; float32 mirrors the reference's own precision."""

    def __init__(self, mesh, iterations=None, energy=None, cg_tolerance=None,
                 cg_max_iterations=None, attachment_stiffness=10.0,
                 preconditioner_singular_threshold=1.0e-20, dtype=np.float64,
                 line_search=False, line_search_max_iterations=20, line_search_alpha0=1.0,
                 line_search_tau=0.5, line_search_c=0.01, line_search_threshold=1.0e-8, contact=None):
        spec = mesh.spec
        self.dtype = np.dtype(dtype)
        f = lambda a: np.asarray(a).astype(self.dtype)
        self.iterations = spec.iterations if iterations is None else iterations
        self.energy = spec.energy if energy is None else energy
        self.tol = spec.cg_tolerance if cg_tolerance is None else cg_tolerance
        self.maxiter = spec.cg_max_iterations if cg_max_iterations is None else cg_max_iterations
        self.n = mesh.n
        self.T = mesh.T
        self.tets = mesh.tet_indices.astype(np.int64)
        self.DmInv = f(mesh.tet_poses)
        self.materials = f(mesh.tet_materials)
        self.mass = f(mesh.particle_mass)
        self.inv_mass = f(mesh.particle_inv_mass)
        self.gravity = f(mesh.gravity)
        self.k_attach = self.dtype.type(attachment_stiffness)
        self.singular_threshold = preconditioner_singular_threshold
        rest = f(mesh.rest_q)
        # attachments: vertices with inv_mass == 0, pinned to their rest
        # position (src/mfem/refinement/solver.py:345-393)
        self.pinned = self.inv_mass == 0.0
        self.pin_target = rest.copy()
        # Hessian mass: identity on pinned vertices, I / inv_mass elsewhere
        # (src/mfem/refinement/kernels.py:21-27)
        with np.errstate(divide="ignore"):
            m_h = np.where(self.pinned, self.dtype.type(1.0), self.dtype.type(1.0) / self.inv_mass)
        self.hess_mass = m_h.astype(self.dtype)
        self.hess_attach = np.where(self.pinned, self.k_attach, self.dtype.type(0.0))
        self.s = precompute_tet_stretch(rest, self.tets, self.DmInv)
        self.lmbda = np.zeros((self.T, 6), dtype=self.dtype)
        self.row_ptr, self.col_idx = bsr_sparsity(self.tets, self.n)
        self.last_pcg: list[PCGResult] = []
        self.line_search = line_search
        self.ls_max_iterations = line_search_max_iterations
        self.ls_alpha0 = line_search_alpha0
        self.ls_tau = line_search_tau
        self.ls_c = line_search_c
        self.ls_threshold = line_search_threshold
        self.last_line_search: list[LineSearchResult] = []
        # contact against rigid shapes (oracle/contact_oracle.ContactOracle)
        # and the body poses the step reads (state_out.body_q)
        self.contact = contact
        self.body_q = np.zeros((0, 7))

    # -- stages ------------------------------------------------------------
    def element_terms(self, x):
        """Everything per tet that one Newton iteration needs, evaluated at
        (x, s): constraint c, G, g_s, H_s, H_s^-1, H_lambda, g_lambda."""
        dt = self.dtype
        c, G = compute_constraints(x, self.tets, self.DmInv, self.s)
        if self.energy == "arap":
            _, g_s, H_s, H_si = arap_energy(self.s, self.materials, self.DmInv)
        else:
            _, g_s, H_s, H_si = neohookean_energy(self.s, self.materials, self.DmInv)
        INV = INV_SYM_DIAG.astype(dt)
        SYM = SYM_DIAG.astype(dt)
        H_l = INV[:, None] * H_s * INV[None, :]
        g_l = c + SYM * np.einsum("tij,tj->ti", H_si, g_s)
        return dict(c=c, G=G, g_s=g_s, H_s=H_s, H_si=H_si, H_l=H_l, g_l=g_l)

    def kinetic_gradient(self, x, x_tilde, dt):
        """m (x - x~)/dt^2 + (Q x + b)/dt^2 (src/mfem/refinement/kernels.py:172-185;
        solver.py:946-947)."""
        dt2 = self.dtype.type(dt) * self.dtype.type(dt)
        g = self.mass[:, None] * (x - x_tilde) / dt2
        att = self.hess_attach[:, None] * x - self.hess_attach[:, None] * self.pin_target
        return g + att / dt2

    def assemble(self, x, x_tilde, dt, el):
        """Dense-block BSR values [nnzb, 3, 3] and rhs [n, 3]."""
        import scipy.sparse as sp
        dtp = self.dtype
        G = el["G"]
        P = el["H_l"] @ G                                   # H_lambda G, [T, 6, 12]
        K = np.swapaxes(G, -1, -2) @ P                      # [T, 12, 12]
        f = np.einsum("tji,tj->ti", P, el["g_l"])           # (H_l G)^T g_l, [T, 12]
        n = self.n
        rows = (3 * self.tets[:, :, None] + np.arange(3)[None, None, :]).reshape(-1, 12)
        I = np.repeat(rows, 12, axis=1).ravel()
        J = np.tile(rows, (1, 12)).ravel()
        Hs = sp.coo_matrix((K.reshape(-1).astype(np.float64), (I, J)), shape=(3 * n, 3 * n)).tocsr()
        diag = (self.hess_mass + self.hess_attach) / (dtp.type(dt) * dtp.type(dt))
        Hs = Hs + sp.diags(np.repeat(diag.astype(np.float64), 3))
        Hs = Hs.tocsr()
        g = np.zeros((n, 3), dtype=np.float64)
        np.add.at(g, self.tets.ravel(), f.reshape(-1, 3).astype(np.float64))
        g = g - self.kinetic_gradient(x, x_tilde, dt)
        if self.contact is not None:
            # barrier + friction blocks on the diagonal, tri blocks on tri
            # vertex pairs; their gradients leave g (solver.py:734-779)
            _, gv, Hv = self.contact.vertex_terms(x.astype(np.float64), self.body_q, dt)
            _, gt, tri_blocks = self.contact.tri_terms(x.astype(np.float64), self.body_q)
            rows = np.repeat(3 * np.arange(n), 9) + np.tile(np.repeat(np.arange(3), 3), n)
            cols = np.repeat(3 * np.arange(n), 9) + np.tile(np.tile(np.arange(3), 3), n)
            C = sp.coo_matrix((Hv.reshape(-1), (rows, cols)), shape=(3 * n, 3 * n))
            if tri_blocks:
                bi = np.array([b[0] for b in tri_blocks])
                bj = np.array([b[1] for b in tri_blocks])
                bv = np.stack([b[2] for b in tri_blocks])
                r2 = (3 * bi[:, None, None] + np.arange(3)[None, :, None]).repeat(3, axis=2).reshape(-1)
                c2 = (3 * bj[:, None, None] + np.arange(3)[None, None, :]).repeat(3, axis=1).reshape(-1)
                C = C + sp.coo_matrix((bv.reshape(-1), (r2, c2)), shape=(3 * n, 3 * n))
            Hs = (Hs + C).tocsr()
            g = g - gv - gt
        # gather the BSR blocks in slot order
        rp, ci = self.row_ptr, self.col_idx
        br = np.repeat(np.arange(n), np.diff(rp))
        blocks = np.empty((ci.shape[0], 3, 3), dtype=np.float64)
        for a in range(3):
            for b_ in range(3):
                blocks[:, a, b_] = np.asarray(Hs[3 * br + a, 3 * ci + b_]).ravel()
        return blocks.astype(dtp), g.astype(dtp), Hs

    def bsr_apply(self, blocks):
        """v -> H v for H's 3x3 blocks in slot order (warp.sparse.bsr_mv), as
        scipy's block-sparse product in the blocks' dtype."""
        import scipy.sparse as sp
        n = self.n
        H = sp.bsr_matrix((blocks, self.col_idx, self.row_ptr), shape=(3 * n, 3 * n))

        def apply(v):
            return (H @ np.ascontiguousarray(v).reshape(-1)).reshape(n, 3)
        return apply

    def diag_blocks(self, blocks):
        rp, ci = self.row_ptr, self.col_idx
        n = self.n
        br = np.repeat(np.arange(n), np.diff(rp))
        d = np.flatnonzero(br == ci)
        return blocks[d]

    def local_solve(self, el, dx):
        """lambda = -H_l (g_l - G dx_e); ds = -H_s^-1 (SYM lambda + g_s)
        (src/mfem/refinement/kernels.py:252-283)."""
        dxe = dx[self.tets].reshape(self.T, 12)
        Gdx = np.einsum("tij,tj->ti", el["G"], dxe)
        lam = -np.einsum("tij,tj->ti", el["H_l"], el["g_l"] - Gdx)
        SYM = SYM_DIAG.astype(self.dtype)
        ds = -np.einsum("tij,tj->ti", el["H_si"], SYM * lam + el["g_s"])
        return lam, ds

    def objective(self, x, s, x_tilde, dt):
        """Merit function with lambda fixed: kinetic + attachment terms over
        dt^2 plus, per tet, elastic energy minus lambda . c(x, s)
        (src/mfem/refinement/solver.py:803-869).  The attachment energy
        0.5 k |x - p|^2 is the reference's x.(0.5 Q x + b) + c
        (src/mfem/boundary_condition.py:62-71) in a cancellation-free form."""
        dtp = self.dtype
        d = x - x_tilde
        kin = np.sum(dtp.type(0.5) * self.mass * np.sum(d * d, axis=1), dtype=dtp)
        e = x - self.pin_target
        att = np.sum(dtp.type(0.5) * self.hess_attach * np.sum(e * e, axis=1), dtype=dtp)
        inv_dt2 = dtp.type(1.0 / (dt * dt))
        c, _ = compute_constraints(x, self.tets, self.DmInv, s)
        tet = elastic_energy_only(self.energy, s, self.materials, self.DmInv) - np.sum(c * self.lmbda, axis=1)
        f = inv_dt2 * kin + inv_dt2 * att + np.sum(tet, dtype=dtp)
        if self.contact is not None:
            f = f + dtp.type(self.contact.energy(np.asarray(x, dtype=np.float64), self.body_q, dt))
        return f

    def line_search_update(self, x, x_tilde, dt, el, dx, ds):
        """Backtracking Armijo search along (dx, ds) (src/mfem/line_search.py:
        76-163): alpha = alpha0 tau^j until (f0 - f1) + threshold >= alpha t,
        t = -c (g_x . dx + g_s,lambda . ds) with g_x = kinetic/attachment
        gradient - G^T lambda and g_s,lambda = g_s + SYM lambda
        (src/mfem/refinement/solver.py:897-915).  The update is written only
        if the accepting trial index j has j + 1 < max_iterations; a search
        that never passes stops after trial max_iterations and writes nothing
        (the counter test of src/mfem/line_search.py:44-63, 148-161).  The
        x-gradient keeps the reference's sign: G is its dC_dX, which is
        -dc/dx (kernels.py:159), so g_x - G^T lambda is not the gradient of
        the merit function, whose x-part is g_x + G^T lambda."""
        dtp = self.dtype
        SYM = SYM_DIAG.astype(dtp)
        gx = self.kinetic_gradient(x, x_tilde, dt)
        GtL = np.zeros_like(x)
        contrib = np.einsum("tik,ti->tk", el["G"], self.lmbda).reshape(self.T, 4, 3)
        np.add.at(GtL, self.tets.ravel(), contrib.reshape(-1, 3))
        grad_x = gx - GtL
        if self.contact is not None:
            # + barrier and friction gradients (solver.py:909)
            _, gv, _ = self.contact.vertex_terms(np.asarray(x, dtype=np.float64), self.body_q, dt)
            _, gt, _ = self.contact.tri_terms(np.asarray(x, dtype=np.float64), self.body_q)
            grad_x = grad_x + (gv + gt).astype(dtp)
        grad_s = el["g_s"] + SYM * self.lmbda
        m = np.sum(grad_x * dx, dtype=dtp) + np.sum(grad_s * ds, dtype=dtp)
        t = -dtp.type(self.ls_c) * m
        f0 = self.objective(x, self.s, x_tilde, dt)
        trial = {}

        def f(alpha):
            trial["x"], trial["s"] = x + alpha * dx, self.s + alpha * ds
            return self.objective(trial["x"], trial["s"], x_tilde, dt)

        res = backtracking(f, f0, t, dtp.type(self.ls_alpha0), dtp.type(self.ls_tau),
                           dtp.type(self.ls_threshold), self.ls_max_iterations)
        self.last_line_search.append(res)
        if res.accepted:
            return trial["x"], trial["s"]
        return x, self.s

    # -- the step ------------------------------------------------------------
    def predictor(self, q, qd, dt):
        """x~ = x + v dt + g dt^2 / 2 (src/mfem/refinement/kernels.py:77-91)."""
        dtp = self.dtype
        dtc = dtp.type(dt)
        return (np.asarray(q).astype(dtp) + np.asarray(qd).astype(dtp) * dtc
                + self.gravity[None, :] * dtc * dtc / dtp.type(2.0))

    def step(self, q, qd, dt):
        """One implicit-Euler step: returns (q_out, qd_out); s and lambda
        persist in the solver (src/mfem/refinement/solver.py:429-579)."""
        dtp = self.dtype
        x_in = np.asarray(q).astype(dtp)
        dtc = dtp.type(dt)
        x_tilde = self.predictor(q, qd, dt)
        x = x_in.copy()
        if self.contact is not None:
            self.contact.begin_step(x_in.astype(np.float64), self.body_q)
        self.last_pcg = []
        self.last_line_search = []
        for _ in range(self.iterations):
            el = self.element_terms(x)
            blocks, g, _ = self.assemble(x, x_tilde, dt, el)
            Minv = block_jacobi_inverse(self.diag_blocks(blocks), self.singular_threshold)
            dx, res = pcg(self.bsr_apply(blocks), g, x_tilde - x, Minv, self.tol, self.maxiter)
            self.last_pcg.append(res)
            lam, ds = self.local_solve(el, dx)
            self.lmbda = lam
            if self.line_search:
                x, self.s = self.line_search_update(x, x_tilde, dt, el, dx, ds)
            else:
                x = x + dx
                self.s = self.s + ds
        v = (x - x_in) / dtc
        return x, v
