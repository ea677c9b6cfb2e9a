"""A float64 reference solve of an assembled 3x3-block BSR system, as test
infrastructure: block-Jacobi CG in float64 on the GPU through torch's
sparse CSR product, run to 1e-13, and certified by its float64 residual
formed independently on the host with scipy.  It judges the library's
mixed-precision solves of the same H; it is not part of the library."""
from __future__ import annotations

import numpy as np
import torch


def scalar_csr(row_ptr: np.ndarray, col_idx: np.ndarray, values: np.ndarray, n: int):
    """The 3n x 3n scalar CSR (indptr, indices, data) of an n x n BSR of 3x3
    blocks with ascending columns per block row."""
    counts = np.diff(row_ptr)
    br = np.repeat(np.arange(n), counts)
    vals = values.reshape(-1, 3, 3)
    # row 3r+a holds, for each block k of block row r, entries (3c+b, vals[k, a, b])
    indptr = np.zeros(3 * n + 1, dtype=np.int64)
    per_row = 3 * counts
    indptr[1:] = np.cumsum(np.repeat(per_row, 3))
    # entries of scalar row 3r+a: blocks of row r in order, b = 0..2
    k_of = np.repeat(np.arange(len(br)), 3)          # block of each entry, within its block row
    b_of = np.tile(np.arange(3), len(br))
    indices = np.empty(indptr[-1], dtype=np.int64)
    data = np.empty(indptr[-1], dtype=np.float64)
    for a in range(3):
        # positions of scalar row 3r+a in the flat arrays
        starts = indptr[3 * np.arange(n) + a]
        pos = np.repeat(starts, per_row) + (np.arange(len(k_of)) - np.repeat(3 * row_ptr[:-1], per_row))
        indices[pos] = 3 * col_idx[k_of] + b_of
        data[pos] = vals[k_of, a, b_of]
    return indptr, indices, data


def solve_fp64(row_ptr, col_idx, values, g, n, device, tol=1e-13, maxiter=200000, check_every=50):
    """x with ||g - H x|| <= tol ||g|| in float64 (block-Jacobi CG from 0).
    Returns (x [n, 3] float64 numpy, iterations, certified relative residual
    computed on the host with scipy)."""
    import scipy.sparse as sp
    indptr, indices, data = scalar_csr(np.asarray(row_ptr), np.asarray(col_idx), np.asarray(values, np.float64), n)
    H = torch.sparse_csr_tensor(torch.as_tensor(indptr, device=device), torch.as_tensor(indices, device=device),
                                torch.as_tensor(data, device=device), size=(3 * n, 3 * n))
    b = torch.as_tensor(np.asarray(g, np.float64).reshape(-1), device=device)
    vals = np.asarray(values, np.float64).reshape(-1, 3, 3)
    br = np.repeat(np.arange(n), np.diff(row_ptr))
    diag = vals[np.flatnonzero(br == np.asarray(col_idx))]
    Minv = torch.as_tensor(np.linalg.inv(diag), device=device)

    def prec(v):
        return torch.bmm(Minv, v.view(n, 3, 1)).view(-1)

    x = torch.zeros_like(b)
    r = b.clone()
    z = prec(r)
    p = z.clone()
    rz = torch.dot(r, z)
    bb = float(torch.dot(b, b))
    thr = tol * tol * bb
    it = 0
    while it < maxiter:
        Ap = torch.mv(H, p)
        alpha = rz / torch.dot(p, Ap)
        x += alpha * p
        r -= alpha * Ap
        it += 1
        if it % check_every == 0 and float(torch.dot(r, r)) <= thr:
            break
        z = prec(r)
        rz_new = torch.dot(r, z)
        p = z + (rz_new / rz) * p
        rz = rz_new
    xs = x.cpu().numpy()
    Hs = sp.csr_matrix((data, indices, indptr), shape=(3 * n, 3 * n))
    gb = np.asarray(g, np.float64).reshape(-1)
    rel = float(np.linalg.norm(gb - Hs @ xs) / np.linalg.norm(gb))
    return xs.reshape(n, 3), it, rel


def residual_fp64(row_ptr, col_idx, values, g, x, n) -> float:
    """||g - H x|| / ||g|| in float64 on the host."""
    import scipy.sparse as sp
    indptr, indices, data = scalar_csr(np.asarray(row_ptr), np.asarray(col_idx), np.asarray(values, np.float64), n)
    Hs = sp.csr_matrix((data, indices, indptr), shape=(3 * n, 3 * n))
    gb = np.asarray(g, np.float64).reshape(-1)
    return float(np.linalg.norm(gb - Hs @ np.asarray(x, np.float64).reshape(-1)) / np.linalg.norm(gb))
