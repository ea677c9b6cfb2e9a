"""Regenerates the golden fixtures of tests/golden/.

known_answers.npz -- the inputs of the reference's own known-answer tests for
    the element math, rebuilt from the seeds and literals those tests use
    (tests/test_kernels.py:59-99, 139-298; tests/test_functions.py:103-149;
    tests/numerical/test_psd_fix.py:227-253), with the float64 oracle's
    outputs for them.
cantilever_fp64.npz -- the float64 oracle's 100-step trajectory of the
    10x2x2 ARAP cantilever (positions after every step, final s and lambda,
    PCG iterations per Newton iteration).
reference_fixture_digests.json -- sha256 digests and shapes of the arrays of
    the reference's fem_beam.npz (written only where the reference tree is
    present), so the 5-tet grid generator is pinned to it without copying it.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "warp-mfem_gb300"), ROOT]

from mfem_gb300 import beams  # noqa: E402
from oracle import mfem_oracle as O  # noqa: E402


def rotation_case():
    """tests/test_kernels.py:59-99: a tet rotated 12 degrees about z."""
    from scipy.spatial.transform import Rotation
    og = np.array([[0.0, 0.0, 0.0], [0.0, 1.0, 0.0], [-1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])
    new = Rotation.from_euler("xyz", [0, 0, 12], degrees=True).apply(og)
    rest_rows = np.hstack([og[1] - og[0], og[2] - og[0], og[3] - og[0]]).reshape(3, 3)
    return new, np.linalg.inv(rest_rows)


def deformations():
    """The five deformations of tests/test_kernels.py:140-142 / test_functions.py:113-116."""
    rng = np.random.default_rng(42)
    return np.stack([np.eye(3)] + [rng.normal(size=(3, 3)) * 0.3 + np.eye(3) for _ in range(4)])


def single_tet(defo):
    base = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    return base @ defo.T, np.array([[0, 1, 2, 3]], dtype=np.int32)


def cube(defo):
    import scipy.spatial
    corners = np.array([[x, y, z] for x in [0.0, 1.0] for y in [0.0, 1.0] for z in [0.0, 1.0]])
    tri = scipy.spatial.Delaunay(corners)
    return corners @ defo.T, tri.simplices.astype(np.int32)


def rest_rows_inverse(pos, tets):
    """tests/utils.py:321-335: DmInv = inv(matrix_from_rows(x1-x0, x2-x0, x3-x0))."""
    x = pos[tets]
    rows = np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], axis=1)
    return np.linalg.inv(rows)


def psd_inputs():
    """tests/numerical/test_psd_fix.py:227-253."""
    A3_pd = np.array([[4.0, 1.0, 1.0], [1.0, 3.0, 1.0], [1.0, 1.0, 5.0]], dtype=np.float32)
    A3_non_pd = np.array([[1.0, 3.0, 2.0], [3.0, 1.0, -4.0], [2.0, -4.0, 1.0]], dtype=np.float32)
    A6_pd = np.diag([4.0, 3.0, 5.0, 2.0, 6.0, 4.0]).astype(np.float32)
    rng = np.random.default_rng(0)
    Q = np.linalg.qr(rng.standard_normal((6, 6)))[0].astype(np.float32)
    D = np.diag([3.0, 2.0, 5.0, -1.0, 1.0, -2.0]).astype(np.float32)
    M = Q @ D @ Q.T
    A6_non_pd = (M + M.T) / 2
    return A3_pd, A3_non_pd, A6_pd, A6_non_pd


def known_answers():
    out = {}
    pos, dm = rotation_case()
    out["rot_pos"] = pos
    out["rot_dminv"] = dm[None]
    defo = deformations()
    out["deformations"] = defo
    for name, maker in (("tet", single_tet), ("cube", cube)):
        for i, d in enumerate(defo):
            p, t = maker(d)
            dminv = rest_rows_inverse(p, t)
            s = O.precompute_tet_stretch(p, t, dminv)
            c, G = O.compute_constraints(p, t, dminv, s)
            out[f"{name}{i}_pos"] = p
            out[f"{name}{i}_tets"] = t
            out[f"{name}{i}_dminv"] = dminv
            out[f"{name}{i}_s"] = s
            out[f"{name}{i}_G"] = G
    for name, A in zip(("A3_pd", "A3_non_pd", "A6_pd", "A6_non_pd"), psd_inputs()):
        fixed, inv = O.psd_fix(A.astype(np.float64)[None])
        out[name] = A
        out[name + "_fixed"] = fixed[0]
        out[name + "_inv"] = inv[0]
    return out


def cantilever_trajectory():
    mesh = beams.build_beam("cantilever")
    solver = O.OracleSolver(mesh, dtype=np.float64)
    q, qd = mesh.q0, mesh.qd0
    qs, iters = [], []
    for _ in range(mesh.spec.steps):
        q, qd = solver.step(q, qd, mesh.spec.dt)
        qs.append(q.copy())
        iters.append([r.iterations for r in solver.last_pcg])
    return dict(q=np.stack(qs), qd_final=qd, s_final=solver.s, lambda_final=solver.lmbda,
                pcg_iterations=np.array(iters, dtype=np.int32))


REFERENCE_TREE = "/root/reference"


def array_digest(a: np.ndarray) -> dict:
    import hashlib
    a = np.ascontiguousarray(a)
    return {"dtype": str(a.dtype), "shape": list(a.shape), "sha256": hashlib.sha256(a.tobytes()).hexdigest()}


def reference_fixture_digests():
    path = os.path.join(REFERENCE_TREE, "fem_beam.npz")
    if not os.path.exists(path):
        return None
    d = np.load(path)
    return {"fem_beam.npz": {k: array_digest(d[k]) for k in ("particles", "tet_indices", "tet_materials")}
            | {"parameters": d["parameters"].tolist()}}


def main():
    import json
    digests = reference_fixture_digests()
    if digests is not None:
        with open(os.path.join(HERE, "reference_fixture_digests.json"), "w") as f:
            json.dump(digests, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "known_answers.npz"), **known_answers())
    np.savez_compressed(os.path.join(HERE, "cantilever_fp64.npz"), **cantilever_trajectory())
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
