"""Regenerates the golden fixtures of tests/golden/.

known_answers.npz -- the inputs of the reference's own known-answer tests for
    the element math, rebuilt from the seeds and literals those tests use
    (tests/test_kernels.py:59-99, 139-298; tests/test_functions.py:103-149;
    tests/numerical/test_psd_fix.py:227-253), with the float64 oracle's
    outputs for them.
cantilever_fp64.npz -- the float64 oracle's 100-step trajectory of the
    10x2x2 ARAP cantilever (positions after every step, final s and lambda,
    PCG iterations per Newton iteration).
nh_beam_fp64.npz -- the float64 oracle's 50-step run of the full Neo-Hookean
    beam (64x16x16 cells, 98,304 tets): displacements from rest (float32)
    after step 1 and every 5th step, PCG iterations per Newton iteration.
    About half an hour on one core.
reference_fixture_digests.json -- sha256 digests and shapes of the arrays of
    the reference's fem_beam.npz (written only where the reference tree is
    given and holds it), so the 5-tet grid generator is pinned to it without
    copying it.

Run from the repository root:
    python tests/golden/make_golden.py [--reference-tree DIR] [fixture ...]
with fixture among known_answers, cantilever, nh_beam, digests (default:
all).  The reference tree comes from --reference-tree or the environment
variable MFEM_REFERENCE_TREE; without either the digests are left as they
are.
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


def nh_beam_trajectory(stride: int = 5):
    """The full nh_beam workload (64x16x16 cells, 50 steps) by the float64
    oracle: displacements q - q_rest after steps 1, stride, 2 stride, ...
    stored as float32 (1e-8 m resolution, far below the 1e-5 relative
    tolerance the GPU test applies to positions of up to 2 m)."""
    mesh = beams.build_beam("nh_beam")
    solver = O.OracleSolver(mesh, dtype=np.float64)
    q, qd = mesh.q0, mesh.qd0
    keep, disp, iters = [], [], []
    for k in range(1, mesh.spec.steps + 1):
        q, qd = solver.step(q, qd, mesh.spec.dt)
        iters.append([r.iterations for r in solver.last_pcg])
        if k == 1 or k % stride == 0:
            keep.append(k)
            disp.append((q - mesh.rest_q).astype(np.float32))
        print(f"nh_beam oracle step {k}: PCG iterations {iters[-1]}", flush=True)
    return dict(steps=np.array(keep, dtype=np.int32), displacement=np.stack(disp),
                pcg_iterations=np.array(iters, dtype=np.int32))


def array_digest(a: np.ndarray) -> dict:
    import hashlib
    a = np.ascontiguousarray(a)
    return {"dtype": str(a.dtype), "shape": list(a.shape), "sha256": hashlib.sha256(a.tobytes()).hexdigest()}


def reference_fixture_digests(reference_tree):
    if not reference_tree:
        return None
    path = os.path.join(reference_tree, "fem_beam.npz")
    if not os.path.exists(path):
        raise SystemExit(f"{path} not found: --reference-tree must name the reference's checkout")
    d = np.load(path)
    return {"fem_beam.npz": {k: array_digest(d[k]) for k in ("particles", "tet_indices", "tet_materials")}
            | {"parameters": d["parameters"].tolist()}}


FIXTURES = ("known_answers", "cantilever", "nh_beam", "digests")


def main(argv=None):
    import argparse
    import json
    ap = argparse.ArgumentParser(description="Regenerates the golden fixtures of tests/golden/.")
    ap.add_argument("--reference-tree", default=os.environ.get("MFEM_REFERENCE_TREE"),
                    help="checkout of the reference (default: $MFEM_REFERENCE_TREE)")
    ap.add_argument("fixtures", nargs="*", help=f"any of {', '.join(FIXTURES)} (default: all)")
    args = ap.parse_args(argv)
    unknown = set(args.fixtures) - set(FIXTURES)
    if unknown:
        ap.error(f"unknown fixture(s) {sorted(unknown)}; choose from {FIXTURES}")
    which = set(args.fixtures or FIXTURES)
    if "digests" in which:
        digests = reference_fixture_digests(args.reference_tree)
        if digests is not None:
            with open(os.path.join(HERE, "reference_fixture_digests.json"), "w") as f:
                json.dump(digests, f, indent=1)
        else:
            print("no reference tree given: reference_fixture_digests.json left as it is")
    if "known_answers" in which:
        np.savez_compressed(os.path.join(HERE, "known_answers.npz"), **known_answers())
    if "cantilever" in which:
        np.savez_compressed(os.path.join(HERE, "cantilever_fp64.npz"), **cantilever_trajectory())
    if "nh_beam" in which:
        np.savez_compressed(os.path.join(HERE, "nh_beam_fp64.npz"), **nh_beam_trajectory())
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
