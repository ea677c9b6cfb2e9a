"""Parity at the workloads' own sizes.

* nh_beam (64x16x16 cells, 98,304 tets, Neo-Hookean, 50 steps): positions
  against the float64 oracle's committed trajectory (tests/golden/
  nh_beam_fp64.npz, written by tests/golden/make_golden.py) after step 1
  and every 5th step, within 1e-5 of the largest position.
* stiff_beam (128x32x32 cells, 786,432 tets, E log-uniform [1e4, 1e7]):
  one step with the mixed-precision solve (fp16 and bf16 blocks with row
  scales, fp32 inner PCG to 1e-3, fp64 refinement to 1e-8).  Each of the 8
  solves is judged against a float64 solve of the same assembled H
  (tests/fp64_reference.py, certified by its host-side residual): the
  solution's relative error and its float64 residual.
* batched512 (512 uneven bodies, seed 4): one step of the batch against each
  body stepped alone by the single-body solver (1e-5 of the body's largest
  position), and a seeded subset with the smallest and the largest body
  against the float64 oracle.

The reference for all of them: RefinementSolver.step
(src/mfem/refinement/solver.py:429-579).
"""
import os

import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib, beams
from mfem_gb300.batched import BatchedSolver
from oracle import mfem_oracle as O
from fp64_reference import residual_fp64, solve_fp64

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
GOLD = os.path.join(os.path.dirname(__file__), "golden", "nh_beam_fp64.npz")


def test_nh_beam_50_steps_match_fp64_trajectory():
    gold = np.load(GOLD)
    mesh = beams.build_beam("nh_beam")
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=mesh.spec.iterations, energy=mesh.spec.energy, line_search=False)
    s0, s1 = model.state(), model.state()
    s0.particle_q.copy_(torch.as_tensor(mesh.q0, device=DEV))
    keep = {int(k): i for i, k in enumerate(gold["steps"])}
    worst = 0.0
    for k in range(1, mesh.spec.steps + 1):
        solver.step(s0, s1, None, None, mesh.spec.dt)
        stats = solver.solve_stats()
        assert all(st["status"] == 0 for st in stats), (k, stats)
        if k in keep:
            q = s1.particle_q.cpu().numpy().astype(np.float64)
            ref = mesh.rest_q.astype(np.float64) + gold["displacement"][keep[k]].astype(np.float64)
            err = np.abs(q - ref).max() / np.abs(ref).max()
            worst = max(worst, err)
            assert err <= 1e-5, (k, err)
        s0, s1 = s1, s0
    assert len(keep) == 11
    print(f"nh_beam 50 steps: worst relative position error {worst:.2e}")


@pytest.mark.parametrize("precision", ["fp16", "bf16"])
def test_stiff_beam_mixed_solves_against_fp64(precision):
    mesh = beams.build_beam("stiff_beam")
    spec = mesh.spec
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=spec.iterations, energy=spec.energy, line_search=False,
                            cg_max_iterations=spec.cg_max_iterations, solver_precision=precision,
                            inner_tolerance=1e-3, outer_tolerance=1e-8, outer_max_iterations=10)
    q = torch.as_tensor(mesh.q0, device=DEV)
    x = q.clone()
    solver.predict(q, torch.zeros_like(q), spec.dt)
    row_ptr = solver.read_buffer("row_ptr").cpu().numpy()
    col_idx = solver.read_buffer("col_idx").cpu().numpy()
    rows = []
    for it in range(spec.iterations):
        solver.update_system(x)
        solver.assemble(x, spec.dt)
        solver.global_solve(it)
        torch.cuda.synchronize()
        H = solver.read_buffer("h_values").cpu().numpy()
        g = solver.read_buffer("rhs").cpu().numpy().reshape(-1, 3)
        dx32 = solver.read_buffer("dx").cpu().numpy().reshape(-1, 3)
        dx64 = solver.read_buffer("mixed_dx").cpu().numpy().reshape(-1, 3)
        z, z_its, z_res = solve_fp64(row_ptr, col_idx, H, g, mesh.n, DEV)
        assert z_res <= 1e-11, f"reference solve residual {z_res:.2e} after {z_its} iterations"
        st = solver.mixed_stats()[it]
        rows.append(dict(
            iteration=it, status=st["status"], outer=st["outer_iterations"], inner=st["inner_iterations"],
            fp32_inner=st["fp32_inner"], reported=st["rel_residual"],
            residual=residual_fp64(row_ptr, col_idx, H, g, dx64, mesh.n),
            residual_fp32_dx=residual_fp64(row_ptr, col_idx, H, g, dx32, mesh.n),
            error=float(np.linalg.norm(dx64 - z) / np.linalg.norm(z)),
            error_fp32_dx=float(np.linalg.norm(dx32 - z) / np.linalg.norm(z))))
        solver.local_solve(x)
    for r in rows:
        print(precision, {k: (f"{v:.2e}" if isinstance(v, float) else v) for k, v in r.items()})
    for r in rows:
        # the refinement's own fp64 residual is the host's, to rounding
        assert abs(r["residual"] - r["reported"]) <= 1e-3 * r["residual"] + 1e-12
        assert np.isfinite(r["error"])
        if r["status"] == _lib.MFEM_OK:
            assert r["residual"] <= 1e-8
    if precision == "fp16":
        assert all(r["status"] == _lib.MFEM_OK for r in rows)
        # a residual of 1e-8 bounds the solution error by cond(H) 1e-8
        assert max(r["error"] for r in rows) <= 1e-3
    assert np.isfinite(x.cpu().numpy()).all()


def test_batched512_bodies_match_single_body_solver_and_oracle():
    batch = beams.batched_bodies(512, seed=4)
    bs = BatchedSolver(batch, device=DEV)
    A, B = bs.state(), bs.model.state()
    bs.step(A, B)
    q = B.particle_q.cpu().numpy()
    stats = bs.body_stats()
    assert (stats["status"] == _lib.MFEM_OK).all()
    voff = batch.vertex_offsets
    worst = 0.0
    for k, m in enumerate(batch.bodies):
        model = Model.from_beam(m, device=DEV)
        solver = MixedFEMSolver(model, iterations=8, energy=m.spec.energy, line_search=False, use_cuda_graph=False)
        s0, s1 = model.state(), model.state()
        solver.step(s0, s1, None, None, m.spec.dt)
        ref = s1.particle_q.cpu().numpy()
        solver.close()
        err = np.abs(q[voff[k]:voff[k + 1]] - ref).max() / np.abs(ref).max()
        worst = max(worst, err)
        assert err <= 1e-5, f"body {k}: relative error {err:.2e}"
    print(f"batched512: worst relative error against the single-body solver {worst:.2e}")
    # the float64 oracle on the smallest, the largest and two seeded bodies
    sizes = np.array([m.T for m in batch.bodies])
    rng = np.random.default_rng(4)
    pick = sorted({int(sizes.argmin()), int(sizes.argmax()), *map(int, rng.choice(len(sizes), 2, replace=False))})
    for k in pick:
        m = batch.bodies[k]
        ref, _ = O.OracleSolver(m, dtype=np.float64).step(m.q0, m.qd0, m.spec.dt)
        err = np.abs(q[voff[k]:voff[k + 1]] - ref).max() / np.abs(ref).max()
        assert err <= 1e-5, f"body {k} ({m.T} tets) against the oracle: relative error {err:.2e}"
