"""Independent bodies stepped in one plan (per-body PCGs in one persistent
launch) against each body stepped alone: by the float64 oracle, and by this
library's single-body solver.  Tolerance: positions 1e-5 relative to each
body's largest position, the bar of the single-body step."""
import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib, beams
from mfem_gb300.batched import BatchedSolver
from oracle import mfem_oracle as O

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def small_batch(n=10, seed=7):
    return beams.batched_bodies(n, seed=seed, nx=(2, 7), nyz=(1, 3))


def run(bs, steps):
    A, B = bs.state(), bs.model.state()
    stats = []
    for _ in range(steps):
        bs.step(A, B)
        A, B = B, A
        stats.append(bs.body_stats())
    return A.particle_q.cpu().numpy(), stats


def close_per_body(q, refs, offsets, rtol=1e-5):
    for k, ref in enumerate(refs):
        got = q[offsets[k]:offsets[k + 1]]
        err = np.abs(got - ref).max()
        assert err <= rtol * np.abs(ref).max(), f"body {k}: max err {err:.3e}"


def test_batch_matches_each_body_alone_by_the_oracle():
    batch = small_batch()
    bs = BatchedSolver(batch, device=DEV)
    q, stats = run(bs, 3)
    refs = []
    for m in batch.bodies:
        S = O.OracleSolver(m, dtype=np.float64)
        qq, vv = m.q0, m.qd0
        for _ in range(3):
            qq, vv = S.step(qq, vv, m.spec.dt)
        refs.append(qq)
    close_per_body(q, refs, batch.vertex_offsets)
    assert all((s["status"] == _lib.MFEM_OK).all() for s in stats)
    assert all((s["iterations"] > 0).any() for s in stats)


def test_batch_matches_the_single_body_solver():
    batch = small_batch(6, seed=3)
    bs = BatchedSolver(batch, device=DEV)
    q, stats = run(bs, 2)
    refs = []
    for m in batch.bodies:
        model = Model.from_beam(m, device=DEV)
        solver = MixedFEMSolver(model, iterations=8, energy=m.spec.energy, line_search=False)
        A, B = model.state(), model.state()
        for _ in range(2):
            solver.step(A, B, None, None, m.spec.dt)
            A, B = B, A
        refs.append(A.particle_q.cpu().numpy())
    close_per_body(q, refs, batch.vertex_offsets)


def test_schedules_agree_and_autotune_picks_one():
    batch = beams.batched_bodies(4, seed=11, nx=(20, 24), nyz=(5, 6))
    outs = []
    for tune in (False, True):
        bs = BatchedSolver(batch, device=DEV)
        if tune:
            # a step first, so the group barriers' counters have moved on
            # before the schedule (and the group sizes) change
            run(bs, 1)
            ms = bs.autotune()
            assert ms > 0.0
        lay = bs.layout()
        assert lay["threads"] in (128, 256, 512) and lay["ctas"] >= batch.n_bodies
        q, stats = run(bs, 2)
        assert all((s["status"] == _lib.MFEM_OK).all() for s in stats)
        outs.append(q)
    scale = np.abs(outs[0]).max()
    assert np.abs(outs[0] - outs[1]).max() <= 1e-5 * scale


def test_multi_cta_bodies_match_the_oracle():
    """Two large bodies split over many CTAs each (group barriers) and a
    small one on a single CTA."""
    bodies = [beams.build_beam(beams.BeamSpec(name="a", cells=(24, 8, 8), extent=(1.2, 0.4, 0.4),
                                              energy="neohookean", E=(1e4, 1e6), nu=0.45, seed=5,
                                              gravity=(0.0, -9.81, 0.0))),
              beams.build_beam(beams.BeamSpec(name="b", cells=(3, 2, 2), extent=(0.15, 0.1, 0.1), energy="arap",
                                              E=(1e5, 1e5), nu=0.4, seed=6, gravity=(9.81, 0.0, 0.0))),
              beams.build_beam(beams.BeamSpec(name="c", cells=(20, 6, 10), extent=(1.0, 0.3, 0.5),
                                              energy="arap", E=(1e4, 1e6), nu=0.35, seed=7,
                                              gravity=(0.0, 0.0, -9.81)))]
    batch = beams.concatenate(bodies)
    bs = BatchedSolver(batch, device=DEV)
    q, stats = run(bs, 2)
    assert bs.layout()["ctas"] > 3  # the large bodies got groups
    refs = []
    for m in bodies:
        S = O.OracleSolver(m, dtype=np.float64)
        qq, vv = m.q0, m.qd0
        for _ in range(2):
            qq, vv = S.step(qq, vv, m.spec.dt)
        refs.append(qq)
    close_per_body(q, refs, batch.vertex_offsets)


def test_batch_graph_and_eager_agree_bitwise():
    batch = small_batch(8, seed=2)
    outs = []
    for graph in (True, False):
        bs = BatchedSolver(batch, device=DEV, use_cuda_graph=graph)
        q, _ = run(bs, 2)
        outs.append(q)
    np.testing.assert_array_equal(outs[0], outs[1])


def test_set_bodies_rejects_bad_input():
    batch = small_batch(3, seed=1)
    voff = batch.vertex_offsets.copy()
    voff[1] += 1  # a tet of body 0 now uses a vertex counted in body 1... or the reverse
    batch_bad = beams.BodyBatch(bodies=batch.bodies, union=batch.union, vertex_offsets=voff,
                                tet_offsets=batch.tet_offsets, energies=batch.energies, gravity=batch.gravity)
    with pytest.raises(_lib.MfemError):
        BatchedSolver(batch_bad, device=DEV)
    u = batch.union
    model = Model(u.rest_q, np.zeros_like(u.rest_q), u.particle_mass, u.particle_inv_mass, u.tet_indices,
                  u.tet_poses, u.tet_materials, u.gravity, device=DEV)
    solver = MixedFEMSolver(model, iterations=2, line_search=True)
    import ctypes
    h = [np.ascontiguousarray(a) for a in (batch.vertex_offsets, batch.tet_offsets,
                                           np.zeros(3, np.int32), batch.gravity)]
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = solver._lib.mfem_plan_set_bodies(solver._plan, 3, *[P(a) for a in h])
    assert rc == _lib.MFEM_BAD_ARG and b"line_search" in solver._lib.mfem_plan_last_error(solver._plan)
