"""The FSAI preconditioner (preconditioner="fsai"), in the persistent factor
PCG (pcg_variant "factor", the default where it fits) and in the
global-memory PCG.

It has no reference counterpart: the reference's PCG is block-Jacobi.  The
bar is:
* the factor G the setup kernel writes equals the FSAI of the same fp32 H
  computed here in float64 numpy (block row i over the row's lower block
  columns P: G[i, P] = the last block row of chol(H[P, P])^-1), to 1e-3 of
  the row's largest entry -- fp32 dense Cholesky of up to 48 x 48 local
  matrices against float64;
* every diagonal block of G H G^T is the identity to 1e-3;
* the solve takes fewer iterations than block-Jacobi on the same system and
  a trajectory stays within 1e-5 of the float64 oracle, the bar of the
  block-Jacobi step.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib, beams
from mfem_gb300.batched import BatchedSolver
from oracle import mfem_oracle as O
from fsai_reference import fsai_numpy, lower_pattern

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def make(name, cells, **kw):
    mesh = beams.build_beam(name, cells=cells)
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=kw.pop("iterations", 8), energy=mesh.spec.energy,
                            line_search=False, **kw)
    return mesh, model, solver


def one_solve(mesh, solver):
    q = torch.as_tensor(mesh.q0, device=DEV)
    x = q.clone()
    solver.predict(q, torch.zeros_like(q), mesh.spec.dt)
    solver.update_system(x)
    solver.assemble(x, mesh.spec.dt)
    solver.global_solve(0)
    torch.cuda.synchronize()
    return solver.solve_stats()[0]


def read_system(solver, n):
    rp = solver.read_buffer("row_ptr").cpu().numpy()
    ci = solver.read_buffer("col_idx").cpu().numpy()
    vals = solver.read_buffer("h_values").cpu().numpy().astype(np.float64).reshape(-1, 3, 3)
    G = solver.read_buffer("precond_factor").cpu().numpy().astype(np.float64).reshape(-1, 3, 3)
    return rp, ci, vals, G


@pytest.mark.parametrize("name,cells", [("nh_beam", (16, 4, 4)), ("stiff_beam", (12, 4, 4))])
def test_factor_matches_float64_fsai(name, cells):
    mesh, _, solver = make(name, cells, preconditioner="fsai")
    assert solver.pcg_layout()["variant"] == "factor"
    st = one_solve(mesh, solver)
    assert st["status"] == _lib.MFEM_OK, st
    rp, ci, vals, G = read_system(solver, mesh.n)
    ref, fallback = fsai_numpy(rp, ci, vals)
    assert not fallback
    lrow, lcol, _ = lower_pattern(rp, ci)
    assert G.shape == ref.shape
    for i in range(mesh.n):
        blk = slice(lrow[i], lrow[i + 1])
        scale = np.abs(ref[blk]).max()
        err = np.abs(G[blk] - ref[blk]).max()
        assert err <= 1e-3 * scale, f"row {i}: {err:.3e} vs {scale:.3e}"
    # diag(G H G^T) = I
    n3 = 3 * mesh.n
    Hs = sp.bsr_matrix((vals, ci, rp), shape=(n3, n3)).tocsr()
    Gs = sp.bsr_matrix((G, lcol, lrow), shape=(n3, n3)).tocsr()
    D = (Gs @ Hs @ Gs.T).toarray()
    for i in range(mesh.n):
        np.testing.assert_allclose(D[3 * i:3 * i + 3, 3 * i:3 * i + 3], np.eye(3), atol=1e-3)


@pytest.mark.parametrize("name,cells", [("nh_beam", (16, 4, 4)), ("stiff_beam", (12, 4, 4))])
def test_fewer_iterations_than_block_jacobi(name, cells):
    its = {}
    for pc in ("block_jacobi", "fsai"):
        mesh, _, solver = make(name, cells, preconditioner=pc)
        st = one_solve(mesh, solver)
        assert st["status"] == _lib.MFEM_OK, (pc, st)
        its[pc] = st["iterations"]
    assert 0 < its["fsai"] < its["block_jacobi"], its


@pytest.mark.parametrize("variant", ["factor", "global_memory"])
def test_trajectory_matches_fp64_oracle(variant):
    mesh, model, solver = make("nh_beam", (16, 4, 4), preconditioner="fsai", pcg_variant=variant)
    assert solver.pcg_layout()["variant"] == variant
    ref = O.OracleSolver(mesh, dtype=np.float64)
    A, B = model.state(), model.state()
    A.particle_q.copy_(torch.as_tensor(mesh.q0, device=DEV))
    q, qd = mesh.q0, mesh.qd0
    for _ in range(3):
        solver.step(A, B, None, None, mesh.spec.dt)
        A, B = B, A
        q, qd = ref.step(q, qd, mesh.spec.dt)
        assert all(s["status"] == _lib.MFEM_OK for s in solver.solve_stats())
        got = A.particle_q.cpu().numpy().astype(np.float64)
        assert np.abs(got - q).max() <= 1e-5 * np.abs(q).max()


def test_batched_bodies_with_fsai_match_the_oracle():
    batch = beams.batched_bodies(6, seed=5, nx=(2, 7), nyz=(1, 3))
    bs = BatchedSolver(batch, device=DEV, preconditioner="fsai")
    A, B = bs.state(), bs.model.state()
    for _ in range(2):
        bs.step(A, B)
        A, B = B, A
        assert (bs.body_stats()["status"] == _lib.MFEM_OK).all()
    q = A.particle_q.cpu().numpy()
    for k, m in enumerate(batch.bodies):
        S = O.OracleSolver(m, dtype=np.float64)
        qq, vv = m.q0, m.qd0
        for _ in range(2):
            qq, vv = S.step(qq, vv, m.spec.dt)
        got = q[batch.vertex_offsets[k]:batch.vertex_offsets[k + 1]]
        assert np.abs(got - qq).max() <= 1e-5 * np.abs(qq).max(), k


def test_graph_and_eager_agree_bitwise():
    outs = []
    for graph in (True, False):
        mesh, model, solver = make("nh_beam", (16, 4, 4), preconditioner="fsai", use_cuda_graph=graph)
        A, B = model.state(), model.state()
        for _ in range(2):
            solver.step(A, B, None, None, mesh.spec.dt)
            A, B = B, A
        outs.append(A.particle_q.clone())
    assert torch.equal(outs[0], outs[1])


def test_bad_combinations_are_refused():
    mesh = beams.build_beam("cantilever", cells=(2, 1, 1))
    model = Model.from_beam(mesh, device=DEV)
    with pytest.raises(ValueError):
        MixedFEMSolver(model, iterations=1, preconditioner="ilu")
    with pytest.raises(_lib.MfemError):
        MixedFEMSolver(model, iterations=1, preconditioner="fsai", pcg_variant="standard")
    with pytest.raises(_lib.MfemError):
        MixedFEMSolver(model, iterations=1, preconditioner="block_jacobi", pcg_variant="factor")


@pytest.mark.parametrize("pc", ["fsai", "learned"])
@pytest.mark.parametrize("name,cells", [("nh_beam", (16, 4, 4)), ("stiff_beam", (12, 4, 4))])
def test_persistent_and_global_memory_pcg_agree(pc, name, cells):
    """The same system through both factor PCGs: the iterates are equal in
    exact arithmetic; the float32 sums run in different orders."""
    out = {}
    for variant in ("factor", "global_memory"):
        mesh, _, solver = make(name, cells, preconditioner=pc, pcg_variant=variant)
        assert solver.pcg_layout()["variant"] == variant
        st = one_solve(mesh, solver)
        assert st["status"] == _lib.MFEM_OK and st["iterations"] > 0, (variant, st)
        out[variant] = (st, solver.read_buffer("dx").cpu().numpy().astype(np.float64))
    (sa, da), (sb, db) = out["factor"], out["global_memory"]
    assert abs(sa["iterations"] - sb["iterations"]) <= max(2, sb["iterations"] // 50), (sa, sb)
    assert np.abs(da - db).max() <= 1e-4 * np.abs(db).max()


@pytest.mark.parametrize("pc", ["fsai", "learned"])
def test_persistent_factor_pcg_with_global_factor_rows(pc):
    """nh_beam on 40 CTAs: 470 rows a CTA leave room in shared memory for the
    factor's row pointers only (columns and blocks through L2); the solve
    agrees with the global-memory PCG's."""
    out = {}
    for variant in ("factor", "global_memory"):
        mesh, _, solver = make("nh_beam", None, preconditioner=pc, pcg_variant=variant, pcg_ctas=40)
        lay = solver.pcg_layout()
        assert lay["variant"] == variant
        if variant == "factor":
            assert not lay["cache_matrix"] and lay["smem_bytes"] < 160 * 1024, lay
        st = one_solve(mesh, solver)
        assert st["status"] == _lib.MFEM_OK and st["iterations"] > 0, (variant, st)
        out[variant] = (st, solver.read_buffer("dx").cpu().numpy().astype(np.float64))
    (sa, da), (sb, db) = out["factor"], out["global_memory"]
    assert abs(sa["iterations"] - sb["iterations"]) <= max(2, sb["iterations"] // 50), (sa, sb)
    assert np.abs(da - db).max() <= 1e-4 * np.abs(db).max()


def test_mesh_too_large_for_the_persistent_factor_pcg():
    """One CTA cannot hold nh_beam's rows: auto falls back to the
    global-memory PCG, an explicit "factor" is refused."""
    mesh = beams.build_beam("nh_beam", cells=(64, 16, 16))
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=1, preconditioner="fsai", pcg_ctas=1)
    assert solver.pcg_layout()["variant"] == "global_memory"
    with pytest.raises(_lib.MfemError):
        MixedFEMSolver(model, iterations=1, preconditioner="fsai", pcg_ctas=1, pcg_variant="factor")


@pytest.mark.parametrize("variant", ["factor", "global_memory"])
def test_step_stats_report_the_factor_solve(variant):
    """mfem_step_stats of a one-body factor plan is the body's record."""
    mesh, _, solver = make("nh_beam", (16, 4, 4), preconditioner="fsai", pcg_variant=variant)
    st = one_solve(mesh, solver)
    assert st["status"] == _lib.MFEM_OK and st["iterations"] > 0 and 0.0 < st["rel_residual"] <= 1e-6, st


@pytest.mark.parametrize("pc", ["fsai", "learned"])
def test_lagged_factor_matches_the_oracle(pc):
    """factor_refresh=8: one factor per step, reused by its eight solves."""
    mesh, model, solver = make("nh_beam", (16, 4, 4), preconditioner=pc, factor_refresh=8)
    ref = O.OracleSolver(mesh, dtype=np.float64)
    A, B = model.state(), model.state()
    A.particle_q.copy_(torch.as_tensor(mesh.q0, device=DEV))
    q, qd = mesh.q0, mesh.qd0
    for _ in range(2):
        solver.step(A, B, None, None, mesh.spec.dt)
        A, B = B, A
        q, qd = ref.step(q, qd, mesh.spec.dt)
        assert all(s["status"] == _lib.MFEM_OK and s["iterations"] > 0 for s in solver.solve_stats())
        got = A.particle_q.cpu().numpy().astype(np.float64)
        assert np.abs(got - q).max() <= 1e-5 * np.abs(q).max()
    with pytest.raises(_lib.MfemError):
        make("nh_beam", (4, 2, 2), preconditioner=pc, factor_refresh=-1)
