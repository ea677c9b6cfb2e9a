"""GPU: models in the reference's npz format through the solver.

The reference's fem_beam layout (Newton's 5-tet soft grid, 8x4x4 cells,
mu 6, lambda 1) saved as npz, loaded with load_sim_model (rotated 90 degrees
about x, mu overridden) and stepped, against the float64 oracle."""
import dataclasses

import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, beams
from mfem_gb300.refinement_model import MFEMRefinementModel, soft_grid
from oracle import mfem_oracle as O

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _fem_beam_mesh(tmp_path, mu, energy):
    p, t, m = soft_grid(8, 4, 4, 1.0, 1.0, 1.0, k_mu=6.0, k_lambda=1.0, k_damp=0.0)
    path = str(tmp_path / "fem_beam.npz")
    MFEMRefinementModel.from_arrays(p, t, m, max_particles=3600, max_tets=20480, density=1.0).save(path)
    model_file = MFEMRefinementModel.load(path)
    x, tets, dminv, mats, mass, inv_mass = model_file.sim_arrays(mu=mu)
    pinned = x[:, 0] <= x[:, 0].min() + 1e-6
    inv_mass = np.where(pinned, 0.0, inv_mass).astype(np.float32)
    spec = dataclasses.replace(beams.CONFIGS["cantilever"], name="fem_beam", energy=energy, dt=1.0 / 60.0)
    return beams.BeamMesh(spec=spec, rest_q=x, q0=x.copy(), qd0=np.zeros_like(x), tet_indices=tets,
                          tet_poses=dminv, tet_materials=mats, particle_mass=mass, particle_inv_mass=inv_mass,
                          gravity=np.array([0.0, -9.81, 0.0], dtype=np.float32))


@pytest.mark.parametrize("energy", ["arap", "neohookean"])
def test_fem_beam_npz_model_steps_match_oracle(tmp_path, energy):
    mesh = _fem_beam_mesh(tmp_path, mu=100.0, energy=energy)
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=8, energy=energy, line_search=False)
    ref = O.OracleSolver(mesh, dtype=np.float64)
    s0, s1 = model.state(), model.state()
    q, qd = mesh.q0, mesh.qd0
    for _ in range(5):
        solver.step(s0, s1, None, None, mesh.spec.dt)
        q, qd = ref.step(q, qd, mesh.spec.dt)
        assert all(st["status"] == 0 for st in solver.solve_stats())
        got = s1.particle_q.cpu().numpy()
        assert np.abs(got - q).max() <= 1e-5 * np.abs(q).max()
        s0, s1 = s1, s0


@pytest.mark.parametrize("pc", ["fsai", "learned"])
def test_fem_beam_with_factor_preconditioner(tmp_path, pc):
    """The 5-tet grid has rows with 9 and 10 lower blocks: FSAI sets them up
    with the warp kernel (the per-thread kernel takes rows of up to 8).  The
    factor equals a float64 FSAI of the same H, and a trajectory stays within
    1e-5 of the oracle."""
    from fsai_reference import fsai_numpy, lower_pattern
    mesh = _fem_beam_mesh(tmp_path, mu=100.0, energy="neohookean")
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=8, energy="neohookean", line_search=False, preconditioner=pc)
    ref = O.OracleSolver(mesh, dtype=np.float64)
    s0, s1 = model.state(), model.state()
    q, qd = mesh.q0, mesh.qd0
    for _ in range(3):
        solver.step(s0, s1, None, None, mesh.spec.dt)
        q, qd = ref.step(q, qd, mesh.spec.dt)
        assert all(st["status"] == 0 and st["iterations"] > 0 for st in solver.solve_stats())
        got = s1.particle_q.cpu().numpy()
        assert np.abs(got - q).max() <= 1e-5 * np.abs(q).max()
        s0, s1 = s1, s0
    if pc == "fsai":
        rp = solver.read_buffer("row_ptr").cpu().numpy()
        ci = solver.read_buffer("col_idx").cpu().numpy()
        vals = solver.read_buffer("h_values").cpu().numpy().astype(np.float64).reshape(-1, 3, 3)
        G = solver.read_buffer("precond_factor").cpu().numpy().astype(np.float64).reshape(-1, 3, 3)
        lrow, _, _ = lower_pattern(rp, ci)
        assert (np.diff(lrow) > 8).any()
        # the factor of the last assembly (the step's 8th Newton iteration)
        ref_G, fallback = fsai_numpy(rp, ci, vals)
        assert not fallback
        for i in range(mesh.n):
            blk = slice(lrow[i], lrow[i + 1])
            assert np.abs(G[blk] - ref_G[blk]).max() <= 1e-3 * np.abs(ref_G[blk]).max(), i
