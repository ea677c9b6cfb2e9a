"""GPU: the solver on meshes whose vertex order is not banded.

A shuffled vertex order makes the per-CTA column windows span the mesh; the
plan must then fall back to the gather PCG and still give the same step.
Reverse Cuthill-McKee restores a band and the window-based PCG."""
import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, beams, reorder

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _model(mesh, order=None):
    arrays = (mesh.rest_q, mesh.q0, mesh.particle_mass, mesh.particle_inv_mass)
    tets = mesh.tet_indices
    if order is not None:
        tets, *arrays = reorder.permute_vertices(order, tets, *arrays)
    rest, q0, mass, inv_mass = arrays
    model = Model(rest, np.zeros_like(rest), mass, inv_mass, tets, mesh.tet_poses, mesh.tet_materials,
                  mesh.gravity, device=DEV)
    return model, q0


def _one_step(mesh, order=None, **kw):
    model, q0 = _model(mesh, order)
    solver = MixedFEMSolver(model, iterations=8, energy=mesh.spec.energy, line_search=False, **kw)
    s0, s1 = model.state(), model.state()
    s0.particle_q.copy_(torch.as_tensor(q0, device=DEV))
    solver.step(s0, s1, None, None, mesh.spec.dt)
    assert all(st["status"] == 0 for st in solver.solve_stats())
    q = s1.particle_q.cpu().numpy()
    if order is not None:
        back = np.empty_like(q)
        back[order] = q
        q = back
    return q, solver.pcg_layout()


def _close(a, b, rtol):
    assert np.abs(a - b).max() <= rtol * np.abs(b).max()


def test_shuffled_vertex_order_falls_back_to_gather_and_agrees():
    mesh = beams.build_beam("nh_beam")
    q_ref, lay_ref = _one_step(mesh)
    assert lay_ref["variant"] == "single_reduction" and lay_ref["cache_matrix"]
    shuffle = np.random.default_rng(1).permutation(mesh.n)
    q, lay = _one_step(mesh, shuffle)
    assert lay["variant"] == "gather", lay
    _close(q, q_ref, 1e-5)
    rcm = reorder.rcm_order(reorder.permute_vertices(shuffle, mesh.tet_indices)[0], mesh.n)
    order = shuffle[rcm]
    q2, lay2 = _one_step(mesh, order)
    assert lay2["variant"] == "single_reduction", lay2
    _close(q2, q_ref, 1e-5)


@pytest.mark.parametrize("variant", ["gather", "standard"])
def test_forced_variants_agree_with_default(variant):
    mesh = beams.build_beam("cantilever")
    q_ref, _ = _one_step(mesh)
    q, lay = _one_step(mesh, pcg_variant=variant)
    assert lay["variant"] == variant
    _close(q, q_ref, 1e-5)
