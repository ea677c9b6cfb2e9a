"""CPU checks of the npz model format and the 5-tet soft-grid generator."""
import hashlib
import json
import os

import numpy as np
import pytest

from mfem_gb300.refinement_model import MFEMRefinementModel, soft_grid

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _digest(a):
    a = np.ascontiguousarray(a)
    return {"dtype": str(a.dtype), "shape": list(a.shape), "sha256": hashlib.sha256(a.tobytes()).hexdigest()}


def test_soft_grid_reproduces_reference_fem_beam_bit_for_bit():
    """The reference builds fem_beam.npz with Newton's add_soft_grid(8, 4, 4,
    cell 1, k_mu 6, k_lambda 1, k_damp 0) (src/mfem/refinement/models/
    make_fem_beam_example.py:8-29); the generator must give the same arrays,
    checked through their sha256 digests."""
    ref = json.load(open(os.path.join(GOLDEN, "reference_fixture_digests.json")))["fem_beam.npz"]
    p, t, m = soft_grid(8, 4, 4, 1.0, 1.0, 1.0, k_mu=6.0, k_lambda=1.0, k_damp=0.0)
    assert _digest(p) == ref["particles"]
    assert _digest(t) == ref["tet_indices"]
    assert _digest(m) == ref["tet_materials"]


def test_soft_grid_tets_are_positive_and_fill_the_box():
    p, t, _ = soft_grid(5, 3, 2, 0.5, 0.25, 0.5)
    x = p.astype(np.float64)[t]
    vol = np.linalg.det(np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], axis=2)) / 6
    assert np.all(vol > 0)
    np.testing.assert_allclose(vol.sum(), 2.5 * 0.75 * 1.0)


def test_npz_round_trip_and_sim_arrays(tmp_path):
    p, t, m = soft_grid(4, 2, 2, k_mu=6.0, k_lambda=1.0)
    model = MFEMRefinementModel.from_arrays(p, t, m, max_particles=4 * p.shape[0], max_tets=8 * t.shape[0],
                                            density=2.0)
    path = str(tmp_path / "beam.npz")
    model.save(path)
    back = MFEMRefinementModel.load(path)
    np.testing.assert_array_equal(back.particles, p)
    np.testing.assert_array_equal(back.tet_indices, t)
    assert back.max_particles == 4 * p.shape[0] and back.max_tets == 8 * t.shape[0]
    assert back.density == 2.0 and back.max_tris == 0
    x, tets, dminv, mats, mass, inv_mass = back.sim_arrays(mu=10.0)
    # rotated 90 degrees about x: (x, y, z) -> (x, -z, y)
    np.testing.assert_allclose(x, np.stack([p[:, 0], -p[:, 2], p[:, 1]], axis=1), atol=1e-6)
    assert np.all(mats[:, 0] == 10.0) and np.all(mats[:, 1] == 1.0)
    np.testing.assert_allclose(mass.sum(), 2.0 * 4 * 2 * 2, rtol=1e-6)
    np.testing.assert_allclose(inv_mass * mass, 1.0, rtol=1e-6)
    vol = 1.0 / (6.0 * np.linalg.det(dminv.astype(np.float64)))
    assert np.all(vol > 0)
