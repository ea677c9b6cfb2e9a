"""The batch of uneven bodies (host side, no GPU)."""
import numpy as np

from mfem_gb300 import beams


def test_batch_generator_matches_the_spec():
    b = beams.batched_bodies(40, seed=4)
    assert b.n_bodies == 40
    cells = np.array([m.spec.cells for m in b.bodies])
    assert cells[:, 0].min() >= 4 and cells[:, 0].max() <= 48
    assert cells[:, 1:].min() >= 2 and cells[:, 1:].max() <= 12
    assert set(b.energies) == {"arap", "neohookean"}
    np.testing.assert_allclose(np.linalg.norm(b.gravity, axis=1), 9.81, rtol=1e-6)
    nus = np.array([m.spec.nu for m in b.bodies])
    assert nus.min() >= 0.3 and nus.max() <= 0.48
    for m in b.bodies:
        assert np.all(m.particle_inv_mass[m.rest_q[:, 0] <= 0.0] == 0.0)
        assert np.all(m.particle_inv_mass[m.rest_q[:, 0] > 0.0] > 0.0)
        np.testing.assert_allclose(np.diff(np.unique(m.rest_q[:, 0])), 0.05, rtol=1e-5)


def test_concatenation_keeps_bodies_apart():
    b = beams.batched_bodies(9, seed=1, nx=(2, 5), nyz=(1, 3))
    u = b.union
    assert b.vertex_offsets[-1] == u.n and b.tet_offsets[-1] == u.T
    for k, m in enumerate(b.bodies):
        t = u.tet_indices[b.tet_offsets[k]:b.tet_offsets[k + 1]]
        assert t.min() >= b.vertex_offsets[k] and t.max() < b.vertex_offsets[k + 1]
        np.testing.assert_array_equal(t - b.vertex_offsets[k], m.tet_indices)
        np.testing.assert_array_equal(u.rest_q[b.vertex_offsets[k]:b.vertex_offsets[k + 1]], m.rest_q)
