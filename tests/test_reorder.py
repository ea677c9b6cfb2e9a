"""CPU checks of the vertex reordering helper."""
import numpy as np

from mfem_gb300 import beams, reorder
from oracle import mfem_oracle as O


def test_rcm_restores_a_narrow_band_and_keeps_the_mesh():
    m = beams.build_beam("nh_beam", cells=(16, 4, 4))
    rng = np.random.default_rng(0)
    shuffle = rng.permutation(m.n)
    tets, q = reorder.permute_vertices(shuffle, m.tet_indices, m.rest_q)
    assert reorder.bandwidth(tets) > 5 * reorder.bandwidth(m.tet_indices)
    order = reorder.rcm_order(tets, m.n)
    assert np.array_equal(np.sort(order), np.arange(m.n))
    tets2, q2 = reorder.permute_vertices(order, tets, q)
    assert reorder.bandwidth(tets2) <= 2 * reorder.bandwidth(m.tet_indices)
    # same geometry: every tet keeps its vertices' positions and its volume
    np.testing.assert_array_equal(q2[tets2], m.rest_q[m.tet_indices])
    # same sparsity up to the relabelling
    rp, ci = O.bsr_sparsity(tets2, m.n)
    rp0, ci0 = O.bsr_sparsity(m.tet_indices, m.n)
    assert ci.shape == ci0.shape


def test_permute_vertices_round_trip():
    m = beams.build_beam("cantilever")
    order = np.random.default_rng(3).permutation(m.n)
    tets, q, mass = reorder.permute_vertices(order, m.tet_indices, m.rest_q, m.particle_mass)
    inverse = np.empty_like(order)
    inverse[order] = np.arange(m.n)
    back, qb, mb = reorder.permute_vertices(inverse, tets, q, mass)
    np.testing.assert_array_equal(back, m.tet_indices)
    np.testing.assert_array_equal(qb, m.rest_q)
    np.testing.assert_array_equal(mb, m.particle_mass)
