"""CPU checks of the C ABI: the library builds and loads, exports every
function include/mfem_gb300.h declares, and its host-side symbolic analysis
(no GPU involved) matches the oracle bit for bit."""
import ctypes

import numpy as np
import pytest

from mfem_gb300 import _lib, beams
from oracle import mfem_oracle as O


def test_every_declared_function_is_exported(built_lib):
    names = _lib.header_functions()
    assert "mfem_step" in names and "mfem_plan_create" in names
    missing = [n for n in names if not hasattr(built_lib, n)]
    assert not missing, missing
    # the ctypes signatures cover the whole header
    assert set(names) <= set(_lib._SIGNATURES)


def test_default_config_matches_reference_defaults(built_lib):
    cfg = _lib.default_config()
    assert cfg.iterations == 8
    assert cfg.energy == 0
    assert cfg.cg_max_iterations == 1000
    assert cfg.cg_tolerance == pytest.approx(1e-6)
    assert cfg.attachment_stiffness == pytest.approx(10.0)
    assert cfg.preconditioner_singular_threshold == pytest.approx(1e-20)
    assert cfg.preconditioner == 1
    # line search on by default (solver.py:99-103, 185)
    assert cfg.line_search == 1
    assert cfg.line_search_max_iterations == 20
    assert cfg.line_search_alpha0 == 1.0 and cfg.line_search_tau == 0.5
    assert cfg.line_search_c == pytest.approx(0.01)
    assert cfg.line_search_threshold == pytest.approx(1e-8)
    assert ctypes.sizeof(_lib.MfemConfig) == 64
    assert ctypes.sizeof(_lib.MfemSolveStats) == 16
    assert ctypes.sizeof(_lib.MfemLineSearchStats) == 40


def test_status_strings(built_lib):
    for code in range(7):
        assert _lib.status_string(code)
    assert "unknown" in _lib.status_string(99)


def _host_sparsity(lib, tets, n):
    tets = np.ascontiguousarray(tets, dtype=np.int32)
    nnzb = ctypes.c_int64()
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.mfem_bsr_sparsity(n, tets.shape[0], P(tets), None, None, ctypes.byref(nnzb)) == 0
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(nnzb.value, np.int32)
    assert lib.mfem_bsr_sparsity(n, tets.shape[0], P(tets), P(rp), P(ci), ctypes.byref(nnzb)) == 0
    slots = np.zeros((tets.shape[0], 16), np.int32)
    assert lib.mfem_tet_slot_map(n, tets.shape[0], P(tets), P(rp), P(ci), P(slots)) == 0
    return rp, ci, slots


@pytest.mark.parametrize("name", ["cantilever", "nh_beam"])
def test_host_sparsity_and_slot_map_bit_exact(built_lib, name):
    m = beams.build_beam(name)
    rp, ci, slots = _host_sparsity(built_lib, m.tet_indices, m.n)
    rp_o, ci_o = O.bsr_sparsity(m.tet_indices, m.n)
    np.testing.assert_array_equal(rp, rp_o)
    np.testing.assert_array_equal(ci, ci_o)
    np.testing.assert_array_equal(slots, O.tet_slot_map(m.tet_indices, rp_o, ci_o))


def test_host_sparsity_with_isolated_vertex_and_shuffled_tets(built_lib):
    rng = np.random.default_rng(5)
    m = beams.build_beam("cantilever", cells=(3, 2, 1))
    tets = m.tet_indices[rng.permutation(m.T)]
    tets = np.ascontiguousarray(tets[:, rng.permutation(4)])
    n = m.n + 1  # one vertex in no tet
    rp, ci, slots = _host_sparsity(built_lib, tets, n)
    rp_o, ci_o = O.bsr_sparsity(tets, n)
    np.testing.assert_array_equal(rp, rp_o)
    np.testing.assert_array_equal(ci, ci_o)
    np.testing.assert_array_equal(slots, O.tet_slot_map(tets, rp_o, ci_o))
    assert rp[-1] - rp[-2] == 1 and ci[-1] == n - 1


def test_host_sparsity_of_a_refined_mesh(built_lib):
    """An irregular mesh: the reference test's grid after three refinement
    passes of the oracle (vertices of valence 4 to 30)."""
    from oracle import refine_oracle as ro
    from tests.refine_cases import deformed, grid_mesh
    mesh = grid_mesh()
    q = deformed(mesh.rest_q)
    cfg = ro.RefineConfig(scoring="legacy", threshold=1e-6, tet_score_weight=1.0)
    rng = np.random.default_rng(8)
    for _ in range(3):
        E = rng.uniform(0.0, 1.0, mesh.tets.shape[0]).astype(np.float32)
        res = ro.refine_pass(mesh, q, q, cfg, tet_scores=E, max_particles=10 ** 6, max_tets=10 ** 6)
        mesh, q = res.mesh, res.q
    n = mesh.rest_q.shape[0]
    rp, ci, slots = _host_sparsity(built_lib, mesh.tets, n)
    rp_o, ci_o = O.bsr_sparsity(mesh.tets, n)
    np.testing.assert_array_equal(rp, rp_o)
    np.testing.assert_array_equal(ci, ci_o)
    np.testing.assert_array_equal(slots, O.tet_slot_map(mesh.tets, rp_o, ci_o))


@pytest.mark.parametrize("bad", ["out_of_range", "negative", "repeated"])
def test_host_sparsity_rejects_bad_meshes(built_lib, bad):
    tets = np.array([[0, 1, 2, 3]], dtype=np.int32)
    if bad == "out_of_range":
        tets[0, 3] = 4
    elif bad == "negative":
        tets[0, 0] = -1
    else:
        tets[0, 2] = 1
    nnzb = ctypes.c_int64()
    rc = built_lib.mfem_bsr_sparsity(4, 1, tets.ctypes.data_as(ctypes.c_void_p), None, None, ctypes.byref(nnzb))
    assert rc == _lib.MFEM_BAD_ARG
    assert built_lib.mfem_plan_last_error(None).decode()


def test_plan_create_rejects_bad_config(built_lib):
    m = beams.build_beam("cantilever", cells=(1, 1, 1))
    cfg = _lib.default_config()
    cfg.energy = 7
    P = lambda a: np.ascontiguousarray(a).ctypes.data_as(ctypes.c_void_p)
    plan = ctypes.c_void_p()
    rc = built_lib.mfem_plan_create(ctypes.byref(cfg), m.n, m.T, P(m.tet_indices), P(m.tet_poses),
                                    P(m.tet_materials), P(m.rest_q), P(m.particle_mass),
                                    P(m.particle_inv_mass), P(m.gravity), 0, ctypes.byref(plan))
    assert rc == _lib.MFEM_BAD_ARG and not plan.value
    assert "energy" in built_lib.mfem_plan_last_error(None).decode()


def test_solver_fails_loudly_without_library(tmp_path, monkeypatch):
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError):
        _lib.load(tmp_path / "missing.so")
