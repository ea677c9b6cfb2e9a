"""Meshes and inputs shared by the refinement tests (CPU and GPU)."""
from __future__ import annotations

import numpy as np

from mfem_gb300 import beams
from mfem_gb300.refinement_model import soft_grid
from oracle import refine_oracle as ro


def grid_mesh(dims=(3, 2, 2), cell=0.2, mu=10.0, lam=1.0, density=1.0, pin_first=True, seed=0):
    """The reference test's soft grid (tests/test_refinement.py:29-45: 3 x 2 x 2
    cells of 0.2 m, 5 tets a cell, mu 10, lambda 1, density 1, vertex 0
    kinematic), lumped masses density * volume / 4."""
    x, tets, mats = soft_grid(*dims, cell, cell, cell, mu, lam, 0.0)
    return mesh_from(x, tets, mats, density, pinned=[0] if pin_first else [], seed=seed)


def mesh_from(x, tets, mats, density, pinned=(), seed=0):
    x = np.asarray(x, dtype=np.float32)
    tets = np.asarray(tets, dtype=np.int32)
    Dm = ro.edge_matrix(x, tets.astype(np.int64))
    poses = ro.inverse3_f32(Dm)
    vol = np.linalg.det(Dm.astype(np.float64)) / 6.0
    n, T = x.shape[0], tets.shape[0]
    mass = np.zeros(n, dtype=np.float64)
    np.add.at(mass, tets.ravel().astype(np.int64), np.repeat(density * vol / 4.0, 4))
    mass = mass.astype(np.float32)
    inv = np.where(mass > 0, 1.0 / np.maximum(mass, 1e-30), 0.0).astype(np.float32)
    inv[list(pinned)] = 0.0
    rng = np.random.default_rng(seed)
    s = np.tile(np.array([1, 1, 1, 0, 0, 0], np.float32), (T, 1)) + rng.normal(0, 1e-2, (T, 6)).astype(np.float32)
    lam = rng.normal(0, 1.0, (T, 6)).astype(np.float32)
    return ro.Mesh(x, tets, poses, np.asarray(mats, dtype=np.float32), s, lam, mass, inv,
                   np.zeros((0, 3), dtype=np.int32))


def beam_mesh(name="nh_beam", cells=None, seed=0):
    mesh = beams.build_beam(name, cells=cells) if cells else beams.build_beam(name)
    m = mesh_from(mesh.rest_q, mesh.tet_indices, mesh.tet_materials, 1000.0, seed=seed)
    m.mass = mesh.particle_mass.astype(np.float32)
    m.inv_mass = mesh.particle_inv_mass.astype(np.float32)
    m.poses = mesh.tet_poses.astype(np.float32).reshape(-1, 3, 3)
    return m, mesh


def deformed(x, seed=1, amp=0.02):
    rng = np.random.default_rng(seed)
    return (x + rng.normal(0.0, amp, x.shape)).astype(np.float32)


def hanging_edges(tets_new, selected_pairs):
    """Tets of the refined mesh that still hold both ends of a split edge."""
    pairs = set(selected_pairs)
    bad = 0
    for t in np.asarray(tets_new):
        for i in range(4):
            for j in range(i):
                a, b = sorted((int(t[i]), int(t[j])))
                if (a, b) in pairs:
                    bad += 1
    return bad
