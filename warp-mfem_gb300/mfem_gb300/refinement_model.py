"""The reference's npz tet-mesh model format and its soft-grid generator.

* ``MFEMRefinementModel`` mirrors ``src/mfem/refinement/models/
  refinement_model.py:13-143``: an npz with ``particles`` [n, 3],
  ``tet_indices`` [T, 4], ``tet_materials`` [T, 3] (mu, lambda, damping) and
  ``parameters`` (max_particles, max_tets, density[, max_tris]);
  ``load_sim_model`` turns it into a ``Model`` the way the reference does
  through Newton's ``add_soft_mesh``: the mesh is rotated by 90 degrees about
  x, ``mu`` overrides the per-tet shear modulus, and each vertex gets the mass
  density * volume / 4 of every incident tet.
* ``soft_grid`` builds the 5-tet-per-hex grid of Newton's
  ``ModelBuilder.add_soft_grid`` (used for the reference's ``fem_beam.npz``,
  ``src/mfem/refinement/models/make_fem_beam_example.py:8-29``): vertices
  x-fastest, then y, then z; cells in the same order; the two mirror-image
  5-tet patterns alternate with the parity of the cell so the faces of
  neighbouring cells match.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

PARAM_MAX_PARTICLES = 0
PARAM_MAX_TETS = 1
PARAM_DENSITY = 2
PARAM_MAX_TRIS = 3

# corner offsets (dx, dy, dz) of the two 5-tet patterns
_EVEN = (((1, 0, 0), (1, 0, 1), (1, 1, 0), (0, 0, 0)),
         ((0, 0, 1), (0, 0, 0), (0, 1, 1), (1, 0, 1)),
         ((0, 1, 0), (0, 1, 1), (0, 0, 0), (1, 1, 0)),
         ((1, 1, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1)),
         ((1, 1, 0), (1, 0, 1), (0, 1, 1), (0, 0, 0)))
_ODD = (((0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)),
        ((1, 0, 1), (0, 0, 1), (1, 1, 1), (1, 0, 0)),
        ((1, 1, 0), (0, 1, 0), (1, 0, 0), (1, 1, 1)),
        ((0, 1, 1), (1, 1, 1), (0, 0, 1), (0, 1, 0)),
        ((0, 1, 0), (1, 0, 0), (1, 1, 1), (0, 0, 1)))


def soft_grid(dim_x: int, dim_y: int, dim_z: int, cell_x: float = 1.0, cell_y: float = 1.0, cell_z: float = 1.0,
              k_mu: float = 1.0, k_lambda: float = 1.0, k_damp: float = 0.0, origin=(0.0, 0.0, 0.0)):
    """(particles [n, 3] f32, tet_indices [5 * cells, 4] i32, tet_materials
    [T, 3] f32) of a dim_x x dim_y x dim_z grid of hex cells, 5 tets each."""
    nx, ny, nz = dim_x + 1, dim_y + 1, dim_z + 1
    zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    particles = np.stack([xx.ravel() * cell_x, yy.ravel() * cell_y, zz.ravel() * cell_z], axis=1)
    particles = (particles + np.asarray(origin, dtype=np.float64)).astype(np.float32)

    def vid(i, j, k):
        return i + nx * (j + ny * k)

    tets = []
    for k in range(dim_z):
        for j in range(dim_y):
            for i in range(dim_x):
                pattern = _ODD if (i + j + k) & 1 else _EVEN
                for tet in pattern:
                    tets.append([vid(i + dx, j + dy, k + dz) for dx, dy, dz in tet])
    tets = np.asarray(tets, dtype=np.int32).reshape(-1, 4)
    materials = np.tile(np.asarray([k_mu, k_lambda, k_damp], dtype=np.float32), (tets.shape[0], 1))
    return particles, tets, materials


def quat_rotation_matrix_euler_x(angle: float) -> np.ndarray:
    c, s = math.cos(angle), math.sin(angle)
    return np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])


@dataclasses.dataclass
class MFEMRefinementModel:
    particles: np.ndarray
    tet_indices: np.ndarray
    tet_materials: np.ndarray
    parameters: np.ndarray

    @classmethod
    def from_arrays(cls, particles, tet_indices, tet_materials, max_particles: int, max_tets: int,
                    density: float = 1.0, max_tris: int = 0) -> "MFEMRefinementModel":
        return cls(np.asarray(particles, dtype=np.float32), np.asarray(tet_indices, dtype=np.int32),
                   np.asarray(tet_materials, dtype=np.float32),
                   np.array([max_particles, max_tets, density, max_tris], dtype=np.float64))

    def save(self, file: str) -> None:
        np.savez(file, particles=self.particles, tet_indices=self.tet_indices, tet_materials=self.tet_materials,
                 parameters=self.parameters)

    @staticmethod
    def load(file: str, scale: float = 1.0, translation: float = 0.0) -> "MFEMRefinementModel":
        d = np.load(file, allow_pickle=True)
        return MFEMRefinementModel(particles=d["particles"] * scale + translation, tet_indices=d["tet_indices"],
                                   tet_materials=d["tet_materials"], parameters=d["parameters"])

    @property
    def max_particles(self) -> int:
        return int(self.parameters[PARAM_MAX_PARTICLES])

    @property
    def max_tets(self) -> int:
        return int(self.parameters[PARAM_MAX_TETS])

    @property
    def max_tris(self) -> int:
        return int(self.parameters[PARAM_MAX_TRIS]) if len(self.parameters) > PARAM_MAX_TRIS else 0

    @property
    def density(self) -> float:
        return float(self.parameters[PARAM_DENSITY])

    def sim_arrays(self, mu: float, rotate: bool = True):
        """Host arrays of the simulation model the reference builds with
        ``load_sim_model`` (refinement_model.py:104-143; unpadded): rest positions, DmInv, materials with `mu`,
        lumped masses and inverse masses."""
        x = np.asarray(self.particles, dtype=np.float64)
        if rotate:
            x = x @ quat_rotation_matrix_euler_x(math.pi / 2.0).T
        tets = np.asarray(self.tet_indices, dtype=np.int64)
        xe = x[tets]
        Dm = np.stack([xe[:, 1] - xe[:, 0], xe[:, 2] - xe[:, 0], xe[:, 3] - xe[:, 0]], axis=2)
        vol = np.linalg.det(Dm) / 6.0
        if np.any(vol <= 0.0):
            raise ValueError("the mesh has inverted or flat tets")
        mass = np.zeros(x.shape[0])
        np.add.at(mass, tets.ravel(), np.repeat(self.density * vol / 4.0, 4))
        with np.errstate(divide="ignore"):
            inv_mass = np.where(mass > 0.0, 1.0 / mass, 0.0)
        materials = np.array(self.tet_materials, dtype=np.float64)
        materials[:, 0] = mu
        return (x.astype(np.float32), tets.astype(np.int32), np.linalg.inv(Dm).astype(np.float32),
                materials.astype(np.float32), mass.astype(np.float32), inv_mass.astype(np.float32))

    def load_sim_model(self, mu: float, gravity=(0.0, -9.81, 0.0), device="cuda:0", rotate: bool = True,
                       max_particles: int | None = None):
        """``max_particles`` pads the particle arrays for refinement
        (refinement_model.py:104-143); None (the default here) leaves them
        unpadded, which is what a solver without refinement wants."""
        from .model import Model
        x, tets, dminv, materials, mass, inv_mass = self.sim_arrays(mu, rotate)
        model = Model(x, np.zeros_like(x), mass, inv_mass, tets, dminv, materials,
                      np.asarray(gravity, dtype=np.float32), device=device)
        return model.pad_particles(max_particles) if max_particles is not None else model
