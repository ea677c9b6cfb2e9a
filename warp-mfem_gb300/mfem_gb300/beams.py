"""Synthetic tetrahedral beams: the workloads the global step is measured on.

A beam is an ``nx x ny x nz`` grid of hexahedral cells, each split into six
tetrahedra that share the cell's main diagonal (the Kuhn / Freudenthal split).
Vertices are numbered x-major (``i * (ny+1) * (nz+1) + j * (nz+1) + k``), so a
vertex's neighbours sit within ``(ny+1)(nz+1)`` rows of it: the BSR system has a
narrow band and the PCG's gathers stay local.

Conventions follow the reference's model data:

* ``tet_poses`` holds ``DmInv = inv([x1-x0, x2-x0, x3-x0])`` with the edges as
  COLUMNS, the convention ``compute_constraints`` uses
  (src/mfem/refinement/kernels.py:151-156).  Every tet has a positive volume
  ``1 / (6 det DmInv)`` (src/mfem/refinement/elastic_energy.py:143-145).
* ``tet_materials`` rows are ``(mu, lambda, damping)``
  (src/mfem/refinement/additional_state.py:150), Lame parameters from
  ``E, nu`` as in src/mfem/refinement/sim_octopus.py:327-332.
* lumped mass ``rho * vol / 4`` per incident tet, as the legacy
  ``precompute_mass_matrix`` (src/mfem/kernels.py:39-75) does.
* pinned vertices (the ``x == 0`` face) get ``inv_mass = 0`` and keep their
  mass, like the reference's fixture (tests/test_refinement.py:58-60); the
  solver attaches them with a penalty spring
  (src/mfem/refinement/solver.py:390-393).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Optional

import numpy as np

# The six Kuhn tetrahedra of a unit cell: each is the monotone lattice path
# v000 -> v000+e_a -> v000+e_a+e_b -> v111 for one permutation (a, b, c) of
# the axes.  det[e_a, e_a+e_b, e_a+e_b+e_c] = sign(a, b, c), so the odd
# permutations get their last two vertices swapped to keep every volume > 0.
_PERMS = ((0, 1, 2), (1, 2, 0), (2, 0, 1), (0, 2, 1), (2, 1, 0), (1, 0, 2))


def _kuhn_cell_tets() -> np.ndarray:
    tets = []
    for perm_idx, (a, b, _c) in enumerate(_PERMS):
        p0 = np.zeros(3, dtype=np.int64)
        p1 = p0.copy()
        p1[a] = 1
        p2 = p1.copy()
        p2[b] = 1
        p3 = np.ones(3, dtype=np.int64)
        corners = [p0, p1, p2, p3]
        if perm_idx >= 3:  # odd permutation: swap to make det > 0
            corners[2], corners[3] = corners[3], corners[2]
        tets.append(np.stack(corners))
    return np.stack(tets)  # [6, 4, 3] corner offsets


def lame(E, nu):
    """Lame parameters from Young's modulus and Poisson ratio
    (src/mfem/refinement/sim_octopus.py:327-332)."""
    E = np.asarray(E, dtype=np.float64)
    mu = E / (2.0 * (1.0 + nu))
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    return mu, lam


@dataclasses.dataclass
class BeamSpec:
    """One synthetic beam workload (mesh, material, initial state, run)."""

    name: str
    cells: tuple[int, int, int]
    extent: tuple[float, float, float]
    energy: str                      # "arap" | "neohookean"
    E: tuple[float, float]           # (lo, hi): equal -> constant, else log-uniform per tet
    nu: float
    density: float = 1000.0
    gravity: tuple[float, float, float] = (0.0, -9.81, 0.0)
    dt: float = 1.0 / 60.0
    steps: int = 100
    iterations: int = 8              # local/global (Newton) iterations per step
    noise: float = 0.0               # std of the N(0, noise) perturbation of free vertices
    seed: int = 0
    cg_tolerance: float = 1.0e-6
    cg_max_iterations: int = 1000


# The workloads of the global step.  "cantilever" is the CPU-runnable plain
# ARAP case; "nh_beam" is the Neo-Hookean beam at scale that the step rate is
# quoted on; "stiff_beam" is the large ill-conditioned mesh.
CONFIGS = {
    "cantilever": BeamSpec(
        name="cantilever", cells=(10, 2, 2), extent=(1.0, 0.2, 0.2), energy="arap",
        E=(1.0e5, 1.0e5), nu=0.4, steps=100, seed=1),
    "nh_beam": BeamSpec(
        name="nh_beam", cells=(64, 16, 16), extent=(2.0, 0.5, 0.5), energy="neohookean",
        E=(1.0e4, 1.0e6), nu=0.45, steps=50, noise=1.0e-3, seed=2),
    "stiff_beam": BeamSpec(
        name="stiff_beam", cells=(128, 32, 32), extent=(4.0, 1.0, 1.0), energy="neohookean",
        E=(1.0e4, 1.0e7), nu=0.45, steps=10, seed=3),
}


@dataclasses.dataclass
class BeamMesh:
    """Host-side (numpy) model data of one beam, fp32 like the reference."""

    spec: BeamSpec
    rest_q: np.ndarray          # [n, 3] f32 rest positions (model.particle_q)
    q0: np.ndarray              # [n, 3] f32 initial positions (state_0.particle_q)
    qd0: np.ndarray             # [n, 3] f32 initial velocities
    tet_indices: np.ndarray     # [T, 4] i32
    tet_poses: np.ndarray       # [T, 3, 3] f32 DmInv
    tet_materials: np.ndarray   # [T, 3] f32 (mu, lambda, damping)
    particle_mass: np.ndarray   # [n] f32
    particle_inv_mass: np.ndarray  # [n] f32 (0 on pinned vertices)
    gravity: np.ndarray         # [3] f32

    @property
    def n(self) -> int:
        return int(self.rest_q.shape[0])

    @property
    def T(self) -> int:
        return int(self.tet_indices.shape[0])


def grid_vertices(cells, extent):
    nx, ny, nz = cells
    xs = np.linspace(0.0, extent[0], nx + 1)
    ys = np.linspace(0.0, extent[1], ny + 1)
    zs = np.linspace(0.0, extent[2], nz + 1)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def kuhn_tets(cells) -> np.ndarray:
    """[6 * nx*ny*nz, 4] int32 tets of the 6-tet split, cell-major order."""
    nx, ny, nz = cells
    offs = _kuhn_cell_tets()  # [6, 4, 3]
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = np.stack([I.ravel(), J.ravel(), K.ravel()], axis=1)  # [C, 3]
    corner = base[:, None, None, :] + offs[None, :, :, :]        # [C, 6, 4, 3]
    vid = corner[..., 0] * ((ny + 1) * (nz + 1)) + corner[..., 1] * (nz + 1) + corner[..., 2]
    return vid.reshape(-1, 4).astype(np.int32)


def rest_inverse_poses(rest_q: np.ndarray, tets: np.ndarray) -> np.ndarray:
    x = rest_q.astype(np.float64)[tets]                      # [T, 4, 3]
    Dm = np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], axis=2)  # edges as columns
    return np.linalg.inv(Dm)


def build_beam(spec: BeamSpec | str, cells: Optional[tuple[int, int, int]] = None) -> BeamMesh:
    """Builds the beam of ``spec`` (optionally with a different cell count,
    for small parity cases of the same workload)."""
    if isinstance(spec, str):
        spec = CONFIGS[spec]
    if cells is not None:
        scale = [c / c0 for c, c0 in zip(cells, spec.cells)]
        spec = dataclasses.replace(
            spec, cells=tuple(cells), extent=tuple(e * s for e, s in zip(spec.extent, scale)))
    rest = grid_vertices(spec.cells, spec.extent)
    tets = kuhn_tets(spec.cells)
    dminv = rest_inverse_poses(rest, tets)
    vol = 1.0 / (6.0 * np.linalg.det(dminv))
    if not np.all(vol > 0.0):
        raise AssertionError("Kuhn split produced a non-positive volume")
    T, n = tets.shape[0], rest.shape[0]

    rng = np.random.default_rng(spec.seed)
    lo, hi = spec.E
    if lo == hi:
        E = np.full(T, lo)
    else:
        E = np.exp(rng.uniform(math.log(lo), math.log(hi), size=T))
    mu, lam = lame(E, spec.nu)
    materials = np.stack([mu, lam, np.zeros(T)], axis=1)

    mass = np.zeros(n)
    np.add.at(mass, tets.ravel(), np.repeat(spec.density * vol / 4.0, 4))
    pinned = rest[:, 0] <= 0.0
    inv_mass = np.where(pinned, 0.0, 1.0 / mass)

    q0 = rest.copy()
    if spec.noise > 0.0:
        noise = rng.normal(0.0, spec.noise, size=(n, 3))
        noise[pinned] = 0.0
        q0 = q0 + noise

    f32 = np.float32
    return BeamMesh(
        spec=spec,
        rest_q=rest.astype(f32),
        q0=q0.astype(f32),
        qd0=np.zeros((n, 3), dtype=f32),
        tet_indices=tets.astype(np.int32),
        tet_poses=dminv.astype(f32),
        tet_materials=materials.astype(f32),
        particle_mass=mass.astype(f32),
        particle_inv_mass=inv_mass.astype(f32),
        gravity=np.asarray(spec.gravity, dtype=f32),
    )


@dataclasses.dataclass
class BodyBatch:
    """Independent bodies concatenated into one mesh (vertices and tets of
    body b contiguous), plus each body's own mesh for per-body checks."""

    bodies: list                # [BeamMesh] per body
    union: BeamMesh             # the concatenated mesh (tets renumbered)
    vertex_offsets: np.ndarray  # [B+1] int32
    tet_offsets: np.ndarray     # [B+1] int32
    energies: list              # per body "arap" | "neohookean"
    gravity: np.ndarray         # [B, 3] f32
    dt: float = 1.0 / 60.0
    iterations: int = 8

    @property
    def n_bodies(self) -> int:
        return len(self.bodies)


def concatenate(bodies: list) -> BodyBatch:
    """The union of independent meshes: vertex and tet arrays stacked, tet
    indices offset by each body's first vertex."""
    voff = np.zeros(len(bodies) + 1, dtype=np.int64)
    toff = np.zeros(len(bodies) + 1, dtype=np.int64)
    for b, m in enumerate(bodies):
        voff[b + 1] = voff[b] + m.n
        toff[b + 1] = toff[b] + m.T
    cat = lambda key: np.concatenate([getattr(m, key) for m in bodies])
    tets = np.concatenate([m.tet_indices.astype(np.int64) + voff[b] for b, m in enumerate(bodies)])
    first = bodies[0]
    union = BeamMesh(spec=first.spec, rest_q=cat("rest_q"), q0=cat("q0"), qd0=cat("qd0"),
                     tet_indices=tets.astype(np.int32), tet_poses=cat("tet_poses"),
                     tet_materials=cat("tet_materials"), particle_mass=cat("particle_mass"),
                     particle_inv_mass=cat("particle_inv_mass"), gravity=first.gravity)
    return BodyBatch(bodies=bodies, union=union, vertex_offsets=voff.astype(np.int32),
                     tet_offsets=toff.astype(np.int32), energies=[m.spec.energy for m in bodies],
                     gravity=np.stack([m.gravity for m in bodies]).astype(np.float32), dt=first.spec.dt,
                     iterations=first.spec.iterations)


def batched_bodies(n_bodies: int = 512, seed: int = 4, cell: float = 0.05, nx=(4, 48), nyz=(2, 12),
                   E=(1.0e4, 1.0e6), nu=(0.3, 0.48)) -> BodyBatch:
    """The batch of uneven beams: per body nx ~ U{4..48}, ny, nz ~ U{2..12}
    hex cells of `cell` m (6 tets each), ARAP or Neo-Hookean with p = 0.5,
    per-tet E log-uniform in E, nu ~ U(nu), gravity 9.81 m/s^2 along a
    direction uniform on the sphere, the x = 0 face pinned, at rest."""
    rng = np.random.default_rng(seed)
    bodies = []
    for b in range(n_bodies):
        cells = (int(rng.integers(nx[0], nx[1] + 1)), int(rng.integers(nyz[0], nyz[1] + 1)),
                 int(rng.integers(nyz[0], nyz[1] + 1)))
        energy = "arap" if rng.random() < 0.5 else "neohookean"
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        spec = BeamSpec(name=f"body{b}", cells=cells, extent=tuple(c * cell for c in cells), energy=energy,
                        E=E, nu=float(rng.uniform(nu[0], nu[1])), gravity=tuple(9.81 * d),
                        steps=10, seed=int(rng.integers(0, 2 ** 31 - 1)))
        bodies.append(build_beam(spec))
    return concatenate(bodies)
