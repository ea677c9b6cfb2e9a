"""Minimal Newton-compatible ``Model`` / ``State`` holders.

The reference's solver reads these fields of ``newton.Model``
(src/mfem/refinement/solver.py, additional_state.py): ``particle_q``
(rest positions), ``particle_qd``, ``particle_mass``, ``particle_inv_mass``,
``tet_indices``, ``tet_poses`` (DmInv), ``tet_materials`` (mu, lambda,
damping), ``gravity``, ``particle_count``, ``tet_count``, and for contact
``shape_transform``, ``shape_type``, ``shape_scale``, ``shape_body``,
``shape_count``, ``body_count``, ``tri_indices`` (src/mfem/refinement/
contact.py:864-875, solver.py:248-265); and of ``newton.State``:
``particle_q``, ``particle_qd``, ``body_q`` and ``assign``.  Newton is not a
dependency here, so these duck-typed classes carry the same names, with
torch tensors as device buffers.  ``shape_type`` holds this package's codes
(``SHAPE_PLANE``, ``SHAPE_CAPSULE``) in place of Newton's GeoType values.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch


SHAPE_PLANE = 0
SHAPE_CAPSULE = 1


@dataclass
class State:
    particle_q: torch.Tensor   # [n, 3] float32
    particle_qd: torch.Tensor  # [n, 3] float32
    body_q: Optional[torch.Tensor] = None  # [bodies, 7] float32 (px, py, pz, qx, qy, qz, qw)

    def assign(self, other: "State") -> None:
        self.particle_q.copy_(other.particle_q)
        self.particle_qd.copy_(other.particle_qd)
        if self.body_q is not None and other.body_q is not None:
            self.body_q.copy_(other.body_q)


class Model:
    def __init__(self, particle_q, particle_qd, particle_mass, particle_inv_mass, tet_indices, tet_poses,
                 tet_materials, gravity, device="cuda:0"):
        dev = torch.device(device)

        def f32(a, shape):
            t = torch.as_tensor(np.asarray(a, dtype=np.float32) if not torch.is_tensor(a) else a,
                                dtype=torch.float32, device=dev)
            return t.reshape(shape).contiguous()

        n = int(np.asarray(particle_q.shape)[0])
        T = int(np.asarray(tet_indices.shape)[0])
        self.device = dev
        self.particle_q = f32(particle_q, (n, 3))
        self.particle_qd = f32(particle_qd, (n, 3))
        self.particle_mass = f32(particle_mass, (n,))
        self.particle_inv_mass = f32(particle_inv_mass, (n,))
        self.tet_indices = torch.as_tensor(
            np.asarray(tet_indices, dtype=np.int32) if not torch.is_tensor(tet_indices) else tet_indices,
            dtype=torch.int32, device=dev).reshape(T, 4).contiguous()
        self.tet_poses = f32(tet_poses, (T, 3, 3))
        self.tet_materials = f32(tet_materials, (T, 3))
        self.gravity = f32(gravity, (1, 3))
        # rigid shapes and bodies for contact, surface tris for tri contact
        self.shape_transform = torch.zeros((0, 7), dtype=torch.float32, device=dev)
        self.shape_type = torch.zeros((0,), dtype=torch.int32, device=dev)
        self.shape_scale = torch.zeros((0, 3), dtype=torch.float32, device=dev)
        self.shape_body = torch.zeros((0,), dtype=torch.int32, device=dev)
        self.body_q = torch.zeros((0, 7), dtype=torch.float32, device=dev)
        self.tri_indices = torch.zeros((0, 3), dtype=torch.int32, device=dev)

    @property
    def particle_count(self) -> int:
        return int(self.particle_q.shape[0])

    @property
    def tet_count(self) -> int:
        return int(self.tet_indices.shape[0])

    @property
    def shape_count(self) -> int:
        return int(self.shape_type.shape[0])

    @property
    def body_count(self) -> int:
        return int(self.body_q.shape[0])

    def add_body(self, pose=(0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0)) -> int:
        """A kinematic rigid body at `pose`; returns its index."""
        p = torch.as_tensor(np.asarray(pose, dtype=np.float32), device=self.device).reshape(1, 7)
        self.body_q = torch.cat([self.body_q, p]).contiguous()
        return self.body_count - 1

    def _add_shape(self, kind, pose, scale, body) -> int:
        t = lambda a, dt, shape: torch.as_tensor(np.asarray(a, dtype=dt), device=self.device).reshape(shape)
        self.shape_transform = torch.cat([self.shape_transform, t(pose, np.float32, (1, 7))]).contiguous()
        self.shape_type = torch.cat([self.shape_type, t([kind], np.int32, (1,))]).contiguous()
        self.shape_scale = torch.cat([self.shape_scale, t(scale, np.float32, (1, 3))]).contiguous()
        self.shape_body = torch.cat([self.shape_body, t([body], np.int32, (1,))]).contiguous()
        return self.shape_count - 1

    def add_shape_plane(self, pose=(0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0), body=-1) -> int:
        """Infinite plane through the pose's origin, normal along local +Z."""
        return self._add_shape(SHAPE_PLANE, pose, (0.0, 0.0, 0.0), body)

    def add_shape_capsule(self, radius, half_height, pose=(0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0), body=-1) -> int:
        """Capsule along local +Z, centred on the pose's origin."""
        return self._add_shape(SHAPE_CAPSULE, pose, (radius, half_height, 0.0), body)

    def set_tri_indices(self, tris) -> None:
        self.tri_indices = torch.as_tensor(np.asarray(tris, dtype=np.int32), device=self.device).reshape(-1, 3)

    def pad_particles(self, max_particles: int) -> "Model":
        """The same model with its particle arrays padded to `max_particles`
        rows (zero position, velocity and mass, inverse mass 0): the headroom
        an adaptive refinement grows into, as the reference's
        ``load_sim_model(..., max_particles=...)`` pads Newton's particle
        buffer (src/mfem/refinement/models/refinement_model.py:104-143)."""
        n = self.particle_count
        if max_particles < n:
            raise ValueError(f"max_particles={max_particles} is below particle_count={n}")
        pad = max_particles - n

        def grow(t):
            return torch.cat([t, torch.zeros((pad,) + tuple(t.shape[1:]), dtype=t.dtype, device=t.device)])

        out = Model(grow(self.particle_q), grow(self.particle_qd), grow(self.particle_mass),
                    grow(self.particle_inv_mass), self.tet_indices, self.tet_poses, self.tet_materials, self.gravity,
                    device=self.device)
        for name in ("shape_transform", "shape_type", "shape_scale", "shape_body", "body_q", "tri_indices"):
            setattr(out, name, getattr(self, name).clone())
        return out

    def state(self) -> State:
        return State(self.particle_q.clone(), self.particle_qd.clone(),
                     self.body_q.clone() if self.body_count > 0 else None)

    def control(self):
        return None

    def contacts(self):
        return None

    @classmethod
    def from_beam(cls, mesh, device="cuda:0") -> "Model":
        """Model of a synthetic beam (``mfem_gb300.beams.build_beam``)."""
        return cls(mesh.rest_q, np.zeros_like(mesh.rest_q), mesh.particle_mass, mesh.particle_inv_mass,
                   mesh.tet_indices, mesh.tet_poses, mesh.tet_materials, mesh.gravity, device=device)
