"""Minimal Newton-compatible ``Model`` / ``State`` holders.

The reference's solver reads these fields of ``newton.Model``
(src/mfem/refinement/solver.py, additional_state.py): ``particle_q``
(rest positions), ``particle_qd``, ``particle_mass``, ``particle_inv_mass``,
``tet_indices``, ``tet_poses`` (DmInv), ``tet_materials`` (mu, lambda,
damping), ``gravity``, ``particle_count``, ``tet_count``; and of
``newton.State``: ``particle_q``, ``particle_qd`` and ``assign``.  Newton is
not a dependency here, so these duck-typed classes carry the same names, with
torch tensors as device buffers.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch


@dataclass
class State:
    particle_q: torch.Tensor   # [n, 3] float32
    particle_qd: torch.Tensor  # [n, 3] float32
    body_q: Optional[torch.Tensor] = None

    def assign(self, other: "State") -> None:
        self.particle_q.copy_(other.particle_q)
        self.particle_qd.copy_(other.particle_qd)


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

    @property
    def particle_count(self) -> int:
        return int(self.particle_q.shape[0])

    @property
    def tet_count(self) -> int:
        return int(self.tet_indices.shape[0])

    def state(self) -> State:
        return State(self.particle_q.clone(), self.particle_qd.clone())

    def control(self):
        return None

    def contacts(self):
        return None

    @classmethod
    def from_beam(cls, mesh, device="cuda:0") -> "Model":
        """Model of a synthetic beam (``mfem_gb300.beams.build_beam``)."""
        return cls(mesh.rest_q, np.zeros_like(mesh.rest_q), mesh.particle_mass, mesh.particle_inv_mass,
                   mesh.tet_indices, mesh.tet_poses, mesh.tet_materials, mesh.gravity, device=device)
