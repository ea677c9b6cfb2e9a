"""Many independent bodies stepped together on one GPU.

``BatchedSolver`` concatenates the bodies of a ``beams.BodyBatch`` into one
mesh and one plan: the element, assembly and local-solve kernels run on the
union, while the global solve is one block-Jacobi PCG per body (its own
scalars and stopping test, as if each body were stepped alone with the
reference's ``RefinementSolver.step``) in a single persistent launch.  The
reference has no counterpart: it steps one body per solver.
The plain update is used (no line search), with the fp32 PCG.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .model import Model, State
from .solver import MixedFEMSolver, _stream_handle


class BatchedSolver:
    def __init__(self, batch, device="cuda:0", iterations=None, **kwargs):
        self.batch = batch
        u = batch.union
        self.model = Model(u.rest_q, np.zeros_like(u.rest_q), u.particle_mass, u.particle_inv_mass, u.tet_indices,
                           u.tet_poses, u.tet_materials, u.gravity, device=device)
        kwargs.setdefault("cg_tolerance", u.spec.cg_tolerance)
        kwargs.setdefault("cg_max_iterations", u.spec.cg_max_iterations)
        self.solver = MixedFEMSolver(self.model, iterations=iterations or batch.iterations, line_search=False,
                                     **kwargs)
        self._lib = self.solver._lib
        self._plan = self.solver._plan
        self._host = dict(voff=np.ascontiguousarray(batch.vertex_offsets, dtype=np.int32),
                          toff=np.ascontiguousarray(batch.tet_offsets, dtype=np.int32),
                          energy=np.array([_lib.ENERGY[e] for e in batch.energies], dtype=np.int32),
                          gravity=np.ascontiguousarray(batch.gravity, dtype=np.float32))
        h = self._host
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        _lib.check(self._lib.mfem_plan_set_bodies(self._plan, batch.n_bodies, P(h["voff"]), P(h["toff"]),
                                                  P(h["energy"]), P(h["gravity"])), self._plan)
        if kwargs.get("preconditioner") == "learned":
            # rest positions relative to each body's centroid
            self.solver.set_factor_net(kwargs.get("factor_net_params"), vertex_offsets=h["voff"])

    @property
    def n_bodies(self) -> int:
        return self.batch.n_bodies

    def state(self) -> State:
        s = self.model.state()
        s.particle_q.copy_(torch.as_tensor(self.batch.union.q0, device=self.model.device))
        return s

    def step(self, state_in: State, state_out: State, dt: float | None = None) -> None:
        self.solver.step(state_in, state_out, None, None, self.batch.dt if dt is None else dt)

    def layout(self) -> dict:
        c, t = ctypes.c_int32(), ctypes.c_int32()
        _lib.check(self._lib.mfem_plan_batch_layout(self._plan, ctypes.byref(c), ctypes.byref(t)), self._plan)
        return dict(ctas=c.value, threads=t.value)

    def autotune(self, q: torch.Tensor | None = None) -> float:
        """Picks the fastest PCG schedule on the system at q (default: the
        batch's initial positions); returns that solve's time in ms."""
        q = self.state().particle_q if q is None else q
        best = ctypes.c_double()
        _lib.check(self._lib.mfem_plan_autotune_batch(self._plan, ctypes.c_void_p(q.data_ptr()),
                                                      float(self.batch.dt), ctypes.byref(best),
                                                      _stream_handle(self.model.device)), self._plan)
        return best.value

    def body_stats(self) -> np.ndarray:
        """[iterations, bodies] records (iterations, status, rel_residual) of
        the last step."""
        B, K = self.n_bodies, self.solver.iterations
        buf = (_lib.MfemSolveStats * (B * K))()
        count = ctypes.c_int32()
        _lib.check(self._lib.mfem_step_body_stats(self._plan, buf, B * K, ctypes.byref(count),
                                                  _stream_handle(self.model.device)), self._plan)
        out = np.zeros((K, B), dtype=[("iterations", np.int32), ("status", np.int32), ("rel_residual", np.float32)])
        flat = out.reshape(-1)
        for i in range(count.value):
            flat[i] = (buf[i].iterations, buf[i].status, buf[i].rel_residual)
        return out

    def split(self, q: torch.Tensor) -> list:
        """Per-body views of a union array."""
        o = self.batch.vertex_offsets
        return [q[o[b]:o[b + 1]] for b in range(self.n_bodies)]
