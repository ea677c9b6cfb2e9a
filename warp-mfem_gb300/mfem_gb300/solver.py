"""The reference-facing solver: ``RefinementSolver``'s constructor and
``step(state_in, state_out, control, contacts, dt)`` over the CUDA library.

Reference: src/mfem/refinement/solver.py:40-579.  Every step runs on the GPU
through libmfem_gb300 (element kernel, assembly, persistent PCG, local solve,
replayed as one CUDA graph); there is no CPU path.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from . import _lib
from .model import Model, State

_REFINE_COUNTS = 8  # mfem_refine_mesh.counts


def _stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


class MixedFEMSolver:
    """Mixed variational FEM global step on one GPU.

    Accepts ``RefinementSolver``'s arguments (src/mfem/refinement/solver.py:41-128).
    ``line_search`` defaults to True like the reference's (solver.py:185),
    with its ``line_search_max_iterations`` / ``_alpha0`` / ``_tau`` / ``_c`` /
    ``_threshold`` (solver.py:99-103); ``line_search=False`` gives the plain
    update x += dx, s += ds.  Contact against the model's rigid shapes
    (planes, capsules) takes the reference's ``contact_d0``, ``contact_d1``,
    ``contact_stiffness``, ``friction_mu`` (one value or one per shape),
    ``friction_eps_v`` and ``tri_contact`` (solver.py:241-265); it is on when
    the model has shapes.  Refinement and the membrane shell are outside this
    solver: ``enable_refinement`` defaults to False here and raises if set
    True; ``shell_mu`` must be 0.

    ``solver_precision`` ("fp32", the reference's float32 PCG and the
    default; "bf16" or "fp16") selects the mixed-precision global solve:
    16-bit BSR blocks with per-row scales in an inner PCG to
    ``inner_tolerance`` (1e-3) inside an fp64-residual iterative refinement
    to ``outer_tolerance`` (1e-8), at most ``outer_max_iterations`` (10)
    corrections.  "fp32_refined" runs the same refinement with the fp32
    blocks in the inner PCG: the plain fp32 PCG brought to an fp64-checked
    residual.

    ``preconditioner`` is the reference's flag (True: block-Jacobi, False:
    none), "fsai": a factorized sparse approximate inverse M = G^T G with G
    lower block-triangular on H's block pattern, recomputed after every
    assembly, or "learned": M = L L^T with L written by the factor net
    (``factor_net``; parameters ``factor_net_params`` or the shipped
    weights).  Both factor forms run the persistent factor PCG where its
    per-CTA ranges fit in shared memory, else the global-memory PCG
    (``pcg_variant`` "factor" or "global_memory" forces one); with a 16-bit
    ``solver_precision`` they precondition the inner PCG.
    ``factor_refresh`` k recomputes the factor at every k-th Newton
    iteration of a step (default 1: every assembly).

    ``enable_refinement=True`` (default False here; the reference defaults to
    True but, with its default weights and no contact, never splits) runs an
    edge-bisection refinement pass on the GPU (``mfem_refine``) at the start
    of every ``refine_every_n_steps``-th step, counted from the first, with
    the reference's ``refine_*`` kwargs (solver.py:56-87): ``refine_scoring``
    "legacy" (threshold ``min_refine_score``) or "geometric" (threshold
    ``refine_geometric_threshold``), ``refine_tet_score_weight``,
    ``refine_vertex_score_weight``, ``penetrating_edge_score``,
    ``refine_min_edge_length`` (default ``contact_d1``),
    ``refine_elastic_weight``, ``refine_contact_weight``,
    ``refine_tri_contact_weight``, ``refine_conflict_iterations``,
    ``refine_split_position`` and ``refine_density`` (the lumped masses of a
    refined mesh; default 1.0 as the reference's).  As in the reference the
    model's particle arrays are padded to ``max_particles`` rows and the
    mesh's vertices are those its tets reference; states carry all
    ``max_particles`` rows and ``max_tets`` bounds the tets.  A pass that
    splits edges writes the new vertices into state_out and state_in (the
    reference copies them into state_in too, solver.py:500) and rebuilds the
    plan on the refined mesh, carrying s and lambda over; the host reads the
    pass's counts back, so a refining step synchronises.

    ``pcg_variant``: "auto" (default), "standard", "single_reduction",
    "gather" (block-Jacobi / no preconditioner), "factor" (the persistent
    factor PCG) or "global_memory" (the batched kernel's PCG on one body).
    """

    def __init__(self, model: Model, iterations: int, max_tets: Optional[int] = None,
                 max_particles: Optional[int] = None, max_tris: Optional[int] = None,
                 refine_every_n_steps: int = 10, min_refine_score: float = 10.1, **kwargs):
        if kwargs.get("shell_mu", 0.0) != 0.0:
            raise NotImplementedError("shell_mu > 0: the membrane shell is not part of this solver")
        if max_particles is not None and max_particles != model.particle_count:
            raise ValueError(
                f"max_particles={max_particles} does not match model.particle_count={model.particle_count}")
        if max_tets is not None and max_tets < model.tet_count:
            raise ValueError(f"max_tets={max_tets} is below model.tet_count={model.tet_count}")
        self.refine_enabled = bool(kwargs.get("enable_refinement", False))
        if self.refine_enabled and max_tets is None:
            raise ValueError("enable_refinement=True needs max_tets")
        energy = kwargs.get("energy", "arap")
        if energy not in _lib.ENERGY:
            raise ValueError(f"Unknown energy type: {energy}")
        if model.device.type != "cuda":
            raise ValueError("the model must live on a CUDA device")

        self.model = model
        self.iterations = int(iterations)
        self.device = model.device
        self._lib = _lib.load()
        cfg = _lib.default_config()
        cfg.iterations = self.iterations
        cfg.energy = _lib.ENERGY[energy]
        cfg.cg_max_iterations = int(kwargs.get("cg_max_iterations", 1000))
        cfg.cg_tolerance = float(kwargs.get("cg_tolerance", 1.0e-6))
        cfg.attachment_stiffness = float(kwargs.get("attachment_stiffness", 10.0))
        cfg.preconditioner_singular_threshold = float(kwargs.get("preconditioner_singular_threshold", 1.0e-20))
        pc = kwargs.get("preconditioner", True)
        if isinstance(pc, str):
            if pc not in _lib.PRECONDITIONER:
                raise ValueError(f"unknown preconditioner {pc!r}")
            cfg.preconditioner = _lib.PRECONDITIONER[pc]
        else:
            cfg.preconditioner = 1 if pc else 0
        cfg.use_cuda_graph = 1 if kwargs.get("use_cuda_graph", True) else 0
        cfg.pcg_ctas = int(kwargs.get("pcg_ctas", 0))
        cfg.pcg_variant = {"auto": 0, "standard": 1, "single_reduction": 2, "gather": 3, "factor": 4,
                           "global_memory": 5}[kwargs.get("pcg_variant", "auto")]
        self.line_search = bool(kwargs.get("line_search", True))
        cfg.line_search = 1 if self.line_search else 0
        cfg.line_search_max_iterations = int(kwargs.get("line_search_max_iterations", 20))
        cfg.line_search_alpha0 = float(kwargs.get("line_search_alpha0", 1.0))
        cfg.line_search_tau = float(kwargs.get("line_search_tau", 0.5))
        cfg.line_search_c = float(kwargs.get("line_search_c", 0.01))
        cfg.line_search_threshold = float(kwargs.get("line_search_threshold", 1.0e-8))
        self.config = cfg

        self.solver_precision = kwargs.get("solver_precision", "fp32")
        if self.solver_precision not in _lib.PRECISION:
            raise ValueError(f"Unknown solver_precision {self.solver_precision!r}")
        self._kwargs = dict(kwargs)
        self._residual_check = False
        self._diagnostics = False
        self._plan = None

        host = lambda t, dt: np.ascontiguousarray(t.detach().to("cpu").numpy(), dtype=dt)
        h = dict(
            tets=host(model.tet_indices, np.int32), poses=host(model.tet_poses, np.float32),
            materials=host(model.tet_materials, np.float32), rest=host(model.particle_q, np.float32),
            mass=host(model.particle_mass, np.float32), inv_mass=host(model.particle_inv_mass, np.float32),
            gravity=host(model.gravity.reshape(-1)[:3], np.float32))
        tris = getattr(model, "tri_indices", None)
        h["tris"] = host(tris, np.int32).reshape(-1, 3) if tris is not None else np.zeros((0, 3), np.int32)
        self.max_particles = model.particle_count
        if self.refine_enabled:
            # the mesh's vertices are those its tets reference (get_active_particles,
            # additional_state.py:7-15); the rest of the particle arrays is headroom
            n_active = int(h["tets"].max()) + 1 if h["tets"].size else model.particle_count
            for key in ("rest", "mass", "inv_mass"):
                h[key] = np.ascontiguousarray(h[key][:n_active])
        self._host = h
        self._create_plan(model)
        if self.refine_enabled:
            self._init_refinement(model, max_tets, max_tris, refine_every_n_steps, min_refine_score, kwargs)

    def _create_plan(self, model) -> None:
        """Plan of the mesh in self._host, with the contact, factor net and
        solver settings of the constructor's arguments."""
        h = self._host
        kwargs = self._kwargs
        plan = ctypes.c_void_p()
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        n_rows = h["rest"].shape[0]
        rc = self._lib.mfem_plan_create(
            ctypes.byref(self.config), n_rows, h["tets"].shape[0], P(h["tets"]), P(h["poses"]),
            P(h["materials"]), P(h["rest"]), P(h["mass"]), P(h["inv_mass"]), P(h["gravity"]),
            self.device.index if self.device.index is not None else torch.cuda.current_device(), ctypes.byref(plan))
        if rc != _lib.MFEM_OK:
            msg = self._lib.mfem_plan_last_error(None).decode()
            raise _lib.MfemError(rc, f"mfem_plan_create: {msg}")
        self._plan = plan
        n = ctypes.c_int32()
        T = ctypes.c_int32()
        nnzb = ctypes.c_int64()
        self._lib.mfem_plan_sizes(plan, ctypes.byref(n), ctypes.byref(T), ctypes.byref(nnzb))
        self.n, self.T, self.nnzb = n.value, T.value, nnzb.value
        self.n_bodies = 0
        self.n_contact_tris = 0
        if getattr(model, "shape_count", 0) > 0:
            self._set_contact(model, kwargs, h["tris"])
        if self.config.preconditioner == _lib.PRECONDITIONER["learned"]:
            self.set_factor_net(kwargs.get("factor_net_params"))
        if self.solver_precision != "fp32" or "factor_refresh" in kwargs:
            scfg = _lib.MfemSolverConfig()
            self._lib.mfem_solver_config_default(ctypes.byref(scfg))
            scfg.precision = _lib.PRECISION[self.solver_precision]
            scfg.factor_refresh = int(kwargs.get("factor_refresh", 1))
            scfg.inner_tolerance = float(kwargs.get("inner_tolerance", 1.0e-3))
            scfg.outer_tolerance = float(kwargs.get("outer_tolerance", 1.0e-8))
            scfg.outer_max_iterations = int(kwargs.get("outer_max_iterations", 10))
            _lib.check(self._lib.mfem_plan_set_solver(self._plan, ctypes.byref(scfg)), self._plan)
        if self._residual_check:
            self.set_residual_check(True)
        if self._diagnostics:
            self.set_diagnostics(True)

    # -- adaptive refinement -----------------------------------------------------
    def _init_refinement(self, model, max_tets, max_tris, refine_every_n_steps, min_refine_score, kwargs) -> None:
        """Capacity buffers and settings of the refinement passes
        (RefinementSolver.__init__, src/mfem/refinement/solver.py:56-87, 139-170)."""
        self._model = model
        self.max_tets = int(max_tets)
        headroom = max(1, -(-self.max_tets // max(1, model.tet_count)))
        self.max_tris = int(max_tris) if max_tris else int(self._host["tris"].shape[0]) * headroom
        self.refine_every_n_steps = int(refine_every_n_steps)
        scoring = kwargs.get("refine_scoring", "legacy")
        if scoring not in _lib.REFINE_SCORING:
            raise ValueError(f"Unknown refine_scoring {scoring!r} (expected 'legacy' or 'geometric')")
        rc = _lib.MfemRefineConfig()
        self._lib.mfem_refine_config_default(ctypes.byref(rc))
        rc.scoring = _lib.REFINE_SCORING[scoring]
        rc.threshold = float(kwargs.get("refine_geometric_threshold", 1.0) if scoring == "geometric"
                             else min_refine_score)
        rc.tet_score_weight = float(kwargs.get("refine_tet_score_weight", 0.0))
        rc.vertex_score_weight = float(kwargs.get("refine_vertex_score_weight", 0.1))
        rc.penetrating_edge_score = float(kwargs.get("penetrating_edge_score", 1.0e6))
        d1 = float(kwargs.get("contact_d1", 1.0e-1))
        min_edge = kwargs.get("refine_min_edge_length", None)
        rc.min_edge_length = float(min_edge) if min_edge is not None else d1
        rc.contact_d1 = d1
        rc.elastic_weight = float(kwargs.get("refine_elastic_weight", 1.0))
        rc.vertex_contact_weight = float(kwargs.get("refine_contact_weight", 1.0))
        rc.tri_contact_weight = float(kwargs.get("refine_tri_contact_weight", 1.0))
        rc.split_position = float(kwargs.get("refine_split_position", 0.5))
        rc.density = float(kwargs.get("refine_density", 1.0))
        rc.conflict_iterations = int(kwargs.get("refine_conflict_iterations", 5))
        rc.refine_every = max(self.refine_every_n_steps, 1)
        self.refine_config = rc
        self._refine_pass = 0
        self.refine_history: list[dict] = []
        dev = self.device
        z = lambda shape, dt: torch.zeros(shape, dtype=dt, device=dev)
        self._rmesh = dict(tets=z((self.max_tets, 4), torch.int32), poses=z((self.max_tets, 9), torch.float32),
                           materials=z((self.max_tets, 3), torch.float32),
                           stretch=z((self.max_tets, 6), torch.float32), lam=z((self.max_tets, 6), torch.float32),
                           rest=z((self.max_particles, 3), torch.float32), mass=z((self.max_particles,), torch.float32),
                           inv_mass=z((self.max_particles,), torch.float32),
                           tris=z((max(self.max_tris, 1), 3), torch.int32), counts=z((_REFINE_COUNTS,), torch.int32))
        r = self._rmesh
        m = _lib.MfemRefineMesh()
        m.max_particles, m.max_tets, m.max_tris = self.max_particles, self.max_tets, self.max_tris
        for field, key in (("tet_indices", "tets"), ("tet_poses", "poses"), ("tet_materials", "materials"),
                           ("tet_stretch", "stretch"), ("tet_lambda", "lam"), ("rest_q", "rest"),
                           ("particle_mass", "mass"), ("particle_inv_mass", "inv_mass"), ("tri_indices", "tris"),
                           ("counts", "counts")):
            setattr(m, field, r[key].data_ptr())
        self._rmesh_struct = m

    @property
    def active_particle_count(self) -> int:
        return self.n

    @property
    def active_tet_count(self) -> int:
        return self.T

    def _refine(self, state_in: State, state_out: State) -> None:
        """One refinement pass at state_out (= state_in) and, when it splits
        edges, the plan rebuilt on the refined mesh."""
        every = max(self.refine_every_n_steps, 1)
        refining = self._refine_pass % every == 0
        self._refine_pass += 1
        if not refining:
            return
        stream = _stream_handle(self.device)
        rc = self._lib.mfem_refine(self._plan, ctypes.byref(self.refine_config), None,
                                   ctypes.c_void_p(state_out.particle_q.data_ptr()),
                                   ctypes.c_void_p(state_out.particle_qd.data_ptr()), None,
                                   ctypes.byref(self._rmesh_struct), stream)
        _lib.check(rc, self._plan)
        counts = self._rmesh["counts"].cpu().tolist()
        n_new, T_new, m_new, split, overflow = counts[:5]
        self.refine_history.append(dict(pass_index=self._refine_pass - 1, split_edges=split, overflow=bool(overflow),
                                        particles=n_new, tets=T_new, tris=m_new))
        if split == 0:
            return
        n_old = self.n
        r = self._rmesh
        host = lambda t: np.ascontiguousarray(t.cpu().numpy())
        self._host = dict(tets=host(r["tets"][:T_new]), poses=host(r["poses"][:T_new]),
                          materials=host(r["materials"][:T_new]), rest=host(r["rest"][:n_new]),
                          mass=host(r["mass"][:n_new]), inv_mass=host(r["inv_mass"][:n_new]),
                          gravity=self._host["gravity"],
                          tris=host(r["tris"][:m_new]) if self.n_contact_tris > 0 else self._host["tris"])
        stretch = r["stretch"][:T_new].clone()
        lam = r["lam"][:T_new].clone()
        torch.cuda.current_stream(self.device).synchronize()
        self.close()
        self._create_plan(self._model)
        self.write_buffer("tet_stretch", stretch.reshape(-1))
        self.write_buffer("tet_lambda", lam.reshape(-1))
        state_in.particle_q[n_old:n_new].copy_(state_out.particle_q[n_old:n_new])
        state_in.particle_qd[n_old:n_new].copy_(state_out.particle_qd[n_old:n_new])

    def refined_mesh(self) -> dict:
        """The current mesh as host arrays (tets, DmInv, materials, rest
        positions, masses, inverse masses, contact tris) and s, lambda."""
        out = {k: v.copy() for k, v in self._host.items() if k != "gravity"}
        out["tet_stretch"] = self.tet_stretch.cpu().numpy()
        out["tet_lambda"] = self.tet_lambda.cpu().numpy()
        return out

    def set_factor_net(self, params=None, vertex_offsets=None) -> None:
        """Loads the learned preconditioner's parameters (packed float32,
        ``factor_net.LAYOUT``; None: the weights shipped with the package)
        and the static vertex inputs of the model (per-body centroids for
        ``vertex_offsets``)."""
        from . import factor_net
        if params is None:
            params = factor_net.load_weights()
        params = np.ascontiguousarray(params, dtype=np.float32).reshape(-1)
        h = self._host
        vs = np.ascontiguousarray(factor_net.static_features(
            h["rest"], h["tets"].reshape(-1, 4), h["materials"].reshape(-1, 3), vertex_offsets), dtype=np.float32)
        self._factor_net = (params, vs)  # kept alive while the call copies them
        _lib.check(self._lib.mfem_plan_set_factor_net(self._plan, params.ctypes.data_as(ctypes.c_void_p),
                                                      params.size, vs.ctypes.data_as(ctypes.c_void_p)),
                   self._plan)

    def _set_contact(self, model, kwargs, tris) -> None:
        """Contact against the model's shapes (Contact.__init__,
        src/mfem/refinement/contact.py:778-862)."""
        ccfg = _lib.MfemContactConfig()
        self._lib.mfem_contact_config_default(ctypes.byref(ccfg))
        ccfg.d0 = float(kwargs.get("contact_d0", 1.0e-2))
        ccfg.d1 = float(kwargs.get("contact_d1", 1.0e-1))
        ccfg.stiffness = float(kwargs.get("contact_stiffness", 1.0e7))
        ccfg.friction_eps_v = float(kwargs.get("friction_eps_v", 1.0e-3))
        ccfg.tri_contact = 1 if kwargs.get("tri_contact", True) else 0
        S = model.shape_count
        mu = np.asarray(kwargs.get("friction_mu", 0.0), dtype=np.float32)
        if mu.ndim == 0:
            mu = np.full(S, float(mu), dtype=np.float32)
        elif mu.shape[0] != S:
            raise ValueError(f"friction_mu has {mu.shape[0]} entries but the model has {S} shapes")
        host = lambda t, dt: np.ascontiguousarray(t.detach().to("cpu").numpy(), dtype=dt)
        tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1, 3)
        self._contact_host = dict(type=host(model.shape_type, np.int32), pose=host(model.shape_transform, np.float32),
                                  scale=host(model.shape_scale, np.float32), body=host(model.shape_body, np.int32),
                                  mu=np.ascontiguousarray(mu), tris=np.ascontiguousarray(tris))
        h = self._contact_host
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        n_bodies = int(getattr(model, "body_count", 0))
        rc = self._lib.mfem_plan_set_contact(self._plan, ctypes.byref(ccfg), S, P(h["type"]), P(h["pose"]),
                                             P(h["scale"]), P(h["body"]), P(h["mu"]), n_bodies, tris.shape[0],
                                             P(h["tris"]))
        _lib.check(rc, self._plan)
        self.contact_config = ccfg
        self.n_bodies = n_bodies
        self.n_contact_tris = tris.shape[0] if ccfg.tri_contact else 0
        if n_bodies > 0:
            self.set_body_poses(model.body_q)

    def set_body_poses(self, body_q: torch.Tensor) -> None:
        """Body poses [bodies, 7] the next steps read (asynchronous)."""
        if not (body_q.is_cuda and body_q.dtype == torch.float32 and body_q.is_contiguous()
                and tuple(body_q.shape) == (self.n_bodies, 7)):
            raise ValueError(f"body_q must be a contiguous float32 CUDA tensor of shape ({self.n_bodies}, 7)")
        _lib.check(self._lib.mfem_set_body_poses(self._plan, ctypes.c_void_p(body_q.data_ptr()), self.n_bodies,
                                                 _stream_handle(self.device)), self._plan)

    def autotune(self, q: torch.Tensor, dt: float) -> float:
        """For a plan on the global-memory PCG (a mesh too large for the
        persistent PCGs, or pcg_variant="global_memory"): picks the fastest schedule
        on the system at q (at rest); returns that solve's time in ms."""
        if self.pcg_layout()["variant"] != "global_memory":
            raise ValueError("autotune serves plans on the global-memory PCG")
        best = ctypes.c_double()
        _lib.check(self._lib.mfem_plan_autotune_batch(self._plan, ctypes.c_void_p(self._check_state(q, "q")),
                                                      float(dt), ctypes.byref(best), _stream_handle(self.device)),
                   self._plan)
        return best.value

    def pcg_layout(self) -> dict:
        """The persistent PCG this plan uses (variant, CTAs, matrix cached in
        shared memory, dynamic shared memory per CTA)."""
        v, c, m = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        smem = ctypes.c_int64()
        _lib.check(self._lib.mfem_plan_pcg_layout(self._plan, ctypes.byref(v), ctypes.byref(c), ctypes.byref(m),
                                                  ctypes.byref(smem)), self._plan)
        name = {0: "global_memory", 1: "standard", 2: "single_reduction", 3: "gather", 4: "factor"}[v.value]
        return dict(variant=name, ctas=c.value, cache_matrix=bool(m.value), smem_bytes=smem.value)

    # ------------------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_plan", None):
            self._lib.mfem_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check_state(self, t: torch.Tensor, name: str) -> int:
        rows = self.max_particles if self.refine_enabled else self.n
        if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous() and tuple(t.shape) == (rows, 3)):
            raise ValueError(f"{name} must be a contiguous float32 CUDA tensor of shape ({rows}, 3)")
        if t.device != self.device:
            raise ValueError(f"{name} lives on {t.device}, the solver on {self.device}")
        return t.data_ptr()

    # ------------------------------------------------------------------
    def step(self, state_in: State, state_out: State, control, contacts, dt: float) -> None:
        """One implicit-Euler step (src/mfem/refinement/solver.py:429-579): writes
        state_out.particle_q / particle_qd; state_in is not modified."""
        q_in = self._check_state(state_in.particle_q, "state_in.particle_q")
        qd_in = self._check_state(state_in.particle_qd, "state_in.particle_qd")
        q_out = self._check_state(state_out.particle_q, "state_out.particle_q")
        qd_out = self._check_state(state_out.particle_qd, "state_out.particle_qd")
        if self.refine_enabled:
            # refinement writes the new vertices into state_out first
            # (solver.py:443-500)
            state_out.assign(state_in)
            if self.n_bodies > 0 and getattr(state_out, "body_q", None) is not None:
                self.set_body_poses(state_out.body_q)
            self._refine(state_in, state_out)
        if self.n_bodies > 0 and getattr(state_out, "body_q", None) is not None:
            # the reference reads the rigid bodies' poses from state_out
            self.set_body_poses(state_out.body_q)
        rc = self._lib.mfem_step(self._plan, q_in, qd_in, q_out, qd_out, float(dt), _stream_handle(self.device))
        _lib.check(rc, self._plan)

    def solve_stats(self) -> list[dict]:
        """PCG outcome of each Newton iteration of the last step (synchronises)."""
        buf = (_lib.MfemSolveStats * max(1, self.iterations))()
        count = ctypes.c_int32()
        rc = self._lib.mfem_step_stats(self._plan, buf, max(1, self.iterations), ctypes.byref(count),
                                       _stream_handle(self.device))
        _lib.check(rc, self._plan)
        return [dict(iterations=buf[i].iterations, status=buf[i].status, rel_residual=buf[i].rel_residual)
                for i in range(count.value)]

    def mixed_stats(self) -> list[dict]:
        """Mixed-precision solve outcome of each Newton iteration of the last
        step (synchronises; empty with the fp32 solve)."""
        buf = (_lib.MfemMixedSolveStats * max(1, self.iterations))()
        count = ctypes.c_int32()
        rc = self._lib.mfem_step_mixed_stats(self._plan, buf, max(1, self.iterations), ctypes.byref(count),
                                             _stream_handle(self.device))
        _lib.check(rc, self._plan)
        return [dict(outer_iterations=buf[i].outer_iterations, inner_iterations=buf[i].inner_iterations,
                     status=buf[i].status, fp32_inner=bool(buf[i].fp32_inner), rel_residual=buf[i].rel_residual)
                for i in range(count.value)]

    def line_search_stats(self) -> list[dict]:
        """Line-search outcome of each Newton iteration of the last step
        (synchronises; all zero with the line search off)."""
        buf = (_lib.MfemLineSearchStats * max(1, self.iterations))()
        count = ctypes.c_int32()
        rc = self._lib.mfem_step_line_search_stats(self._plan, buf, max(1, self.iterations), ctypes.byref(count),
                                                   _stream_handle(self.device))
        _lib.check(rc, self._plan)
        return [dict(evaluations=buf[i].evaluations, accepted=bool(buf[i].accepted), alpha=buf[i].alpha,
                     status=buf[i].status, f0=buf[i].f0, f1=buf[i].f1, t=buf[i].t) for i in range(count.value)]

    # -- stages (the reference's operators) ----------------------------------
    def predict(self, q: torch.Tensor, qd: torch.Tensor, dt: float) -> None:
        _lib.check(self._lib.mfem_predict(self._plan, self._check_state(q, "q"), self._check_state(qd, "qd"),
                                          float(dt), _stream_handle(self.device)), self._plan)

    def update_system(self, x: torch.Tensor) -> None:
        _lib.check(self._lib.mfem_update_system(self._plan, self._check_state(x, "x"), _stream_handle(self.device)),
                   self._plan)

    def assemble(self, x: torch.Tensor, dt: float) -> None:
        _lib.check(self._lib.mfem_assemble(self._plan, self._check_state(x, "x"), float(dt),
                                           _stream_handle(self.device)), self._plan)

    def global_solve(self, slot: int = 0) -> None:
        _lib.check(self._lib.mfem_global_solve(self._plan, int(slot), _stream_handle(self.device)), self._plan)

    def local_solve(self, x: torch.Tensor) -> None:
        """Local solve and update of x and s: the plain x += dx, s += ds, or
        with the line search on, the search along (dx, ds) at the dt of the
        last assemble(), recorded in the slot of the last global_solve()."""
        _lib.check(self._lib.mfem_local_solve(self._plan, self._check_state(x, "x"), _stream_handle(self.device)),
                   self._plan)

    def true_residual(self) -> float:
        out = ctypes.c_double()
        _lib.check(self._lib.mfem_true_residual(self._plan, ctypes.byref(out), _stream_handle(self.device)),
                   self._plan)
        return out.value

    def set_diagnostics(self, on: bool) -> None:
        """Turns on or off the element stage's diagnostic outputs (H_s^-1 and
        g_lambda buffers, the reference's intermediates that the step does not
        read)."""
        _lib.check(self._lib.mfem_plan_set_diagnostics(self._plan, int(bool(on))), self._plan)
        self._diagnostics = bool(on)

    def inject_timeout(self) -> None:
        """Sets the plan's sticky device error flag, as a bounded wait that
        gave up does (host-side failure injection for tests): the next step's
        persistent kernels leave at once, its stats calls raise MFEM_TIMEOUT
        and re-arm the grid barriers, and the step after runs normally."""
        _lib.check(self._lib.mfem_plan_inject_timeout(self._plan), self._plan)

    def set_residual_check(self, on: bool) -> None:
        """Turns on or off the fp64 check of every global solve inside step()
        (read back with step_true_residuals); the trajectory is unchanged."""
        _lib.check(self._lib.mfem_plan_set_residual_check(self._plan, int(bool(on))), self._plan)
        self._residual_check = bool(on)

    def step_true_residuals(self) -> list[float]:
        """||g - H dx|| / ||g|| in float64 of each global solve of the last
        step, for the float32 dx the local solve read (synchronises)."""
        buf = (ctypes.c_double * max(1, self.iterations))()
        count = ctypes.c_int32()
        rc = self._lib.mfem_step_true_residuals(self._plan, buf, max(1, self.iterations), ctypes.byref(count),
                                                _stream_handle(self.device))
        _lib.check(rc, self._plan)
        return [buf[i] for i in range(count.value)]

    # -- buffers ---------------------------------------------------------------
    _BUF_DTYPE = {"row_ptr": torch.int32, "col_idx": torch.int32, "tet_slots": torch.int32,
                  "mixed_dx": torch.float64}

    def contact_tris(self) -> np.ndarray:
        """The per-tri contact record [m, 12] (d, k b, k b', k max(b'', 0),
        n[3], w[3], shape, 0) of the last assembly."""
        return self.read_buffer("tri_contact").cpu().numpy().reshape(-1, 12)

    def read_buffer(self, name: str) -> torch.Tensor:
        """Device copy of an internal buffer (flat; layouts in include/mfem_gb300.h)."""
        which = _lib.BUF[name]
        nbytes = ctypes.c_size_t()
        _lib.check(self._lib.mfem_plan_buffer_bytes(self._plan, which, ctypes.byref(nbytes)), self._plan)
        dt = self._BUF_DTYPE.get(name, torch.float32)
        out = torch.empty(nbytes.value // (8 if dt == torch.float64 else 4), dtype=dt, device=self.device)
        _lib.check(self._lib.mfem_plan_copy_out(self._plan, which, ctypes.c_void_p(out.data_ptr()), nbytes.value,
                                                _stream_handle(self.device)), self._plan)
        return out

    def write_buffer(self, name: str, values: torch.Tensor) -> None:
        which = _lib.BUF[name]
        nbytes = ctypes.c_size_t()
        _lib.check(self._lib.mfem_plan_buffer_bytes(self._plan, which, ctypes.byref(nbytes)), self._plan)
        src = values.to(self.device).contiguous()
        if src.numel() * src.element_size() != nbytes.value:
            raise ValueError(f"{name}: expected {nbytes.value} bytes")
        _lib.check(self._lib.mfem_plan_copy_in(self._plan, which, ctypes.c_void_p(src.data_ptr()), nbytes.value,
                                               _stream_handle(self.device)), self._plan)
        torch.cuda.current_stream(self.device).synchronize()

    @property
    def tet_stretch(self) -> torch.Tensor:
        return self.read_buffer("tet_stretch").reshape(self.T, 6)

    @property
    def tet_lambda(self) -> torch.Tensor:
        return self.read_buffer("tet_lambda").reshape(self.T, 6)

    # -- checkpoint / resume ---------------------------------------------------
    def save_state(self, path: str, state: State) -> None:
        """Writes x, v, s and lambda to an npz file."""
        np.savez(path, particle_q=state.particle_q.cpu().numpy(), particle_qd=state.particle_qd.cpu().numpy(),
                 tet_stretch=self.tet_stretch.cpu().numpy(), tet_lambda=self.tet_lambda.cpu().numpy())

    def load_state(self, path: str, state: State) -> None:
        d = np.load(path)
        state.particle_q.copy_(torch.as_tensor(d["particle_q"], device=self.device))
        state.particle_qd.copy_(torch.as_tensor(d["particle_qd"], device=self.device))
        self.write_buffer("tet_stretch", torch.as_tensor(d["tet_stretch"]).reshape(-1))
        self.write_buffer("tet_lambda", torch.as_tensor(d["tet_lambda"]).reshape(-1))


# The reference's class name, for drop-in use.
RefinementSolver = MixedFEMSolver
