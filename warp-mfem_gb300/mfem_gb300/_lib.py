"""ctypes binding of libmfem_gb300.so (include/mfem_gb300.h).

The library is the only compute path: if it is missing this module raises,
there is no fallback.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

from . import build as _build

LIB_PATH = _build.LIB_PATH
HEADER = _build.INCLUDE / "mfem_gb300.h"

MFEM_OK = 0
MFEM_MAXITER = 1
MFEM_STAGNATION = 2
MFEM_NONFINITE = 3
MFEM_BAD_ARG = 4
MFEM_CUDA_ERROR = 5
MFEM_TIMEOUT = 6

ENERGY = {"arap": 0, "neohookean": 1}
PRECONDITIONER = {"none": 0, "block_jacobi": 1, "fsai": 2, "learned": 3}
FACTOR_NET_PARAMS = 35663

BUF = {
    "tet_stretch": 0, "tet_lambda": 1, "constraint": 2, "grad_constraint": 3, "grad_s": 4,
    "h_lambda": 5, "hess_s_inv": 6, "g_lambda": 7, "element_hessian": 8, "element_rhs": 9,
    "row_ptr": 10, "col_idx": 11, "tet_slots": 12, "h_values": 13, "rhs": 14, "precond": 15,
    "x_tilde": 16, "dx": 17, "stretch_direction": 18, "contact_block": 19, "contact_gradient": 20,
    "contact_energy": 21, "tri_contact": 22, "friction_normal": 23, "friction_force": 24, "mixed_dx": 25,
    "precond_factor": 26,
}

SHAPE_PLANE = 0
SHAPE_CAPSULE = 1


class MfemConfig(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int32),
        ("energy", ctypes.c_int32),
        ("cg_max_iterations", ctypes.c_int32),
        ("cg_tolerance", ctypes.c_float),
        ("attachment_stiffness", ctypes.c_float),
        ("preconditioner_singular_threshold", ctypes.c_float),
        ("preconditioner", ctypes.c_int32),
        ("use_cuda_graph", ctypes.c_int32),
        ("pcg_ctas", ctypes.c_int32),
        ("pcg_variant", ctypes.c_int32),
        ("line_search", ctypes.c_int32),
        ("line_search_max_iterations", ctypes.c_int32),
        ("line_search_alpha0", ctypes.c_float),
        ("line_search_tau", ctypes.c_float),
        ("line_search_c", ctypes.c_float),
        ("line_search_threshold", ctypes.c_float),
    ]


class MfemSolveStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int32),
        ("status", ctypes.c_int32),
        ("rel_residual", ctypes.c_float),
        ("reserved", ctypes.c_float),
    ]


class MfemLineSearchStats(ctypes.Structure):
    _fields_ = [
        ("evaluations", ctypes.c_int32),
        ("accepted", ctypes.c_int32),
        ("alpha", ctypes.c_float),
        ("status", ctypes.c_int32),
        ("f0", ctypes.c_double),
        ("f1", ctypes.c_double),
        ("t", ctypes.c_double),
    ]


class MfemContactConfig(ctypes.Structure):
    _fields_ = [
        ("d0", ctypes.c_float),
        ("d1", ctypes.c_float),
        ("stiffness", ctypes.c_float),
        ("friction_eps_v", ctypes.c_float),
        ("tri_contact", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 3),
    ]


class MfemSolverConfig(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int32),
        ("inner_tolerance", ctypes.c_float),
        ("outer_max_iterations", ctypes.c_int32),
        ("factor_refresh", ctypes.c_int32),
        ("outer_tolerance", ctypes.c_double),
        ("reserved", ctypes.c_int32 * 4),
    ]


class MfemMixedSolveStats(ctypes.Structure):
    _fields_ = [
        ("outer_iterations", ctypes.c_int32),
        ("inner_iterations", ctypes.c_int32),
        ("status", ctypes.c_int32),
        ("fp32_inner", ctypes.c_int32),
        ("rel_residual", ctypes.c_double),
    ]


PRECISION = {"fp32": 0, "bf16": 1, "fp16": 2, "fp32_refined": 3}

REFINE_SCORING = {"legacy": 0, "geometric": 1}


class MfemRefineConfig(ctypes.Structure):
    _fields_ = [
        ("scoring", ctypes.c_int32),
        ("threshold", ctypes.c_float),
        ("tet_score_weight", ctypes.c_float),
        ("vertex_score_weight", ctypes.c_float),
        ("penetrating_edge_score", ctypes.c_float),
        ("min_edge_length", ctypes.c_float),
        ("contact_d1", ctypes.c_float),
        ("elastic_weight", ctypes.c_float),
        ("vertex_contact_weight", ctypes.c_float),
        ("tri_contact_weight", ctypes.c_float),
        ("split_position", ctypes.c_float),
        ("density", ctypes.c_float),
        ("conflict_iterations", ctypes.c_int32),
        ("refine_every", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 4),
    ]


class MfemRefineInputs(ctypes.Structure):
    _fields_ = [
        ("tet_scores", ctypes.c_void_p),
        ("vertex_scores", ctypes.c_void_p),
        ("particle_distance", ctypes.c_void_p),
        ("particle_shape_id", ctypes.c_void_p),
        ("tri_distance", ctypes.c_void_p),
        ("tri_bary", ctypes.c_void_p),
    ]


class MfemRefineMesh(ctypes.Structure):
    _fields_ = [
        ("max_particles", ctypes.c_int32),
        ("max_tets", ctypes.c_int32),
        ("max_tris", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("tet_indices", ctypes.c_void_p),
        ("tet_poses", ctypes.c_void_p),
        ("tet_materials", ctypes.c_void_p),
        ("tet_stretch", ctypes.c_void_p),
        ("tet_lambda", ctypes.c_void_p),
        ("rest_q", ctypes.c_void_p),
        ("particle_mass", ctypes.c_void_p),
        ("particle_inv_mass", ctypes.c_void_p),
        ("tri_indices", ctypes.c_void_p),
        ("counts", ctypes.c_void_p),
    ]


class MfemError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{message} (status {code})")
        self.code = code


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_F32 = ctypes.c_float

_SIGNATURES = {
    "mfem_config_default": (None, [ctypes.POINTER(MfemConfig)]),
    "mfem_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "mfem_kernel_launch_count": (ctypes.c_uint64, []),
    "mfem_bsr_sparsity": (ctypes.c_int, [_I32, _I32, _P, _P, _P, ctypes.POINTER(_I64)]),
    "mfem_tet_slot_map": (ctypes.c_int, [_I32, _I32, _P, _P, _P, _P]),
    "mfem_plan_create": (ctypes.c_int, [ctypes.POINTER(MfemConfig), _I32, _I32, _P, _P, _P, _P, _P, _P, _P, _I32,
                                        ctypes.POINTER(_P)]),
    "mfem_plan_destroy": (None, [_P]),
    "mfem_plan_last_error": (ctypes.c_char_p, [_P]),
    "mfem_plan_sizes": (ctypes.c_int, [_P, ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(_I64)]),
    "mfem_plan_buffer_bytes": (ctypes.c_int, [_P, _I32, ctypes.POINTER(ctypes.c_size_t)]),
    "mfem_plan_pcg_layout": (ctypes.c_int, [_P, ctypes.POINTER(_I32), ctypes.POINTER(_I32), ctypes.POINTER(_I32),
                                            ctypes.POINTER(_I64)]),
    "mfem_plan_copy_out": (ctypes.c_int, [_P, _I32, _P, ctypes.c_size_t, _P]),
    "mfem_plan_copy_in": (ctypes.c_int, [_P, _I32, _P, ctypes.c_size_t, _P]),
    "mfem_step": (ctypes.c_int, [_P, _P, _P, _P, _P, _F32, _P]),
    "mfem_step_stats": (ctypes.c_int, [_P, ctypes.POINTER(MfemSolveStats), _I32, ctypes.POINTER(_I32), _P]),
    "mfem_step_line_search_stats": (ctypes.c_int, [_P, ctypes.POINTER(MfemLineSearchStats), _I32,
                                                   ctypes.POINTER(_I32), _P]),
    "mfem_contact_config_default": (None, [ctypes.POINTER(MfemContactConfig)]),
    "mfem_plan_set_contact": (ctypes.c_int, [_P, ctypes.POINTER(MfemContactConfig), _I32, _P, _P, _P, _P, _P, _I32,
                                             _I32, _P]),
    "mfem_set_body_poses": (ctypes.c_int, [_P, _P, _I32, _P]),
    "mfem_solver_config_default": (None, [ctypes.POINTER(MfemSolverConfig)]),
    "mfem_plan_set_solver": (ctypes.c_int, [_P, ctypes.POINTER(MfemSolverConfig)]),
    "mfem_step_mixed_stats": (ctypes.c_int, [_P, ctypes.POINTER(MfemMixedSolveStats), _I32, ctypes.POINTER(_I32),
                                             _P]),
    "mfem_plan_set_bodies": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P]),
    "mfem_plan_set_factor_net": (ctypes.c_int, [_P, _P, _I64, _P]),
    "mfem_plan_batch_layout": (ctypes.c_int, [_P, ctypes.POINTER(_I32), ctypes.POINTER(_I32)]),
    "mfem_plan_autotune_batch": (ctypes.c_int, [_P, _P, _F32, ctypes.POINTER(ctypes.c_double), _P]),
    "mfem_step_body_stats": (ctypes.c_int, [_P, ctypes.POINTER(MfemSolveStats), _I32, ctypes.POINTER(_I32), _P]),
    "mfem_predict": (ctypes.c_int, [_P, _P, _P, _F32, _P]),
    "mfem_update_system": (ctypes.c_int, [_P, _P, _P]),
    "mfem_assemble": (ctypes.c_int, [_P, _P, _F32, _P]),
    "mfem_global_solve": (ctypes.c_int, [_P, _I32, _P]),
    "mfem_local_solve": (ctypes.c_int, [_P, _P, _P]),
    "mfem_true_residual": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), _P]),
    "mfem_plan_set_residual_check": (ctypes.c_int, [_P, _I32]),
    "mfem_plan_inject_timeout": (ctypes.c_int, [_P]),
    "mfem_plan_set_diagnostics": (ctypes.c_int, [_P, _I32]),
    "mfem_step_true_residuals": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), _I32, ctypes.POINTER(_I32),
                                                _P]),
    "mfem_refine_config_default": (None, [ctypes.POINTER(MfemRefineConfig)]),
    "mfem_refine": (ctypes.c_int, [_P, ctypes.POINTER(MfemRefineConfig), ctypes.POINTER(MfemRefineInputs), _P, _P,
                                   _P, ctypes.POINTER(MfemRefineMesh), _P]),
    "mfem_pcg_solve_noalloc": (ctypes.c_int, [_I32, _P, _P, _P, _P, _P, _P, _F32, _I32, _P, _P]),
    "mfem_train_gemm": (ctypes.c_int, [_I32, _I32, _I32, _P, _I32, _I32, _P, _I32, _I32, _P, _I32, _I32, _P, _I64,
                                       _P]),
    "mfem_train_adam": (ctypes.c_int, [_P, _P, _P, _P, _I64, _F32, _F32, _F32, _F32, _I32, _P]),
    "mfem_train_last_error": (ctypes.c_char_p, []),
}

_lib = None


def header_functions() -> list[str]:
    """Names of every function the public header declares."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mfem_[a-z0-9_]+)\s*\(", text)))


def load(path: Path | str | None = None) -> ctypes.CDLL:
    """Loads the library (once) and declares every entry point's signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def status_string(code: int) -> str:
    return load().mfem_status_string(code).decode()


def check(code: int, plan=None) -> int:
    """Raises MfemError for error codes (>= MFEM_NONFINITE)."""
    if code >= MFEM_NONFINITE:
        msg = load().mfem_plan_last_error(plan).decode() or status_string(code)
        raise MfemError(code, msg)
    return code


def default_config() -> MfemConfig:
    cfg = MfemConfig()
    load().mfem_config_default(ctypes.byref(cfg))
    return cfg


def kernel_launch_count() -> int:
    return int(load().mfem_kernel_launch_count())
