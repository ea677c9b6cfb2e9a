"""ctypes binding and build recipe of the OpenMP CPU restatement of the step
(oracle/cpu_step.cpp).

Test and measurement infrastructure: bench.py times it as the CPU baseline
(kind "port": the reference's own Warp path cannot run here) and
tests/test_cpu_step.py checks it against the float64 numpy oracle.  Nothing
in the library imports it.

Build:  python -m oracle.cpu_step   (g++ -O3 -fopenmp, into oracle/_build/)
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpu_step.cpp")
LIB = os.path.join(HERE, "_build", "libcpu_step.so")
INCLUDE = os.path.join(ROOT, "warp-mfem_gb300", "csrc")


def build(force: bool = False) -> str:
    """Compiles libcpu_step.so if it is missing or older than its sources."""
    deps = [SRC, os.path.join(INCLUDE, "element_math.cuh")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC", f"-I{INCLUDE}", SRC, "-o", LIB + ".tmp"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"building the CPU step failed:\n{' '.join(cmd)}\n{proc.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        lib.cpu_step_create.restype = P
        lib.cpu_step_create.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_float, ctypes.c_int, ctypes.c_float]
        lib.cpu_step_destroy.argtypes = [P]
        lib.cpu_step_threads.restype = ctypes.c_int
        lib.cpu_step_set_threads.argtypes = [ctypes.c_int]
        lib.cpu_step_run.restype = ctypes.c_int
        lib.cpu_step_run.argtypes = [P, P, P, P, P, ctypes.c_float, P]
        _lib = lib
    return _lib


class CpuStep:
    """The step of one mesh (a beams.BeamMesh or anything with its fields) on
    `threads` host threads (default: OpenMP's, all cores)."""

    def __init__(self, mesh, iterations=None, energy=None, cg_tolerance=None, cg_max_iterations=None,
                 attachment_stiffness=10.0, threads=0):
        spec = mesh.spec
        self._lib = load()
        self._lib.cpu_step_set_threads(int(threads))
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
        self._keep = dict(tets=np.ascontiguousarray(mesh.tet_indices, dtype=np.int32), poses=f32(mesh.tet_poses),
                          mats=f32(mesh.tet_materials), rest=f32(mesh.rest_q), mass=f32(mesh.particle_mass),
                          inv_mass=f32(mesh.particle_inv_mass), gravity=f32(mesh.gravity))
        k = self._keep
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self.n, self.T = int(mesh.n), int(mesh.T)
        self.iterations = spec.iterations if iterations is None else iterations
        energy = spec.energy if energy is None else energy
        self._h = self._lib.cpu_step_create(
            self.n, self.T, P(k["tets"]), P(k["poses"]), P(k["mats"]), P(k["rest"]), P(k["mass"]),
            P(k["inv_mass"]), P(k["gravity"]), self.iterations, 0 if energy == "arap" else 1,
            spec.cg_tolerance if cg_tolerance is None else cg_tolerance,
            spec.cg_max_iterations if cg_max_iterations is None else cg_max_iterations, attachment_stiffness)
        if not self._h:
            raise ValueError("cpu_step_create rejected the mesh")
        self.last_iterations = np.zeros(self.iterations, dtype=np.int32)

    @property
    def threads(self) -> int:
        return int(self._lib.cpu_step_threads())

    def step(self, q, qd, dt):
        q = np.ascontiguousarray(q, dtype=np.float32)
        qd = np.ascontiguousarray(qd, dtype=np.float32)
        qo = np.empty_like(q)
        qdo = np.empty_like(q)
        P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        self._lib.cpu_step_run(self._h, P(q), P(qd), P(qo), P(qdo), float(dt), P(self.last_iterations))
        return qo, qdo

    def close(self):
        if self._h:
            self._lib.cpu_step_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
