"""The C ABI from C: a plain C program (tests/c_abi/step_client.c), built
with gcc against include/mfem_gb300.h, libmfem_gb300.so and the CUDA runtime,
steps the cantilever with the default configuration (line search on, CUDA
graphs) on buffers it allocates itself.  Its positions and PCG iteration
counts equal those of the Python binding bit for bit: both drive the same
plan through the same entry points."""
import os
import shutil
import subprocess

import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib, beams

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def cuda_home():
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "include", "cuda_runtime_api.h")):
            return root
    pytest.skip("CUDA toolkit headers not found")


def test_c_client_matches_python_binding(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    cuda = cuda_home()
    lib_dir = os.path.dirname(str(_lib.LIB_PATH))
    exe = tmp_path / "step_client"
    libdirs = [os.path.join(cuda, d) for d in ("lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib")
               if os.path.exists(os.path.join(cuda, d))]
    cmd = ["gcc", "-O2", "-std=c99", os.path.join(HERE, "c_abi", "step_client.c"), "-o", str(exe),
           "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"), "-L", lib_dir,
           "-lmfem_gb300", f"-Wl,-rpath,{lib_dir}"]
    for d in libdirs:
        cmd += ["-L", d, f"-Wl,-rpath,{d}"]
    cmd += ["-lcudart"]
    subprocess.run(cmd, check=True)

    mesh = beams.build_beam("cantilever")
    steps = 5
    head = np.array([mesh.n, mesh.T, steps, _lib.ENERGY[mesh.spec.energy]], dtype=np.int32)
    with open(tmp_path / "mesh.bin", "wb") as f:
        head.tofile(f)
        np.array([mesh.spec.dt], dtype=np.float32).tofile(f)
        for a in (mesh.rest_q, mesh.particle_mass, mesh.particle_inv_mass):
            np.ascontiguousarray(a, dtype=np.float32).tofile(f)
        np.ascontiguousarray(mesh.tet_indices, dtype=np.int32).tofile(f)
        for a in (mesh.tet_poses, mesh.tet_materials, mesh.gravity):
            np.ascontiguousarray(a, dtype=np.float32).tofile(f)
    subprocess.run([str(exe), str(tmp_path / "mesh.bin"), str(tmp_path / "out.bin")], check=True)
    raw = np.fromfile(tmp_path / "out.bin", dtype=np.float32)
    q_c = raw[:3 * mesh.n].reshape(-1, 3)
    its_c = raw[3 * mesh.n:].view(np.int32)

    model = Model.from_beam(mesh, device="cuda:0")
    solver = MixedFEMSolver(model, iterations=8, energy=mesh.spec.energy)
    A, B = model.state(), model.state()
    for _ in range(steps):
        solver.step(A, B, None, None, mesh.spec.dt)
        A, B = B, A
    q_py = A.particle_q.cpu().numpy()
    its_py = np.array([s["iterations"] for s in solver.solve_stats()], dtype=np.int32)
    np.testing.assert_array_equal(q_c, q_py)
    np.testing.assert_array_equal(its_c, its_py)
