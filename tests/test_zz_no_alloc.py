"""The allocation-free PCG entry point, mfem_pcg_solve_noalloc.

Callers that cannot allocate device memory when they solve (a framework's
caching allocator owns the GPU heap, or the host forbids allocation after
start-up) pass their own arrays to this entry point; its scratch lives in a
fixed array inside the library.  These tests call it through the C ABI on
systems assembled by a plan and compare its solution with the plan's own
global solve (mfem_global_solve) within the PCG-solution tolerance the parity
tests use (1e-4 of the largest component), on two calls in a row.

This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

from mfem_gb300 import Model, MixedFEMSolver, _lib, beams

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
MAX_ROWS = 32768


def _assembled(name, cells, seed):
    """An assembled system (H, g, block-Jacobi inverse, warm start) of a
    deformed beam and the plan's PCG solution of it."""
    mesh = beams.build_beam(name, cells=cells)
    model = Model.from_beam(mesh, device=DEV)
    solver = MixedFEMSolver(model, iterations=8, energy=mesh.spec.energy, line_search=False)
    rng = np.random.default_rng(seed)
    x = torch.as_tensor((mesh.q0 + rng.normal(0, 0.01, mesh.q0.shape)).astype(np.float32), device=DEV)
    q = torch.as_tensor(mesh.q0, device=DEV)
    solver.predict(q, torch.zeros_like(q), mesh.spec.dt)
    solver.update_system(x)
    solver.assemble(x, mesh.spec.dt)
    sysd = dict(
        n=mesh.n, row_ptr=solver.read_buffer("row_ptr"), col_idx=solver.read_buffer("col_idx"),
        values=solver.read_buffer("h_values"), precond=solver.read_buffer("precond"),
        rhs=solver.read_buffer("rhs"), x0=solver.read_buffer("dx"))
    solver.global_solve(0)
    stats = solver.solve_stats()
    assert stats[0]["status"] == 0
    sysd["x_ref"] = solver.read_buffer("dx")
    torch.cuda.synchronize()
    sysd["solver"] = solver  # keep the plan (and its buffers) alive
    return sysd


def _solve_noalloc(lib, sysd, tol=1e-6, maxiter=1000):
    x = sysd["x0"].clone()
    stats = torch.zeros(4, dtype=torch.int32, device=DEV)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    rc = lib.mfem_pcg_solve_noalloc(
        sysd["n"], P(sysd["row_ptr"]), P(sysd["col_idx"]), P(sysd["values"]), P(sysd["precond"]),
        P(sysd["rhs"]), P(x), tol, maxiter, P(stats), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.MFEM_OK, lib.mfem_plan_last_error(None).decode()
    torch.cuda.synchronize()
    st = stats.cpu().numpy()
    return x, dict(iterations=int(st[0]), status=int(st[1]), rel_residual=float(st[2:3].view(np.float32)[0]))


def _close(a, b, rtol):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    err = np.abs(a - b).max()
    assert err <= rtol * np.abs(b).max(), f"max err {err:.3e} vs scale {np.abs(b).max():.3e}"


def test_noalloc_solve_matches_plan_solve_on_two_calls():
    lib = _lib.load()
    systems = [_assembled("cantilever", None, 3), _assembled("nh_beam", (16, 4, 4), 4)]
    # two calls in a row, on systems of different sizes
    for sysd in systems:
        x, st = _solve_noalloc(lib, sysd)
        assert st["status"] == _lib.MFEM_OK and st["iterations"] > 0, st
        assert st["rel_residual"] <= 1e-6, st
        _close(x, sysd["x_ref"], 1e-4)
    # the same system twice more: the shared scratch carries nothing over
    a, sa = _solve_noalloc(lib, systems[0])
    b, sb = _solve_noalloc(lib, systems[0])
    assert torch.equal(a, b) and sa == sb
    _close(a, systems[0]["x_ref"], 1e-4)


def test_noalloc_call_leaves_free_device_memory_unchanged():
    """The property the entry point exists for: after a warm-up call, a call
    changes the device's free memory (cudaMemGetInfo) by nothing, so it
    allocated nothing.  Every tensor the call touches exists before the
    first reading."""
    lib = _lib.load()
    sysd = _assembled("nh_beam", (16, 4, 4), 5)
    x = sysd["x0"].clone()
    stats = torch.zeros(4, dtype=torch.int32, device=DEV)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call():
        x.copy_(sysd["x0"])
        rc = lib.mfem_pcg_solve_noalloc(sysd["n"], P(sysd["row_ptr"]), P(sysd["col_idx"]), P(sysd["values"]),
                                        P(sysd["precond"]), P(sysd["rhs"]), P(x), 1e-6, 1000, P(stats), stream)
        assert rc == _lib.MFEM_OK, lib.mfem_plan_last_error(None).decode()
        torch.cuda.synchronize()

    call()  # warm-up: the module and its scratch array are loaded by now
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(3):
        call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    assert torch.cuda.memory_reserved() == reserved0
    _close(x, sysd["x_ref"], 1e-4)


def test_noalloc_rejects_oversized_and_invalid_arguments():
    lib = _lib.load()
    dummy = torch.zeros(16, dtype=torch.float32, device=DEV)
    P = ctypes.c_void_p(dummy.data_ptr())
    rc = lib.mfem_pcg_solve_noalloc(MAX_ROWS + 1, P, P, P, None, P, P, 1e-6, 10, None, None)
    assert rc == _lib.MFEM_BAD_ARG
    assert str(MAX_ROWS) in lib.mfem_plan_last_error(None).decode()
    rc = lib.mfem_pcg_solve_noalloc(10, None, P, P, None, P, P, 1e-6, 10, None, None)
    assert rc == _lib.MFEM_BAD_ARG
    rc = lib.mfem_pcg_solve_noalloc(0, P, P, P, None, P, P, 1e-6, 10, None, None)
    assert rc == _lib.MFEM_BAD_ARG
