"""The OpenMP CPU restatement of the step (oracle/cpu_step.cpp, the timed CPU
baseline) against the float64 numpy oracle: positions within 1e-5 of the
largest position, the GPU path's own bar."""
import numpy as np
import pytest

from mfem_gb300 import beams
from oracle import mfem_oracle as O

cpu_step = pytest.importorskip("oracle.cpu_step")


@pytest.mark.parametrize("name,cells,steps", [("cantilever", None, 5), ("nh_beam", (16, 4, 4), 2)])
def test_cpu_step_matches_oracle(name, cells, steps):
    try:
        cpu_step.build()
    except RuntimeError as e:  # no g++ / OpenMP here
        pytest.skip(str(e))
    mesh = beams.build_beam(name, cells=cells)
    cs = cpu_step.CpuStep(mesh, threads=2)
    ref = O.OracleSolver(mesh, dtype=np.float64)
    q, qd = mesh.q0, mesh.qd0
    rq, rqd = mesh.q0, mesh.qd0
    for _ in range(steps):
        q, qd = cs.step(q, qd, mesh.spec.dt)
        rq, rqd = ref.step(rq, rqd, mesh.spec.dt)
        assert (cs.last_iterations > 0).any()
        err = np.abs(q - rq).max() / np.abs(rq).max()
        assert err <= 1e-5, err
    assert cs.threads >= 1
