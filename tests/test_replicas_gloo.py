"""The multi-GPU path of bench.py runs independent replicas (the global step
does not shard); these CPU tests run its cross-rank logic on a world of two
gloo ranks: the job time is the maximum over ranks, the job rate counts the
steps of every rank, and the reference arm's non-zero ranks exit without
work."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.0 + rank, world)     # rank 1 is the slow one
        rate = bench.job_rate(10, world, t)
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump({"t": t, "rate": rate}, f)
    finally:
        dist.destroy_process_group()


def test_job_time_is_max_over_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        d = json.load(open(tmp_path / f"r{r}.json"))
        assert d["t"] == pytest.approx(2.0)
        assert d["rate"] == pytest.approx(2 * 10 / 2.0)


def test_single_rank_helpers():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_rate(50, 1, 2.0) == 25.0
    assert bench.pcg_bytes_per_iteration(262_177, 18_785) == 40 * 262_177 + 172 * 18_785


def test_reference_arm_nonzero_rank_exits_without_work():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1")
    proc = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                          capture_output=True, text=True, env=env, timeout=300)
    assert proc.returncode == 0, proc.stderr
    assert proc.stdout.strip() == ""
