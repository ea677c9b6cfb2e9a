#!/usr/bin/env python
"""Step-rate benchmark of the GB300 global step.

Workload: the Neo-Hookean beam (64x16x16 hex cells, 6 tets each: 98,304 tets,
18,785 vertices), 8 local/global iterations per implicit-Euler step, plain
float32 block-Jacobi PCG to 1e-6 relative residual.  A "step" is one solver
step; the timed run is the workload's 50 steps from its initial state.

  value  steps/s with the state resident on the GPU (CUDA-graph replays),
         L2 flushed between steps outside the timed events.
  e2e    the same steps through the public solver API with the state in
         pinned host memory: H2D copy of (q, qd), step, D2H copy of (q, qd).
  roofline  the persistent PCG kernel (the dominant kernel), from an eager
         stage-by-stage pass timed with CUDA events on the launch stream.

--workload batched512 steps the batch of 512 uneven beams (per-body PCGs in
one persistent launch): value = batch steps/s (every body advanced one step).

--impl reference times the OpenMP C++ restatement of the step
(oracle/cpu_step.cpp) on all host cores instead: the reference's own Warp
path cannot run here.  With --gpus N under torchrun every rank runs an
independent replica (the step does not shard across GPUs).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "warp-mfem_gb300"), ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "steps/s to 1e-6 rel. residual: learned+mixed PCG vs plain FP32 PCG, same GB300"
FALLBACK_HBM_GBS = 6800.0
L2_FLUSH_BYTES = 512 << 20


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", default="nh_beam")
    ap.add_argument("--profile-steps", type=int, default=10, help="steps of the eager stage profile")
    ap.add_argument("--pcg-ctas", type=int, default=0, help="persistent PCG CTAs (0: one per SM)")
    ap.add_argument("--pcg-variant", default="auto",
                    choices=["auto", "standard", "single_reduction", "gather", "factor", "global_memory"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "bf16", "fp16", "fp32_refined"],
                    help="global solve: fp32 PCG (the workload's) or fp64 iterative refinement around an "
                         "inner PCG on 16-bit (bf16, fp16) or fp32 (fp32_refined) blocks")
    ap.add_argument("--outer-tolerance", type=float, default=1.0e-6,
                    help="fp64 relative residual of the mixed-precision solve")
    ap.add_argument("--inner-tolerance", type=float, default=1.0e-3,
                    help="relative residual of the mixed-precision solve's inner PCG")
    ap.add_argument("--outer-max-iterations", type=int, default=10,
                    help="corrections of the mixed-precision solve before it reports MAXITER")
    ap.add_argument("--preconditioner", default="block_jacobi", choices=["block_jacobi", "fsai", "learned"],
                    help="PCG preconditioner: the workload's block-Jacobi, or the FSAI / learned factor "
                         "(global-memory PCG)")
    ap.add_argument("--factor-refresh", type=int, default=1,
                    help="factor preconditioners: recompute the factor every this many Newton iterations")
    ap.add_argument("--line-search", action="store_true",
                    help="run the workload with the reference's backtracking line search")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the solve variants (learned / FSAI factors, fp16) of the default line")
    ap.add_argument("--no-extra-workloads", action="store_true",
                    help="skip the stiff_beam and batched512 entries of the default line")
    ap.add_argument("--cpu-budget-s", type=float, default=30.0, help="CPU time budget of the oracle leg")
    ap.add_argument("--variant-inner-tolerance", type=float, default=1.0e-2,
                    help="inner PCG tolerance of the refined solve variants of the default line")
    return ap.parse_args()


def workload_config(mesh, extra=None, precision="fp32", outer_tolerance=1e-6, preconditioner="block_jacobi",
                    factor_refresh=1, pcg_variant="global_memory", inner_tolerance=1e-3):
    spec = mesh.spec
    if precision == "fp32" and preconditioner == "block_jacobi":
        pcg = "plain fp32 block-Jacobi, the reference's (persistent PCG)"
    elif precision == "fp32":
        kind = "persistent factor PCG" if pcg_variant == "factor" else "global-memory PCG"
        pcg = (f"fp32 PCG with the {preconditioner} factor preconditioner ({kind}), factor recomputed "
               f"every {factor_refresh} Newton iteration(s)")
    else:
        pcg = (f"{precision} blocks with per-row scales, fp32 {preconditioner} inner PCG to {inner_tolerance:g}, "
               f"fp64 iterative refinement to {outer_tolerance:g}")
    cfg = {
        "workload": (f"{spec.name}: {spec.cells[0]}x{spec.cells[1]}x{spec.cells[2]} hex cells x 6 tets "
                     f"({mesh.T} tets, {mesh.n} vertices, {3 * mesh.n} DoF), {spec.energy}, "
                     f"E log-uniform [{spec.E[0]:.0e}, {spec.E[1]:.0e}] Pa (seed {spec.seed}), nu {spec.nu}, "
                     f"rho {spec.density:g}, dt 1/{round(1 / spec.dt)}, {spec.iterations} local/global iterations, "
                     f"block-Jacobi fp32 PCG to {spec.cg_tolerance:g}"),
        "tets": mesh.T,
        "vertices": mesh.n,
        "steps_per_run": spec.steps,
        "pcg": pcg,
        "parallelism": "replicas",
        "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MiB write, outside the timed events)",
    }
    if extra:
        cfg.update(extra)
    return cfg


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        power = [float(r[3]) for r in rows if re.match(r"^[0-9.]+$", r[3])]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "power_w_max": max(power) if power else None}


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------
def hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback 6.8 TB/s"


def ncu_traffic_per_launch(summary="pcg_kernel_nh_beam.md"):
    """DRAM bytes (read + write) of one PCG launch from the committed ncu
    summary of this workload (profiles/<summary>)."""
    path = os.path.join(ROOT, "profiles", summary)
    try:
        text = open(path).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", text)
    return float(m.group(1)) if m else None


def max_over_ranks(seconds: float, world: int, device=None) -> float:
    """Largest per-rank time of the job (a no-op on one rank)."""
    if world <= 1:
        return seconds
    import torch
    import torch.distributed as dist
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(steps_per_rank: int, world: int, t_max: float) -> float:
    """Whole-job steps/s of `world` independent replicas."""
    return world * steps_per_rank / t_max


def pcg_bytes_per_iteration(nnzb: int, n: int) -> int:
    """Algorithmic bytes of one plain fp32 PCG iteration: 36 B values + 4 B
    column index per block; per row 4 B row pointer + 24 B (read p, write Ap)
    + 48 B (read x, p, r, Ap) + 36 B block-Jacobi block + 36 B (write x, r, z)
    + 36 B (read z, p, write p) = 40 nnzb + 172 n."""
    return 40 * nnzb + 172 * n


def host_cpu() -> dict:
    """This host's core count and CPU model (lscpu, else /proc/cpuinfo)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        m = re.search(r"^Model name:\s*(.+)$", out, re.M)
        model = m.group(1).strip() if m else None
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None:
        try:
            m = re.search(r"^model name\s*:\s*(.+)$", open("/proc/cpuinfo").read(), re.M)
            model = m.group(1).strip() if m else None
        except OSError:
            pass
    return {"nproc": os.cpu_count(), "model": model}


def cpu_step_rate(mesh, budget_s: float, max_steps: int):
    """Steps/s of the OpenMP C++ restatement of the step (oracle/cpu_step.cpp)
    on all host cores, from the workload's initial state: at least one step,
    more while within budget, at most max_steps.  Returns (rate, steps,
    seconds, threads)."""
    from oracle import cpu_step
    cs = cpu_step.CpuStep(mesh)
    q, qd = mesh.q0, mesh.qd0
    t0 = time.perf_counter()
    steps = 0
    while True:
        q, qd = cs.step(q, qd, mesh.spec.dt)
        steps += 1
        el = time.perf_counter() - t0
        if el * (steps + 1) / steps > budget_s or steps >= max_steps:
            break
    threads = cs.threads
    cs.close()
    return steps / el, steps, el, threads


def cpu_baseline_line(mesh, budget_s: float, max_steps: int, workload: str) -> dict:
    rate, steps, el, threads = cpu_step_rate(mesh, budget_s, max_steps)
    cpu = host_cpu()
    return {"value": rate, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": (f"{steps} step(s) of {workload} ({mesh.T} tets, {mesh.spec.iterations} local/global "
                       f"iterations each) from its initial state by the OpenMP C++ restatement of the step "
                       f"(oracle/cpu_step.cpp, float32, block-Jacobi PCG to 1e-6; restatement, not the "
                       f"reference) on {threads} threads in {el:.1f} s"),
            "host": cpu}


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    from mfem_gb300 import beams
    if rank != 0:
        return 0
    if args.workload.startswith("batched"):
        return run_reference_batched(args)
    mesh = beams.build_beam(args.workload)
    # one untimed step pages the code and data in; the timed run is the
    # workload's first --steps steps from its initial state, like the GPU
    # arm's, within a budget of a few minutes
    cpu_step_rate(mesh, 0.0, 1)
    cpu = cpu_baseline_line(mesh, 180.0, max(1, args.steps), args.workload)
    rate, steps = cpu["value"], int(re.match(r"(\d+)", cpu["sample"]).group(1))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": 1, "ms_per_step": 1000.0 / rate, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(mesh, {"reference": "OpenMP C++ restatement of the step on all host cores "
                                                      "(the reference's Warp path cannot run: warp-lang / newton "
                                                      "absent, Python >= 3.13 required)"}),
        "cpu_baseline": cpu,
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# batch of independent bodies
# ---------------------------------------------------------------------------
def batched_count(workload: str) -> int:
    return int(workload[len("batched"):] or 512)


def run_batched(args, rank, world, local_rank):
    import numpy as np
    import torch
    from mfem_gb300 import beams, _lib
    from mfem_gb300.batched import BatchedSolver

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    B = batched_count(args.workload)
    batch = beams.batched_bodies(B, seed=4)
    u = batch.union
    fsai = args.preconditioner in ("fsai", "learned")  # a factor preconditioner
    bs = BatchedSolver(batch, device=dev, preconditioner=args.preconditioner, factor_refresh=args.factor_refresh)
    tune_ms = bs.autotune()
    layout = bs.layout()
    s_init = bs.solver.tet_stretch.clone().reshape(-1)
    lam0 = torch.zeros_like(s_init)
    q0 = torch.as_tensor(u.q0, device=dev)
    A, Bst = bs.model.state(), bs.model.state()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def reset():
        A.particle_q.copy_(q0)
        A.particle_qd.zero_()
        bs.solver.write_buffer("tet_stretch", s_init)
        bs.solver.write_buffer("tet_lambda", lam0)

    reset()
    for _ in range(args.warmup):
        bs.step(A, Bst)
        A, Bst = Bst, A
    torch.cuda.synchronize(dev)
    reset()
    sampler = ClockSampler(local_rank)
    torch.cuda.synchronize(dev)
    sampler.start()
    launches0 = _lib.kernel_launch_count()
    total_ms = 0.0
    its = []
    statuses = set()
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bs.step(A, Bst)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        st = bs.body_stats()
        its.append(st["iterations"])
        statuses.update(int(x) for x in np.unique(st["status"]))
        A, Bst = Bst, A
    launches = _lib.kernel_launch_count() - launches0
    torch.cuda.synchronize(dev)
    clocks = sampler.stop()
    t_max = max_over_ranks(total_ms / 1000.0, world, dev)
    value = job_rate(args.steps, world, t_max)
    q_final = A.particle_q.cpu().numpy()

    # e2e: host-resident union state through the public API
    reset()
    hq = torch.empty((u.n, 3), dtype=torch.float32, pin_memory=True)
    hqd = torch.empty_like(hq, pin_memory=True)
    hq.copy_(q0.cpu())
    hqd.zero_()
    e2e_ms = 0.0
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        A.particle_q.copy_(hq, non_blocking=True)
        A.particle_qd.copy_(hqd, non_blocking=True)
        bs.step(A, Bst)
        hq.copy_(Bst.particle_q, non_blocking=True)
        hqd.copy_(Bst.particle_qd, non_blocking=True)
        e1.record(stream)
        e1.synchronize()
        e2e_ms += e0.elapsed_time(e1)
    e2e_s = max_over_ranks(e2e_ms / 1000.0, world, dev)
    e2e_value = job_rate(args.steps, world, e2e_s)
    state_bytes = 2 * u.n * 3 * 4

    # roofline of the batched PCG: eager stages of a few steps
    reset()
    solver = bs.solver
    pcg_ms = 0.0
    assemble_ms = 0.0
    solves = 0
    bytes_pcg = 0.0
    row_ptr = solver.read_buffer("row_ptr").cpu().numpy()
    voff = batch.vertex_offsets
    nnzb_b = (row_ptr[voff[1:]] - row_ptr[voff[:-1]]).astype(np.float64)
    n_b = np.diff(voff).astype(np.float64)
    # a factor preconditioner replaces the 36 n bytes of block-Jacobi blocks
    # by two passes over the factor's nnzl = (nnzb + n)/2 blocks (20 B BF16
    # block + 4 B column each, plus the pass's 12 B vector in and 12 B out
    # per row): 40 nnzb + 136 n + 24 (nnzb + n) + 48 n
    per_it_b = (64.0 * nnzb_b + 208.0 * n_b) if fsai else (40.0 * nnzb_b + 172.0 * n_b)
    x = Bst.particle_q
    prof_steps = max(1, min(3, args.steps))
    for _ in range(prof_steps):
        flush.zero_()
        solver.predict(A.particle_q, A.particle_qd, batch.dt)
        x.copy_(A.particle_q)
        for it in range(solver.iterations):
            solver.update_system(x)
            ea = torch.cuda.Event(enable_timing=True)
            ea.record(stream)
            solver.assemble(x, batch.dt)  # with a factor preconditioner: its setup too
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            solver.global_solve(it)
            e1.record(stream)
            solver.local_solve(x)
            e1.synchronize()
            pcg_ms += e0.elapsed_time(e1)
            assemble_ms += ea.elapsed_time(e0)
            solves += 1
        st = bs.body_stats()
        bytes_pcg += float(((st["iterations"].astype(np.float64) + 1.0) * per_it_b[None, :]).sum())
        Bst.particle_qd.copy_((x - A.particle_q) / batch.dt)
        A, Bst = Bst, A
        x = Bst.particle_q
    achieved = bytes_pcg / (pcg_ms / 1000.0) / 1e9
    peak, peak_src = hbm_peak()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None,
                "kernel": f"batched_pcg_kernel (per-body {args.preconditioner} PCGs, one launch)",
                "algorithmic_bytes_per_launch": bytes_pcg / solves,
                "bytes_per_body_iteration": (("64 nnzb_b + 208 n_b" if fsai else "40 nnzb_b + 172 n_b") +
                                             ", summed over bodies x (iterations_b + 1)"),
                "avg_launch_ms": pcg_ms / solves, "peak_source": peak_src}

    if rank != 0:
        return 0
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = batched_cpu_line(batch, args.cpu_budget_s)
    it_all = np.stack(its)
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": (f"{B} uneven beams in one plan (seed 4): per body nx~U{{4..48}}, ny,nz~U{{2..12}} "
                                f"hex cells of 0.05 m x 6 tets, ARAP or Neo-Hookean (p 0.5), E log-uniform [1e4, 1e6] "
                                f"Pa, nu~U[0.3, 0.48], gravity on the unit sphere, x = 0 face pinned; "
                                f"{u.T} tets, {u.n} vertices; 8 local/global iterations, per-body "
                                f"{args.preconditioner} fp32 PCG to 1e-6"),
                   "preconditioner": args.preconditioner, "factor_refresh": args.factor_refresh,
                   "bodies": B, "tets": u.T, "vertices": u.n, "pcg_schedule": layout,
                   "autotune_best_solve_ms": tune_ms, "parallelism": "replicas",
                   "l2": f"flushed between timed steps ({L2_FLUSH_BYTES >> 20} MiB write, outside the timed events)"},
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes, "matches_resident_run": bool(np.array_equal(hq.numpy(), q_final))},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "body_steps_per_s": B * value,
        "pcg_iterations_per_body_step": {"mean": float(it_all.sum(1).mean()), "max": int(it_all.sum(1).max())},
        "pcg_status_codes": sorted(statuses),
        "eager_ms_per_newton_iteration": {"assemble_and_preconditioner_setup": assemble_ms / solves,
                                          "pcg": pcg_ms / solves},
    }
    print(json.dumps(line), flush=True)
    return 0


def batched_cpu_line(batch, budget_s: float) -> dict:
    """The OpenMP C++ restatement stepping the bodies one after another from
    their initial states, within budget; batch steps/s = body steps/s /
    bodies."""
    from oracle import cpu_step
    B = batch.n_bodies
    t0 = time.perf_counter()
    done, threads = 0, 1
    for m in batch.bodies:
        cs = cpu_step.CpuStep(m)
        cs.step(m.q0, m.qd0, m.spec.dt)
        threads = cs.threads
        cs.close()
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return {"value": done / el / B, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": (f"one step of the first {done} of {B} bodies by the OpenMP C++ restatement of the step "
                       f"(oracle/cpu_step.cpp; restatement, not the reference) on {threads} threads in {el:.1f} s "
                       "(batch steps/s = body steps/s / bodies)"),
            "host": host_cpu()}


def run_reference_batched(args):
    """The C++ restatement steps the bodies one after another (a bounded
    sample); batch steps/s = body steps/s / bodies."""
    from mfem_gb300 import beams
    B = batched_count(args.workload)
    batch = beams.batched_bodies(B, seed=4)
    budget = max(10.0, min(150.0, args.cpu_budget_s * max(1, args.steps) / 10.0))
    cpu = batched_cpu_line(batch, budget)
    rate = cpu["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "steps/s", "n_gpus": args.gpus,
        "steps": 1, "warmup": 0, "ms_per_step": 1000.0 / rate, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{B} uneven beams (seed 4)", "bodies": B,
                   "reference": "OpenMP C++ restatement of the step (the reference's Warp path cannot run here)"},
        "cpu_baseline": cpu,
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GB300 arm
# ---------------------------------------------------------------------------
SOLVE_VARIANTS = (("fp32", "block_jacobi"), ("fp32", "fsai"), ("fp32", "learned"),
                  ("fp32_refined", "block_jacobi"), ("fp32_refined", "fsai"),
                  ("fp16", "block_jacobi"), ("fp16", "fsai"), ("fp16", "learned"))


def checked_summary(residuals, tol):
    """Counts of the solves whose float64 residual meets `tol`, and the
    worst and median residuals."""
    r = sorted(residuals)
    return {"solves": len(r), "meet_tolerance": sum(1 for v in r if v <= tol),
            "worst": r[-1] if r else None, "median": statistics.median(r) if r else None}


def run_checked(solver, model, q0, s_init, dt, steps):
    """The first `steps` steps from the initial state with the fp64 check of
    every global solve on (graph replays, untimed).  Returns the float64
    residuals of the float32 dx of each solve, the mixed solves' own
    residuals (of their float64 dx; empty for the fp32 PCG) and the final
    positions."""
    import torch
    st = [model.state(), model.state()]
    st[0].particle_q.copy_(q0)
    st[0].particle_qd.zero_()
    solver.write_buffer("tet_stretch", s_init)
    solver.write_buffer("tet_lambda", torch.zeros_like(s_init))
    solver.set_residual_check(True)
    res32, res_own = [], []
    for _ in range(steps):
        solver.step(st[0], st[1], None, None, dt)
        res32 += solver.step_true_residuals()
        res_own += [r["rel_residual"] for r in solver.mixed_stats()]
        st.reverse()
    q = st[0].particle_q.cpu().numpy()
    solver.set_residual_check(False)
    return res32, res_own, q


def measure_variant(mesh, dev, precision, pc, steps, warmup, inner_tolerance, outer_tolerance=None,
                    outer_max_iterations=20, factor_refresh=8, profile=False):
    """One solve variant on `mesh`: steps/s over the workload's first `steps`
    steps (graph replays, L2 flushed between steps, after `warmup` steps),
    the float64 check of every one of their solves (a separate untimed run
    with the check on, bit-identical positions), and with `profile` the
    persistent PCG's roofline from one eager step timed stage by stage."""
    import numpy as np
    import torch
    from mfem_gb300 import Model, MixedFEMSolver
    spec = mesh.spec
    tol = spec.cg_tolerance
    q0 = torch.as_tensor(mesh.q0, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    model = Model.from_beam(mesh, device=dev)
    kw = dict(iterations=spec.iterations, energy=spec.energy, cg_tolerance=tol,
              cg_max_iterations=spec.cg_max_iterations, line_search=False, preconditioner=pc,
              solver_precision=precision, outer_tolerance=tol if outer_tolerance is None else outer_tolerance,
              inner_tolerance=inner_tolerance, outer_max_iterations=outer_max_iterations)
    if pc != "block_jacobi":
        kw["factor_refresh"] = factor_refresh
    solver = MixedFEMSolver(model, **kw)
    if solver.pcg_layout()["variant"] == "global_memory":
        solver.autotune(q0, spec.dt)
    s_init = solver.tet_stretch.clone().reshape(-1)
    st = [model.state(), model.state()]

    def reset():
        st[0].particle_q.copy_(q0)
        st[0].particle_qd.zero_()
        solver.write_buffer("tet_stretch", s_init)
        solver.write_buffer("tet_lambda", torch.zeros_like(s_init))

    res32, res_own, q_checked = run_checked(solver, model, q0, s_init, spec.dt, steps)
    reset()
    for _ in range(max(2, warmup)):  # both state orientations captured before timing
        solver.step(st[0], st[1], None, None, spec.dt)
        st.reverse()
    reset()
    total_ms, its, codes = 0.0, 0, []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.step(st[0], st[1], None, None, spec.dt)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        if precision == "fp32":
            rec = solver.solve_stats()
            its += sum(r["iterations"] for r in rec)
        else:
            rec = solver.mixed_stats()
            its += sum(r["inner_iterations"] for r in rec)
        codes += [int(r["status"]) for r in rec]
        st.reverse()
    q_timed = st[0].particle_q.cpu().numpy()
    own = res_own if precision != "fp32" else res32
    out = {
        "steps_per_s": 1000.0 * steps / total_ms, "pcg_iterations_per_step": its / steps,
        "status_codes": sorted(set(codes)),
        "converged_fraction": sum(1 for c in codes if c == 0) / max(1, len(codes)),
        "pcg": ("fp64 iterative refinement" if precision != "fp32" else solver.pcg_layout()["variant"]),
        "fp64_check": {"solution": checked_summary(own, tol), "fp32_dx": checked_summary(res32, tol)},
        "checked_run_matches_timed": bool(np.array_equal(q_checked, q_timed)),
    }
    if profile and precision == "fp32":
        # one eager step, the global solves timed on the launch stream
        reset()
        x = st[1].particle_q
        solver.predict(st[0].particle_q, st[0].particle_qd, spec.dt)
        x.copy_(st[0].particle_q)
        pcg_ms = 0.0
        for it in range(spec.iterations):
            solver.update_system(x)
            solver.assemble(x, spec.dt)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            solver.global_solve(it)
            e1.record(stream)
            solver.local_solve(x)
            e1.synchronize()
            pcg_ms += e0.elapsed_time(e1)
        its1 = sum(r["iterations"] for r in solver.solve_stats())
        factor = pc != "block_jacobi"
        b_it = (64 * solver.nnzb + 208 * mesh.n) if factor else pcg_bytes_per_iteration(solver.nnzb, mesh.n)
        peak, _ = hbm_peak()
        achieved = b_it * (its1 + spec.iterations) / (pcg_ms / 1000.0) / 1e9
        out["pcg_roofline"] = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                               "frac": achieved / peak, "bytes_per_iteration": b_it,
                               "formula": "64 nnzb + 208 n" if factor else "40 nnzb + 172 n",
                               "us_per_iteration": 1000.0 * pcg_ms / (its1 + spec.iterations)}
    solver.close()
    return out


def solve_variants(mesh, dev, steps=20, warmup=2, inner_tolerance=1e-2):
    """steps/s over the workload's first `steps` steps for each solve
    variant -- the plain fp32 block-Jacobi PCG (the reference's), the FSAI
    and learned factor preconditioners, the fp32 and fp16 blocks inside the
    fp64 iterative refinement -- beside the float64 check of every one of
    their solves: how many meet the 1e-6 tolerance in the float64 residual
    ||g - H dx|| / ||g||, and the worst.  Timed runs are graph replays with the
    L2 flushed between steps; the checked run (check on, untimed) follows the
    same trajectory, which `checked_run_matches_timed` confirms bit for bit."""
    tol = mesh.spec.cg_tolerance
    out = {"steps": steps, "tolerance": tol, "factor_refresh": 8, "inner_tolerance": inner_tolerance,
           "fp64_check": ("float64 ||g - H dx|| / ||g|| of every solve, with the assembled float32 H and g: "
                          "'solution' is the solve's own output (float32 dx for the fp32 PCG, the refinement's "
                          "float64 dx for the refined solves), 'fp32_dx' the float32 dx the local solve reads")}
    for precision, pc in SOLVE_VARIANTS:
        out[f"{precision}+{pc}"] = measure_variant(mesh, dev, precision, pc, steps, warmup, inner_tolerance)

    def rate(k):
        return out[k]["steps_per_s"]

    def all_checked(k):
        c = out[k]["fp64_check"]["solution"]
        return c["meet_tolerance"] == c["solves"]

    plain, plain_checked = rate("fp32+block_jacobi"), rate("fp32_refined+block_jacobi")
    out["ratios"] = {
        "learned_mixed_over_plain": rate("fp16+learned") / plain,
        "learned_mixed_over_plain_fp64_checked": rate("fp16+learned") / plain_checked,
        "fsai_mixed_over_plain_fp64_checked": rate("fp16+fsai") / plain_checked,
        "fsai_refined_fp32_over_plain_fp64_checked": rate("fp32_refined+fsai") / plain_checked,
        "plain_meets_fp64_checked_tolerance": all_checked("fp32+block_jacobi"),
        "note": ("plain = the reference's fp32 block-Jacobi PCG, which stops on its float32 recurrence "
                 "residual; plain_fp64_checked = the same PCG inside the fp64 refinement (fp32_refined), "
                 "whose every solve meets 1e-6 in the float64 residual"),
    }
    checked = [k for k in out if isinstance(out[k], dict) and "fp64_check" in out[k] and all_checked(k)]
    if checked:
        best = max(checked, key=rate)
        out["ratios"]["fastest_fp64_checked"] = {"variant": best, "steps_per_s": rate(best),
                                                 "over_plain_fp64_checked": rate(best) / plain_checked,
                                                 "over_plain": rate(best) / plain}
    return out


def extra_workloads(dev, steps=3):
    """The other configs' step rates on the default line: the stiff beam
    (128x32x32 cells, 786,432 tets, E log-uniform [1e4, 1e7]) with the plain
    fp32 PCG, FSAI, and the fp16 / bf16 blocks in the fp64 refinement at the
    config's tolerances (inner 1e-3, outer 1e-8); and the 512 uneven bodies
    in one launch with block-Jacobi and FSAI."""
    from mfem_gb300 import beams
    out = {}
    mesh = beams.build_beam("stiff_beam")
    sb = {"steps": steps, "workload": f"stiff_beam 128x32x32 cells ({mesh.T} tets, {mesh.n} vertices)"}
    sb["fp32+block_jacobi"] = measure_variant(mesh, dev, "fp32", "block_jacobi", steps, 1, 1e-3, profile=True)
    sb["fp32+fsai"] = measure_variant(mesh, dev, "fp32", "fsai", steps, 1, 1e-3, profile=True)
    sb["fp16+block_jacobi (inner 1e-3, outer 1e-8)"] = measure_variant(mesh, dev, "fp16", "block_jacobi", steps, 1,
                                                                       1e-3, outer_tolerance=1e-8,
                                                                       outer_max_iterations=10)
    sb["fp16+fsai (inner 1e-3, outer 1e-8)"] = measure_variant(mesh, dev, "fp16", "fsai", steps, 1, 1e-3,
                                                               outer_tolerance=1e-8, outer_max_iterations=10)
    out["stiff_beam"] = sb
    del mesh
    out["batched512"] = {pc: measure_batched(dev, pc, steps) for pc in ("block_jacobi", "fsai")}
    out["refinement"] = measure_refinement(dev)
    return out


def measure_refinement(dev, strain_steps=5, repeats=5):
    """One adaptive-refinement pass on the Neo-Hookean beam after a few
    steps of strain: the device time of mfem_refine (legacy scores, tet
    weight 1, threshold 0, so every strained edge competes and the selection
    splits a maximal conflict-free set), then the host rebuild of the plan on
    the refined mesh and the step rate there."""
    import ctypes

    import torch
    from mfem_gb300 import MixedFEMSolver, Model, beams
    mesh = beams.build_beam("nh_beam")
    # a tet holds at most one split edge, so 2 T tets always suffice
    model = Model.from_beam(mesh, device=dev).pad_particles(4 * mesh.n)
    solver = MixedFEMSolver(model, iterations=mesh.spec.iterations, energy=mesh.spec.energy, line_search=False,
                            max_tets=2 * mesh.T, enable_refinement=True, refine_every_n_steps=10 ** 9,
                            refine_tet_score_weight=1.0, min_refine_score=0.0,
                            refine_density=float(mesh.spec.density))
    solver._refine_pass = 1  # no pass during the strain steps
    s0, s1 = model.state(), model.state()
    dt = mesh.spec.dt
    for _ in range(strain_steps):
        solver.step(s0, s1, None, None, dt)
        s0, s1 = s1, s0
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    q = s0.particle_q.clone()
    qd = s0.particle_qd.clone()
    call = lambda: solver._lib.mfem_refine(solver._plan, ctypes.byref(solver.refine_config), None,
                                           ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(qd.data_ptr()), None,
                                           ctypes.byref(solver._rmesh_struct), ctypes.c_void_p(stream.cuda_stream))
    assert call() == 0  # builds the edge lists
    times = []
    for _ in range(repeats):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        assert call() == 0
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    counts = solver._rmesh["counts"].cpu().tolist()
    T0, n0 = solver.active_tet_count, solver.active_particle_count
    s1.assign(s0)
    solver._refine_pass = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    solver._refine(s0, s1)
    torch.cuda.synchronize()
    rebuild_s = time.perf_counter() - t0
    s0.assign(s1)
    solver._refine_pass = 1
    for _ in range(2):
        solver.step(s0, s1, None, None, dt)
        s0, s1 = s1, s0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(strain_steps):
        solver.step(s0, s1, None, None, dt)
        s0, s1 = s1, s0
    torch.cuda.synchronize()
    rate = strain_steps / (time.perf_counter() - t0)
    finite = bool(torch.isfinite(s0.particle_q[:solver.active_particle_count]).all().item())
    return {"workload": f"nh_beam after {strain_steps} steps, legacy scores (tet weight 1, threshold 0), "
                        "5 selection sweeps",
            "pass_ms": statistics.median(times), "pass_ms_all": times, "split_edges": int(counts[3]),
            "tets": [T0, int(counts[1])], "vertices": [n0, int(counts[0])],
            "rebuild_ms": 1000.0 * rebuild_s,
            "rebuild": "host: copy the refined mesh back, build a new plan (sparsity, slot maps, PCG layout), "
                       "carry s and lambda over",
            "refined_steps_per_s": rate, "refined_state_finite": finite}


def measure_batched(dev, pc, steps, B=512):
    """Batch steps/s of the B uneven bodies (seed 4) in one plan after the
    autotuner, and the batched PCG's roofline from one eager step."""
    import numpy as np
    import torch
    from mfem_gb300 import beams
    from mfem_gb300.batched import BatchedSolver
    batch = beams.batched_bodies(B, seed=4)
    kw = {"preconditioner": pc}
    if pc != "block_jacobi":
        kw["factor_refresh"] = 8
    bs = BatchedSolver(batch, device=dev, **kw)
    bs.autotune()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    A, Bst = bs.state(), bs.model.state()
    q0 = A.particle_q.clone()
    s_init = bs.solver.tet_stretch.clone().reshape(-1)

    def reset():
        A.particle_q.copy_(q0)
        A.particle_qd.zero_()
        bs.solver.write_buffer("tet_stretch", s_init)
        bs.solver.write_buffer("tet_lambda", torch.zeros_like(s_init))

    for _ in range(2):  # both state orientations captured before timing
        bs.step(A, Bst)
        A, Bst = Bst, A
    reset()
    total_ms, codes, its = 0.0, set(), []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bs.step(A, Bst)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        st = bs.body_stats()
        codes.update(int(c) for c in np.unique(st["status"]))
        its.append(st["iterations"].sum(0))
        A, Bst = Bst, A
    # roofline: one eager step's global solves
    solver = bs.solver
    row_ptr = solver.read_buffer("row_ptr").cpu().numpy()
    voff = batch.vertex_offsets
    nnzb_b = (row_ptr[voff[1:]] - row_ptr[voff[:-1]]).astype(np.float64)
    n_b = np.diff(voff).astype(np.float64)
    factor = pc != "block_jacobi"
    per_it_b = (64.0 * nnzb_b + 208.0 * n_b) if factor else (40.0 * nnzb_b + 172.0 * n_b)
    reset()
    x = Bst.particle_q
    solver.predict(A.particle_q, A.particle_qd, batch.dt)
    x.copy_(A.particle_q)
    pcg_ms = 0.0
    for it in range(solver.iterations):
        solver.update_system(x)
        solver.assemble(x, batch.dt)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.global_solve(it)
        e1.record(stream)
        solver.local_solve(x)
        e1.synchronize()
        pcg_ms += e0.elapsed_time(e1)
    st = bs.body_stats()
    bytes_pcg = float(((st["iterations"].astype(np.float64) + 1.0) * per_it_b[None, :]).sum())
    peak, _ = hbm_peak()
    achieved = bytes_pcg / (pcg_ms / 1000.0) / 1e9
    it_all = np.stack(its)
    return {"batch_steps_per_s": 1000.0 * steps / total_ms, "body_steps_per_s": B * 1000.0 * steps / total_ms,
            "steps": steps, "status_codes": sorted(codes), "schedule": bs.layout(),
            "pcg_iterations_per_body_step": {"mean": float(it_all.mean()), "max": int(it_all.max())},
            "pcg_roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak,
                             "formula": ("64 nnzb_b + 208 n_b" if factor else "40 nnzb_b + 172 n_b") +
                                        " per body iteration, summed over bodies x (iterations_b + 1)"}}


def run_gb300(args, rank, world, local_rank):
    import numpy as np
    import torch
    import torch.distributed as dist
    from mfem_gb300 import Model, MixedFEMSolver, beams, _lib

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    mesh = beams.build_beam(args.workload)
    spec = mesh.spec
    model = Model.from_beam(mesh, device=dev)
    solver = MixedFEMSolver(model, iterations=spec.iterations, energy=spec.energy,
                            cg_tolerance=spec.cg_tolerance, cg_max_iterations=spec.cg_max_iterations,
                            pcg_ctas=args.pcg_ctas, pcg_variant=args.pcg_variant,
                            # the workload is the plain local/global step unless asked
                            line_search=args.line_search, preconditioner=args.preconditioner,
                            factor_refresh=args.factor_refresh,
                            solver_precision=args.precision, outer_tolerance=args.outer_tolerance,
                            inner_tolerance=args.inner_tolerance, outer_max_iterations=args.outer_max_iterations)
    s_init = solver.tet_stretch.clone().reshape(-1)
    lam0 = torch.zeros_like(s_init)
    q0 = torch.as_tensor(mesh.q0, device=dev)
    A, B = model.state(), model.state()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    # the global-memory PCG (factor preconditioners) picks its schedule
    tune_ms = solver.autotune(q0, spec.dt) if solver.pcg_layout()["variant"] == "global_memory" else None

    def reset():
        A.particle_q.copy_(q0)
        A.particle_qd.zero_()
        solver.write_buffer("tet_stretch", s_init)
        solver.write_buffer("tet_lambda", lam0)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    # ---- the fp64 check of every solve of the timed trajectory (untimed,
    # graph replays with the check on; the check only reads)
    res32, res_own, q_checked = run_checked(solver, model, q0, s_init, spec.dt, args.steps)

    # ---- warm-up (captures the step graphs)
    reset()
    for _ in range(args.warmup):
        solver.step(A, B, None, None, spec.dt)
        A, B = B, A
    torch.cuda.synchronize(dev)

    # ---- value: resident state, graph replays
    reset()
    sampler = ClockSampler(local_rank)
    barrier()
    sampler.start()
    launches0 = _lib.kernel_launch_count()
    total_ms = 0.0
    pcg_iters = []
    statuses = set()
    codes = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        solver.step(A, B, None, None, spec.dt)
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
        st = solver.solve_stats()
        pcg_iters.append(sum(s["iterations"] for s in st))
        statuses.update(s["status"] for s in st)
        codes += [s["status"] for s in st]
        A, B = B, A
    launches = _lib.kernel_launch_count() - launches0
    barrier()
    clocks = sampler.stop()
    t_max = max_over_ranks(total_ms / 1000.0, world, dev)
    value = job_rate(args.steps, world, t_max)
    q_final = A.particle_q.cpu().numpy()

    # ---- e2e: host-resident state through the public API
    reset()
    hq = torch.empty((mesh.n, 3), dtype=torch.float32, pin_memory=True)
    hqd = torch.empty_like(hq, pin_memory=True)
    hq.copy_(q0.cpu())
    hqd.zero_()
    oq = torch.empty_like(hq, pin_memory=True)
    oqd = torch.empty_like(hq, pin_memory=True)
    e2e_ms = 0.0
    barrier()
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        A.particle_q.copy_(hq, non_blocking=True)
        A.particle_qd.copy_(hqd, non_blocking=True)
        solver.step(A, B, None, None, spec.dt)
        oq.copy_(B.particle_q, non_blocking=True)
        oqd.copy_(B.particle_qd, non_blocking=True)
        e1.record(stream)
        e1.synchronize()
        e2e_ms += e0.elapsed_time(e1)
        hq, oq = oq, hq
        hqd, oqd = oqd, hqd
    barrier()
    e2e_s = max_over_ranks(e2e_ms / 1000.0, world, dev)
    e2e_value = job_rate(args.steps, world, e2e_s)
    e2e_match = bool(np.array_equal(hq.numpy(), q_final))
    state_bytes = 2 * mesh.n * 3 * 4

    # ---- stage profile: eager stages, CUDA events on the launch stream
    reset()
    stage_ms = {"element": 0.0, "assemble": 0.0, "pcg": 0.0, "local_solve": 0.0, "predict": 0.0}
    stage_launches = {k: 0 for k in stage_ms}
    prof_iters = 0
    prof_solves = 0
    prof_steps = max(1, min(args.profile_steps, args.steps))
    x = B.particle_q
    for _ in range(prof_steps):
        flush.zero_()
        evs = []

        def mark(name):
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(stream)
            evs.append((name, ev))

        mark("start")
        solver.predict(A.particle_q, A.particle_qd, spec.dt)
        mark("predict")
        x.copy_(A.particle_q)
        mark("copy")
        for it in range(spec.iterations):
            solver.update_system(x)
            mark("element")
            solver.assemble(x, spec.dt)
            mark("assemble")
            solver.global_solve(it)
            mark("pcg")
            solver.local_solve(x)
            mark("local_solve")
        torch.cuda.synchronize(dev)
        for (_, a), (name, b) in zip(evs[:-1], evs[1:]):
            if name in stage_ms:
                stage_ms[name] += a.elapsed_time(b)
                stage_launches[name] += 1
        st = solver.solve_stats()
        prof_iters += sum(s["iterations"] for s in st)
        prof_solves += len(st)
        B.particle_qd.copy_((x - A.particle_q) / spec.dt)
        A, B = B, A
        x = B.particle_q
    nnzb = solver.nnzb
    b_it = pcg_bytes_per_iteration(nnzb, mesh.n)
    pcg_bytes = b_it * (prof_iters + prof_solves)  # +1 pass per solve: the initial residual
    achieved = pcg_bytes / (stage_ms["pcg"] / 1000.0) / 1e9
    peak, peak_src = hbm_peak()
    per_launch_iters = (prof_iters + prof_solves) / prof_solves
    # DRAM bytes of one captured launch of this workload's PCG (committed ncu summaries)
    summary, note = {
        "nh_beam": ("pcg_kernel_nh_beam.md", "about 378 iterations"),
        "stiff_beam": ("pcg_standard_kernel_stiff_beam.md",
                       "about 950 iterations; H stays in the 129 MB L2 across iterations"),
    }.get(args.workload, (None, None))
    traffic = ncu_traffic_per_launch(summary) if summary else None
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
        "traffic": traffic,
        "traffic_note": f"DRAM bytes of one captured launch ({note}), profiles/{summary}" if summary else None,
        "kernel": "pcg_kernel (persistent cooperative block-Jacobi PCG)",
        "algorithmic_bytes_per_launch": b_it * per_launch_iters,
        "bytes_per_pcg_iteration": b_it, "pcg_iterations_per_launch": per_launch_iters - 1,
        "avg_launch_ms": stage_ms["pcg"] / stage_launches["pcg"], "peak_source": peak_src,
    }
    variant = solver.pcg_layout()["variant"]
    if args.precision == "fp32" and args.preconditioner != "block_jacobi" and variant == "factor":
        # the persistent factor PCG: two BF16 factor passes (20 B block + 4 B
        # column each, over the lower and the upper pattern) replace the
        # block-Jacobi block, plus the y and published Ap vectors
        b_it = 64 * nnzb + 208 * mesh.n
        roofline.update({
            "achieved": b_it * (prof_iters + prof_solves) / (stage_ms["pcg"] / 1000.0) / 1e9,
            "traffic": ncu_traffic_per_launch("pcg_factor_kernel_nh_beam.md") if args.workload == "nh_beam" else None,
            "traffic_note": ("DRAM bytes of one captured FSAI launch (about 160 iterations), "
                             "profiles/pcg_factor_kernel_nh_beam.md" if args.workload == "nh_beam" else None),
            "kernel": f"pcg_factor_kernel (persistent cooperative {args.preconditioner} PCG)",
            "algorithmic_bytes_per_launch": b_it * per_launch_iters, "bytes_per_pcg_iteration": b_it,
            "bytes_per_pcg_iteration_formula": "64 nnzb + 208 n"})
        roofline["frac"] = roofline["achieved"] / peak
    elif args.precision != "fp32" or args.preconditioner != "block_jacobi":
        # the persistent fp32 PCG does not run: the mixed-precision or
        # global-memory factor solves are reported as a whole
        # (stage_ms_per_step["pcg"])
        roofline = None
    total_stage = sum(stage_ms.values())
    shares = {k: v / total_stage for k, v in stage_ms.items()}

    if rank != 0:
        return 0
    variants = None
    if (world == 1 and not args.no_variants and args.precision == "fp32" and args.preconditioner == "block_jacobi"
            and not args.line_search):
        variants = solve_variants(mesh, dev, inner_tolerance=args.variant_inner_tolerance)
    extra = None
    if (world == 1 and not args.no_extra_workloads and args.workload == "nh_beam" and args.precision == "fp32"
            and args.preconditioner == "block_jacobi" and not args.line_search):
        extra = extra_workloads(dev)
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_line(mesh, args.cpu_budget_s, spec.steps, args.workload)
    avg_iters = statistics.mean(pcg_iters)
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(mesh, {"line_search": bool(args.line_search),
                                         "preconditioner": args.preconditioner,
                                         "factor_refresh": args.factor_refresh,
                                         "global_memory_autotune_ms": tune_ms},
                                  precision=args.precision, outer_tolerance=args.outer_tolerance,
                                  preconditioner=args.preconditioner, factor_refresh=args.factor_refresh,
                                  pcg_variant=solver.pcg_layout()["variant"],
                                  inner_tolerance=args.inner_tolerance),
        "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes, "matches_resident_run": e2e_match},
        "gpu_launches": int(launches),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clocks,
        "pcg_iterations_per_step": avg_iters,
        "dof_iterations_per_s": world * 3 * mesh.n * sum(pcg_iters) / t_max,
        "pcg_status_codes": sorted(statuses),
        "converged_fraction": sum(1 for c in codes if c == 0) / max(1, len(codes)),
        "fp64_check": {
            "what": ("float64 ||g - H dx|| / ||g|| of every solve of the timed trajectory (a separate untimed run "
                     "with the check on, bit-identical positions); 'solution' is the solve's own output"),
            "solution": checked_summary(res_own if args.precision != "fp32" else res32, spec.cg_tolerance),
            "fp32_dx": checked_summary(res32, spec.cg_tolerance),
            "checked_run_matches_timed": bool(np.array_equal(q_checked, q_final)),
        },
        "stage_share": shares,
        "stage_ms_per_step": {k: v / prof_steps for k, v in stage_ms.items()},
        "solve_variants": variants,
        "extra_workloads": extra,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world != args.gpus and not (world == 1 and args.gpus == 1):
        if world == 1:
            print(json.dumps({"error": f"--gpus {args.gpus} needs torchrun with {args.gpus} processes"}))
            return 2
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    try:
        if args.workload.startswith("batched"):
            return run_batched(args, rank, world, local_rank)
        return run_gb300(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
