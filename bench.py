"""Benchmark: body-steps/s of the GPU collision-and-contact step on the 100k
mixed-body workload (50% spheres r~U[0.2,0.6], 50% oriented boxes with half
extents U[0.2,0.6], positions uniform in 200x100x200 m without overlap,
velocities N(0,1), dt = 1/60, 10 solver iterations, uniform-grid broadphase
with cell = 2x the largest collider extent).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  `value` is device-timed: CUDA events on the
world's own stream around each step, L2 flushed before every timed step.  `e2e`
is the same metric through the C ABI with host buffers: every step writes the
per-body forces from pinned host memory, steps, and reads all poses back.  The
CPU baseline is the oracle port (the reference algorithm restated) timed on the
host cores for a bounded sample of the same workload.  With N > 1 (torchrun)
each rank steps an independent replica of the world ("replicas only": a single
world does not shard) and `value` aggregates all ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = pathlib.Path(__file__).resolve().parent
for _p in (REPO, REPO / "phys-engine_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "body-steps/s at 100k mixed bodies"
UNIT = "body-steps/s"
BODIES = 100_000
DT = 1.0 / 60.0
ITERATIONS = 10
SEED = 42


def workload_scene():
    from phys_gb300 import scenes

    return scenes.generate(scenes.MIXED_VOLUME, BODIES, SEED)


def cell_size(scene):
    """2 x the largest collider extent (sphere radius, box half diagonal)."""
    sph = scene.shape == 0
    ext = np.where(sph, scene.dims[:, 0], np.linalg.norm(scene.dims * 0.5, axis=1))
    return float(2.0 * ext.max())


def workload_config(scene, order):
    return {
        "workload": "mixed_100k",
        "bodies": scene.count,
        "shapes": "50% spheres r~U[0.2,0.6], 50% boxes half-extents~U[0.2,0.6]^3, uniform random orientation",
        "volume_m": [200, 100, 200],
        "velocity": "N(0,1) m/s",
        "density_g_cm3": 1.0,
        "broadphase": "uniform grid",
        "grid_cell_m": round(cell_size(scene), 6),
        "solver_iterations": ITERATIONS,
        "solver_order": order,
        "dt": DT,
        "steps_of_reference_run": 600,
        "l2": "flushed before every timed step (512 MiB write)",
    }


# ----------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            # nvidia-smi's start-up (driver and NVML initialisation) is kept out
            # of the timed steps that follow
            time.sleep(0.5)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def stage_bytes(stats, bodies, iterations):
    """Algorithmic bytes per step by stage (minimum each stage must move, SoA
    FP32; sort and scratch traffic excluded)."""
    P = int(stats["candidate_pairs"])
    M = int(stats["contact_count"])
    K = int(stats["contact_points"])
    I = iterations
    return {
        "integrate": 92 * bodies,                  # velocity + AABB: read 56, write 36
        "broadphase": 24 * bodies + 8 * P,         # AABB read, pair write
        "narrowphase": 112 * P + 32 * M + 32 * K,  # pair + two bodies' pose/shape/material; manifold writes
        "solver": (32 + 112 + 48 + 96 * I) * M + (32 + 36 + 152 + 36 + 176 * I) * K,
        "pose": 80 * bodies,                       # read 52, write 28
    }


# ------------------------------------------------------------ CPU legs
def profiled_traffic(kernel, algorithmic_bytes):
    """DRAM bytes (read + write) of `kernel` from the committed ncu capture
    (profiles/traffic.json), scaled from the captured launch to one of
    `algorithmic_bytes` by the ratio of algorithmic bytes; or None."""
    p = REPO / "profiles" / "traffic.json"
    if not p.exists():
        return None
    entry = json.loads(p.read_text()).get(kernel)
    if not entry:
        return None
    scale = algorithmic_bytes / entry["algorithmic_bytes_per_launch"]
    return {"bytes": entry["dram_bytes_per_launch"] * scale, "source": entry["source"]}


def cpu_port_rate(scene, budget_s: float, max_steps: int, threads: int, warmup: int = 1):
    """Oracle port (reference algorithm, reference order) on the host cores."""
    from oracle import cpu

    w = cpu.OracleWorld(algo=1, iterations=ITERATIONS, order_mode=0, threads=threads)
    t0 = time.perf_counter()
    w.load_scene(scene)
    load_s = time.perf_counter() - t0
    for _ in range(max(warmup, 1)):
        w.step(DT)
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        w.step(DT)
        steps += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return scene.count * steps / el, steps, el, load_s


def max_over_ranks(value, world_size, device):
    """The slowest rank's figure (every rank calls this; world_size 1 is local)."""
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    if world_size > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world_size, units_per_rank, max_seconds):
    """Whole-job throughput of independent replicas: every rank processes
    `units_per_rank`, the job ends with the slowest rank."""
    return world_size * units_per_rank / max_seconds


def run_reference(args, rank, world_size):
    if rank != 0:
        return
    from oracle import cpu

    cpu.build_oracle()
    scene = workload_scene()
    threads = os.cpu_count() or 1
    budget = 150.0
    warmup = max(args.warmup, 1)
    rate, steps, el, _ = cpu_port_rate(scene, budget, max(args.steps, 1), threads, warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": world_size,
        "steps": steps, "warmup": warmup, "ms_per_step": 1000.0 * el / max(steps, 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": f"synthetic (scene generator, seed {SEED})",
        "config": workload_config(scene, "manifold order (the reference's)"),
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} consecutive steps (after {warmup} warm-up steps) of the full 100k-body world; "
                                   f"the reference's own build is not available on this host, so the oracle "
                                   f"restatement of its algorithm (bit-identical to it) is timed"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- GPU leg
def run_gpu(args, rank, world_size, local_rank):
    import torch

    from phys_gb300 import engine

    torch.cuda.set_device(local_rank)
    scene = workload_scene()
    w = engine.GpuWorld(device=local_rank, algo=engine.GRID, cell_size=cell_size(scene), iterations=ITERATIONS,
                        order=engine.ORDER_COLOR)
    w.load_scene(scene)
    stream = torch.cuda.ExternalStream(w.stream(), device=torch.device("cuda", local_rank))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local_rank}")

    for _ in range(args.warmup):
        w.step(DT)

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    acc = {"integrate_ms": 0.0, "broadphase_ms": 0.0, "narrowphase_ms": 0.0, "solver_ms": 0.0, "pose_ms": 0.0}
    stage_b = {k: 0 for k in ("integrate", "broadphase", "narrowphase", "solver", "pose")}
    launches = 0
    totals = {"pairs": 0, "manifolds": 0, "points": 0}
    phases = np.zeros(8)
    if world_size > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.add_(1.0)
            starts[k].record(stream)
            w.step(DT)
            ends[k].record(stream)
            st = w.stats()
            for key in acc:
                acc[key] += float(st[key])
            for key, v in stage_bytes(st, scene.count, ITERATIONS).items():
                stage_b[key] += v
            launches += int(st["kernel_launches"])
            totals["pairs"] += int(st["candidate_pairs"])
            totals["manifolds"] += int(st["contact_count"])
            totals["points"] += int(st["contact_points"])
            phases += w.solver_phases()
        torch.cuda.synchronize()
    elapsed_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    max_ms = max_over_ranks(elapsed_ms, world_size, f"cuda:{local_rank}")
    value = replica_throughput(world_size, scene.count * args.steps, max_ms / 1000.0)

    # e2e: forces in from pinned host memory, step, poses out, every step
    forces = torch.zeros((scene.count, 3), dtype=torch.float32).pin_memory().numpy()
    poses_p = torch.empty((scene.count, 3), dtype=torch.float32).pin_memory().numpy()
    poses_q = torch.empty((scene.count, 4), dtype=torch.float32).pin_memory().numpy()
    e2e_steps = max(1, min(args.steps, 200))
    e2e_s = 0.0
    for k in range(e2e_steps):
        with torch.cuda.stream(stream):
            flush.add_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w.step_io(DT, forces, poses_p, poses_q)
        e2e_s += time.perf_counter() - t0
    e2e_value = replica_throughput(world_size, scene.count * e2e_steps,
                                   max_over_ranks(e2e_s, world_size, f"cuda:{local_rank}"))

    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    stage_ms = {k[:-3]: v for k, v in acc.items()}
    # The top stage of the step is the contact solver: the prepare kernel over
    # the whole GPU and the solver on one thread-block cluster (two launches per
    # step whenever the manifold count fits the cluster's capacity); the solver
    # stage's stamps time exactly those two kernels.
    block_solver = totals["manifolds"] / args.steps < 3000
    dominant = "solver" if block_solver else max(stage_ms, key=stage_ms.get)
    kernel = "k_prepare_islands + k_solve_cluster" if block_solver else f"{dominant} stage"
    achieved = stage_b[dominant] / (stage_ms[dominant] / 1000.0) / 1e9 if stage_ms[dominant] > 0 else 0.0
    step_bytes = sum(stage_b.values())
    traffic = profiled_traffic(kernel, stage_b[dominant] / args.steps)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": max_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": f"synthetic (scene generator, seed {SEED})",
        "config": workload_config(scene, "graph colour"),
        "roofline": {
            "bound": "hbm", "kernel": kernel, "stage": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
            "traffic": traffic["bytes"] if traffic else None,
            "traffic_source": traffic["source"] if traffic else None,
            "algorithmic_bytes_per_launch": stage_b[dominant] / args.steps,
            "stage_ms_per_step": {k: v / args.steps for k, v in stage_ms.items()},
            # the one-cluster solver's phases (global-timer stamps of its rank 0)
            "solver_phases_us_per_step": dict(zip(
                ("gap_after_narrowphase", "prepare_kernel", "gap_to_cluster", "island_lists", "plan_and_stage",
                 "sweeps", "write_back_and_cache", "gap_to_pose"),
                (float(x) for x in phases * 1000.0 / args.steps))),
            "whole_step": {"algorithmic_bytes_per_step": step_bytes / args.steps,
                           "achieved_gbs": step_bytes / (max_ms / 1000.0) / 1e9 / world_size,
                           "frac": step_bytes / (max_ms / 1000.0) / 1e9 / world_size / peak},
        },
        "workload_per_step": {k: v / args.steps for k, v in totals.items()},
        # forces in: 3 floats per body; poses out: 3 + 4 floats per body
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 12 * scene.count,
                "d2h_bytes_per_step": 28 * scene.count, "steps": e2e_steps},
        "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if world_size == 1 and not args.no_configs:
        line["spheres_1k"] = run_spheres_1k(args, local_rank, flush, peak)
        line["stacking_convex"] = run_stacking_convex(args, local_rank, flush, peak)
    if world_size == 1 and not args.no_batched:
        line["batched"] = run_batched(args, local_rank, flush, peak)
        line["differentiable"] = run_differentiable(args, local_rank)
        line["differentiable_batched"] = run_differentiable_batched(args, local_rank)
    if world_size == 1 and not args.no_sleeping:
        line["sleeping"] = run_sleeping(args, local_rank, flush)
    if world_size == 1 and not args.no_field:
        line["reference_scene"] = run_reference_field(args, local_rank, flush)
    if world_size == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        rate, steps, el, _ = cpu_port_rate(scene, 20.0, 60, threads)
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} steps (after 1 warm-up step) of the same 100k-body world, {el:.1f} s; oracle "
                      f"restatement of the reference algorithm (reference order, grid, {ITERATIONS} iterations)"}
    print(json.dumps(line), flush=True)


# Config 1: 1,000 spheres dropped on a floor, SAP, 10 iterations, 300 steps.
SPHERES_BODIES = 1000
SPHERES_STEPS = 300
# Config 3: 256 box pyramids (16 x 16, 210 boxes each) + 20,000 hulls, 20
# iterations with warm start, 1,000 steps.
STACK_PYRAMIDS = 16
STACK_ITERATIONS = 20
STACK_STEPS = 1000

def run_config_leg(args, local_rank, flush, peak, scene, algo, iterations, steps, dt, cpu_budget_s, describe):
    """One whole run of a configured workload: a fresh world stepped `steps`
    times from its initial state, every step device-timed (CUDA events on the
    world's stream, L2 flushed before each step); the same run end to end
    through pe_world_step_io with host buffers (forces in from pinned memory,
    poses out); and the oracle port (reference algorithm and order, all host
    threads) on a bounded sample of the same run's first steps."""
    import torch

    from oracle import cpu
    from phys_gb300 import engine

    dev = torch.device("cuda", local_rank)
    warm = engine.GpuWorld(device=local_rank, algo=algo, iterations=iterations, order=engine.ORDER_COLOR)
    warm.load_scene(scene)
    for _ in range(min(steps, 10)):
        warm.step(dt)
    warm.close()

    w = engine.GpuWorld(device=local_rank, algo=algo, iterations=iterations, order=engine.ORDER_COLOR)
    w.load_scene(scene)
    stream = torch.cuda.ExternalStream(w.stream(), device=dev)
    bodies = int(scene.count - scene.is_static.sum())
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    stage_ms = {k: 0.0 for k in ("integrate", "broadphase", "narrowphase", "solver", "pose")}
    stage_b = {k: 0 for k in stage_ms}
    totals = {"pairs": 0, "manifolds": 0, "points": 0, "hull_contacts": 0}
    launches = 0
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clocks:
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.add_(1.0)
            starts[k].record(stream)
            w.step(dt)
            ends[k].record(stream)
            st = w.stats()
            for key in stage_ms:
                stage_ms[key] += float(st[key + "_ms"])
            for key, v in stage_bytes(st, scene.count, iterations).items():
                stage_b[key] += v
            launches += int(st["kernel_launches"])
            totals["pairs"] += int(st["candidate_pairs"])
            totals["manifolds"] += int(st["contact_count"])
            totals["points"] += int(st["contact_points"])
            totals["hull_contacts"] += int(st["np_contacts"][3])
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
    last = w.stats()
    w.close()

    # end to end: the same run through the C ABI with host buffers
    w = engine.GpuWorld(device=local_rank, algo=algo, iterations=iterations, order=engine.ORDER_COLOR)
    w.load_scene(scene)
    n = scene.count
    forces = torch.zeros((n, 3), dtype=torch.float32).pin_memory().numpy()
    pp = torch.empty((n, 3), dtype=torch.float32).pin_memory().numpy()
    pq = torch.empty((n, 4), dtype=torch.float32).pin_memory().numpy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        w.step_io(dt, forces, pp, pq)
    e2e_s = time.perf_counter() - t0
    w.close()

    # CPU: the oracle port on the first steps of the same run
    threads = os.cpu_count() or 1
    ow = cpu.OracleWorld(algo=algo, iterations=iterations, order_mode=0, threads=threads)
    ow.load_scene(scene)
    k, t0 = 0, time.perf_counter()
    while k < steps and (k == 0 or time.perf_counter() - t0 < cpu_budget_s):
        ow.step(dt)
        k += 1
    cpu_s = time.perf_counter() - t0

    dominant = max(stage_ms, key=stage_ms.get)
    achieved = stage_b[dominant] / (stage_ms[dominant] / 1000.0) / 1e9 if stage_ms[dominant] > 0 else 0.0
    step_bytes = sum(stage_b.values())
    return {
        "metric": f"body-steps/s, {describe}", "value": bodies * steps / (ms / 1000.0), "unit": UNIT,
        "bodies": bodies, "steps": steps, "ms_per_step": ms / steps, "gpu_launches": launches,
        "workload_per_step": {k2: v / steps for k2, v in totals.items()},
        "last_step": {"candidate_pairs": int(last["candidate_pairs"]), "manifolds": int(last["contact_count"]),
                      "points": int(last["contact_points"]), "colors": int(last["color_count"]),
                      "hull_contacts": int(last["np_contacts"][3])},
        "roofline": {
            "bound": "hbm", "stage": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "algorithmic_bytes_per_step": stage_b[dominant] / steps,
            "stage_ms_per_step": {k2: v / steps for k2, v in stage_ms.items()},
            "whole_step": {"algorithmic_bytes_per_step": step_bytes / steps,
                           "achieved_gbs": step_bytes / (ms / 1000.0) / 1e9,
                           "frac": step_bytes / (ms / 1000.0) / 1e9 / peak}},
        "e2e": {"value": bodies * steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 12 * n,
                "d2h_bytes_per_step": 28 * n, "steps": steps},
        "cpu_baseline": {"value": bodies * k / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                         "ms_per_step": 1000.0 * cpu_s / k,
                         "sample": f"the first {k} of the run's {steps} steps ({cpu_s:.1f} s), oracle restatement "
                                   f"of the reference algorithm in the reference's manifold order"},
        "speedup_vs_cpu_baseline": (bodies * steps / (ms / 1000.0)) / (bodies * k / cpu_s),
        "clocks": clocks.summary(),
    }


def run_spheres_1k(args, local_rank, flush, peak):
    """Config 1: 1,000 spheres (r U[0.25,0.5], density 1) dropped from a
    20 x 40 x 20 m box onto a static floor, zero velocity, dt 1/60, 10
    iterations, friction 0.5, restitution 0, SAP, all 300 steps."""
    from phys_gb300 import engine, scenes

    sc = scenes.generate(scenes.SPHERES_ON_FLOOR, SPHERES_BODIES, SEED)
    out = run_config_leg(args, local_rank, flush, peak, sc, engine.SAP, ITERATIONS, args.spheres_steps, DT, 10.0,
                         "1,000 spheres dropped on a floor")
    out["config"] = {"workload": "spheres_1k", "bodies": SPHERES_BODIES, "radius_m": "U[0.25,0.5]",
                     "spawn_m": [20, 40, 20], "broadphase": "SAP", "solver_iterations": ITERATIONS,
                     "friction": 0.5, "restitution": 0.0, "dt": DT, "steps": args.spheres_steps,
                     "solver_order": "graph colour", "l2": "flushed before every timed step (512 MiB write)"}
    return out


def run_stacking_convex(args, local_rank, flush, peak):
    """Config 3: 256 planar box pyramids (16 x 16, rows 20..1, 210 boxes of
    half extent 0.5 m each, 53,760 boxes) on a tiled static floor, plus 20,000
    convex hulls (24 points on ellipsoids, semi-axes U[0.3,0.8]) dropped from
    30-60 m (the GJK/EPA path), 20 iterations with warm start, dt 1/60."""
    from phys_gb300 import engine, scenes

    sc = scenes.generate(scenes.PYRAMIDS, STACK_PYRAMIDS, SEED)
    out = run_config_leg(args, local_rank, flush, peak, sc, engine.SAP, STACK_ITERATIONS, args.stack_steps, DT, 15.0,
                         "256 box pyramids + 20,000 convex hulls")
    out["config"] = {"workload": "stacking_convex", "pyramids": STACK_PYRAMIDS ** 2, "boxes": 53_760,
                     "hulls": int((sc.shape == 2).sum()), "hull_points": 24, "broadphase": "SAP",
                     "solver_iterations": STACK_ITERATIONS, "warm_start": True, "dt": DT, "steps": args.stack_steps,
                     "solver_order": "graph colour", "l2": "flushed before every timed step (512 MiB write)"}
    return out


BATCH_WORLDS = 4096
BATCH_MIN, BATCH_MAX = 16, 2048


def batch_world_sizes(count=BATCH_WORLDS, seed=SEED):
    """Body counts log-uniform in [16, 2048] (Python's Mersenne Twister, stable
    across platforms)."""
    import random

    r = random.Random(seed)
    ratio = BATCH_MAX / BATCH_MIN
    return [int(round(BATCH_MIN * ratio ** r.random())) for _ in range(count)]


def batch_scenes(sizes):
    from phys_gb300 import scenes

    return [scenes.generate(scenes.MIXED_VOLUME, n, SEED + w) for w, n in enumerate(sizes)]


def run_batched(args, local_rank, flush, peak):
    """4,096 independent worlds (each the mixed workload scaled to its body
    count, seed 42 + w) stepped by the batch engine, against looping the plain
    single-world GPU step over a stratified sample of the same worlds."""
    import torch

    from phys_gb300 import engine

    sizes = batch_world_sizes(args.batch_worlds)
    sc = batch_scenes(sizes)
    batch = engine.GpuBatch(sc, device=local_rank, iterations=ITERATIONS)
    stream = torch.cuda.ExternalStream(batch.stream(), device=torch.device("cuda", local_rank))
    for _ in range(args.warmup):
        batch.step(DT)
    batch.autotune(DT, 3)
    for _ in range(2):
        batch.step(DT)
    steps = max(1, min(args.steps, 60))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    algo_bytes = 0.0
    totals = {"pairs": 0, "manifolds": 0, "points": 0}
    sample_worlds = range(0, len(sizes), 64)
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.add_(1.0)
        starts[k].record(stream)
        batch.step(DT)
        ends[k].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
    # workload of the last step, every world (for the roofline bytes)
    for w in range(len(sizes)):
        st = batch.stats(w)
        algo_bytes += sum(stage_bytes(st, sizes[w], ITERATIONS).values())
        totals["pairs"] += int(st["candidate_pairs"])
        totals["manifolds"] += int(st["contact_count"])
        totals["points"] += int(st["contact_points"])
    world_steps = len(sizes) * steps / (ms / 1000.0)
    step_ms = ms / steps

    # e2e through the C ABI with host buffers: forces in, step, poses out
    n = batch.n
    forces = torch.zeros((n, 3), dtype=torch.float32).pin_memory().numpy()
    pp = torch.empty((n, 3), dtype=torch.float32).pin_memory().numpy()
    pq = torch.empty((n, 4), dtype=torch.float32).pin_memory().numpy()
    e2e_steps = max(1, min(steps, 30))
    e2e_s = 0.0
    for _ in range(e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batch.write_forces(forces)
        batch.step(DT)
        batch.read_poses(pp, pq)
        e2e_s += time.perf_counter() - t0
    buckets = batch.buckets()
    batch.close()

    # plain loop: the single-world engine stepping each sampled world in turn
    sample = list(range(0, len(sizes), 16))
    worlds = []
    for w in sample:
        gw = engine.GpuWorld(device=local_rank, algo=engine.SAP, iterations=ITERATIONS, order=engine.ORDER_COLOR)
        gw.load_scene(sc[w])
        worlds.append(gw)
    for _ in range(3):
        for gw in worlds:
            gw.step(DT)
    plain_steps = 5
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(plain_steps):
        for gw in worlds:
            gw.step(DT)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    plain_world_steps = len(worlds) * plain_steps / plain_s
    for gw in worlds:
        gw.close()
    achieved = algo_bytes / (step_ms / 1000.0) / 1e9
    return {
        "metric": f"world-steps/s, {len(sizes)} batched worlds (forward)",
        "value": world_steps, "unit": "world-steps/s", "steps": steps, "ms_per_step": step_ms,
        "body_steps_per_s": sum(sizes) * steps / (ms / 1000.0),
        "config": {"workload": f"batched_{len(sizes)}", "worlds": len(sizes), "bodies": int(sum(sizes)),
                   "bodies_per_world": f"log-uniform in [{BATCH_MIN}, {BATCH_MAX}] (seed {SEED}), "
                                       f"min {min(sizes)}, max {max(sizes)}",
                   "world": "mixed workload scaled to the world's body count, seed 42 + world",
                   "broadphase": "SAP", "solver_iterations": ITERATIONS, "solver_order": "graph colour",
                   "dt": DT, "steps_of_reference_run": 600,
                   "l2": "flushed before every timed step (512 MiB write)"},
        "workload_per_step": totals,
        "roofline": {"bound": "hbm", "kernel": "k_batch_step (one launch per size bucket)", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (profiled_traffic("k_batch_step", algo_bytes) or {}).get("bytes"),
                     "traffic_source": (profiled_traffic("k_batch_step", algo_bytes) or {}).get("source"),
                     "algorithmic_bytes_per_step": algo_bytes},
        "e2e": {"value": len(sizes) * e2e_steps / e2e_s, "unit": "world-steps/s",
                "h2d_bytes_per_step": 12 * n, "d2h_bytes_per_step": 28 * n, "steps": e2e_steps},
        "gpu_launches": int(steps * len(buckets)),
        "autotune": [{"bodies": [int(b["min_bodies"]), int(min(b["max_bodies"], BATCH_MAX))],
                      "worlds": int(b["world_count"]), "threads": int(b["threads"]),
                      "min_blocks_per_sm": int(b["min_blocks_per_sm"]), "blocks": int(b["blocks"]),
                      "ms": float(b["tuned_ms"]), "candidates_ms": [float(x) for x in b["candidate_ms"][:5]]}
                     for b in buckets],
        "plain_loop": {"value": plain_world_steps, "unit": "world-steps/s",
                       "sample": f"every 16th world ({len(worlds)} worlds), {plain_steps} steps each, wall clock "
                                 f"of the single-world engine's step (CUDA graph per world, synchronous step)"},
        "speedup_vs_plain_loop": world_steps / plain_world_steps,
    }


DIFF_WORLDS = 1024
DIFF_BODIES = 64
DIFF_STEPS = 120
DIFF_DT = 1.0 / 120.0
DIFF_CHECKPOINT = 10


def run_differentiable(args, local_rank):
    """1,024 worlds x 64 boxes (half extents U[0.2,0.5], friction U[0.2,0.8],
    restitution U[0,0.3]) at rest on a plane, 120 steps at dt = 1/120; loss =
    squared distance of each world's final centre of mass from a seeded target
    within 5 m; gradients with respect to initial velocities, masses, frictions
    and restitutions through the GPU adjoint (checkpoint every 10 steps)."""
    import random

    import torch

    from phys_gb300 import engine, rollout, scenes

    W = args.diff_worlds
    sc = [scenes.generate(scenes.BOXES_ON_PLANE, DIFF_BODIES, SEED + w) for w in range(W)]
    roll = rollout.GpuRollout(sc, DIFF_STEPS, DIFF_DT, iterations=ITERATIONS, checkpoint_every=DIFF_CHECKPOINT,
                              device=local_rank)
    fn = rollout.rollout_function()
    dev = torch.device("cuda", local_rank)
    r = random.Random(SEED)
    targets = []
    for _ in range(W):
        while True:
            t = [r.uniform(-5, 5) for _ in range(3)]
            if sum(c * c for c in t) <= 25.0:
                break
        targets.append(t)
    target = torch.tensor(targets, device=dev)
    x0n, q0n, v0n, w0n = roll.initial_state()
    dyn = torch.tensor(~roll.is_static.astype(bool), device=dev)
    world_of = torch.tensor(np.repeat(np.arange(W), roll.counts), device=dev)

    def one(host):
        """Host tensors in (pinned), loss + gradients out to the host."""
        ins = [t.to(dev, non_blocking=True) for t in host]
        for t in ins[2:]:
            t.requires_grad_(True)
        x0, q0, v0, w0, m, f, rs = ins
        xT, qT, vT, wT = fn.apply(roll, x0, q0, v0, w0, m, f, rs)
        mw = m * dyn
        msum = torch.zeros(W, device=dev).index_add_(0, world_of, mw)
        com = torch.zeros(W, 3, device=dev).index_add_(0, world_of, mw[:, None] * xT) / msum[:, None]
        loss = ((com - target) ** 2).sum()
        loss.backward()
        grads = [v0.grad, m.grad, f.grad, rs.grad]
        return float(loss.item()), [g.to("cpu", non_blocking=True) for g in grads]

    pin = lambda a: torch.tensor(a).pin_memory()
    host = [pin(x0n), pin(q0n), pin(v0n), pin(w0n), pin(roll.mass), pin(roll.friction), pin(roll.restitution)]
    for _ in range(2):
        one(host)
    reps = 3
    fwd_ms = bwd_ms = 0.0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        loss, grads = one(host)
        f_ms, b_ms = roll.timings()
        fwd_ms += f_ms
        bwd_ms += b_ms
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    device_s = (fwd_ms + bwd_ms) / 1000.0
    ws = W * DIFF_STEPS * reps
    h2d = sum(int(t.numel() * t.element_size()) for t in host)
    d2h = 4 * roll.n * 6 + 4
    # plain loop: forward steps of the single-world engine over a sample of the same worlds
    worlds = []
    for w in range(0, W, 32):
        gw = engine.GpuWorld(device=local_rank, algo=engine.SAP, iterations=ITERATIONS, order=engine.ORDER_COLOR)
        gw.load_scene(sc[w])
        worlds.append(gw)
    for _ in range(3):
        for gw in worlds:
            gw.step(DIFF_DT)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    plain_steps = 10
    for _ in range(plain_steps):
        for gw in worlds:
            gw.step(DIFF_DT)
    torch.cuda.synchronize()
    plain = len(worlds) * plain_steps / (time.perf_counter() - t1)
    for gw in worlds:
        gw.close()
    value = ws / device_s
    return {
        "metric": f"world-steps/s, {W} worlds forward + adjoint", "value": value, "unit": "world-steps/s",
        "rollouts": reps, "forward_ms_per_rollout": fwd_ms / reps, "adjoint_ms_per_rollout": bwd_ms / reps,
        "config": {"workload": f"differentiable_{W}x{DIFF_BODIES}", "worlds": W, "bodies_per_world": DIFF_BODIES,
                   "shapes": "boxes half-extents U[0.2,0.5] on a static 40x1x40 m plane, at rest",
                   "friction": "U[0.2,0.8]", "restitution": "U[0,0.3]", "steps": DIFF_STEPS, "dt": DIFF_DT,
                   "solver_iterations": ITERATIONS, "checkpoint_every": DIFF_CHECKPOINT,
                   "loss": "sum over worlds of |final centre of mass - target|^2, targets seeded within 5 m",
                   "gradients": "initial velocities, masses, frictions, restitutions (torch.autograd)"},
        "loss": loss,
        "e2e": {"value": ws / e2e_s, "unit": "world-steps/s", "h2d_bytes_per_step": h2d / DIFF_STEPS,
                "d2h_bytes_per_step": d2h / DIFF_STEPS,
                "note": "each rollout copies the initial state and parameters in from pinned host memory and "
                        "the loss and the four gradient arrays out; bytes per step = per rollout / 120"},
        "gpu_launches": 2 * reps,
        "plain_loop": {"value": plain, "unit": "world-steps/s",
                       "sample": f"every 32nd world ({len(worlds)} worlds), {plain_steps} forward steps each, "
                                 f"wall clock of the single-world engine's step"},
        "speedup_vs_plain_loop": value / plain,
    }


DIFF_BATCH_STEPS = 60
DIFF_BATCH_DT = 1.0 / 60.0
DIFF_BATCH_CHECKPOINT = 10
# The mixed-volume worlds are sparse (about one manifold per hundred bodies):
# a quarter manifold of capacity per body (plus 32 per world) covers them.
DIFF_BATCH_MANIFOLDS_PER_BODY = 0.25


def run_differentiable_batched(args, local_rank):
    """Forward + adjoint over the 4,096 uneven batched worlds (body counts
    log-uniform in [16, 2048], each the mixed workload scaled to its size, seed
    42 + w): a 60-step rollout at dt 1/60 with checkpoints every 10 steps, loss =
    sum over worlds of the squared distance of the final centre of mass from a
    seeded target within 5 m, gradients with respect to initial velocities,
    masses, frictions and restitutions through the autograd harness; against
    looping the plain single-world GPU step over a sample of the same worlds."""
    import random

    import torch

    from phys_gb300 import engine, rollout

    sizes = batch_world_sizes(args.batch_worlds)
    sc = batch_scenes(sizes)
    W = len(sizes)
    dev = torch.device("cuda", local_rank)
    free0, _ = torch.cuda.mem_get_info(dev)
    roll = rollout.GpuRollout(sc, DIFF_BATCH_STEPS, DIFF_BATCH_DT, iterations=ITERATIONS,
                              checkpoint_every=DIFF_BATCH_CHECKPOINT, device=local_rank,
                              manifolds_per_body=DIFF_BATCH_MANIFOLDS_PER_BODY)
    fn = rollout.rollout_function()
    r = random.Random(SEED)
    targets = []
    for _ in range(W):
        while True:
            t = [r.uniform(-5, 5) for _ in range(3)]
            if sum(c * c for c in t) <= 25.0:
                break
        targets.append(t)
    target = torch.tensor(targets, device=dev)
    x0n, q0n, v0n, w0n = roll.initial_state()
    dyn = torch.tensor(~roll.is_static.astype(bool), device=dev)
    world_of = torch.tensor(np.repeat(np.arange(W), roll.counts), device=dev)

    def one(host):
        ins = [t.to(dev, non_blocking=True) for t in host]
        for t in ins[2:]:
            t.requires_grad_(True)
        x0, q0, v0, w0, m, f, rs = ins
        xT, qT, vT, wT = fn.apply(roll, x0, q0, v0, w0, m, f, rs)
        mw = m * dyn
        msum = torch.zeros(W, device=dev).index_add_(0, world_of, mw)
        com = torch.zeros(W, 3, device=dev).index_add_(0, world_of, mw[:, None] * xT) / msum[:, None]
        loss = ((com - target) ** 2).sum()
        loss.backward()
        grads = [v0.grad, m.grad, f.grad, rs.grad]
        return float(loss.item()), [g.to("cpu", non_blocking=True) for g in grads]

    pin = lambda a: torch.tensor(a).pin_memory()
    host = [pin(x0n), pin(q0n), pin(v0n), pin(w0n), pin(roll.mass), pin(roll.friction), pin(roll.restitution)]
    one(host)  # warm-up (lays out the device slots)
    free1, _ = torch.cuda.mem_get_info(dev)
    reps = 2
    fwd_ms = bwd_ms = 0.0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        loss, grads = one(host)
        f_ms, b_ms = roll.timings()
        fwd_ms += f_ms
        bwd_ms += b_ms
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    finite = all(bool(torch.isfinite(g).all()) for g in grads)
    device_bytes = roll.device_bytes()
    roll.close()
    # plain loop: forward steps of the single-world engine over a sample
    worlds = []
    for w in range(0, W, 64):
        gw = engine.GpuWorld(device=local_rank, algo=engine.SAP, iterations=ITERATIONS, order=engine.ORDER_COLOR)
        gw.load_scene(sc[w])
        worlds.append(gw)
    for _ in range(3):
        for gw in worlds:
            gw.step(DIFF_BATCH_DT)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    plain_steps = 5
    for _ in range(plain_steps):
        for gw in worlds:
            gw.step(DIFF_BATCH_DT)
    torch.cuda.synchronize()
    plain = len(worlds) * plain_steps / (time.perf_counter() - t1)
    for gw in worlds:
        gw.close()
    ws = W * DIFF_BATCH_STEPS * reps
    value = ws / ((fwd_ms + bwd_ms) / 1000.0)
    h2d = sum(int(t.numel() * t.element_size()) for t in host)
    return {
        "metric": f"world-steps/s, {W} uneven batched worlds forward + adjoint", "value": value,
        "unit": "world-steps/s", "rollouts": reps, "forward_ms_per_rollout": fwd_ms / reps,
        "adjoint_ms_per_rollout": bwd_ms / reps,
        "config": {"workload": f"differentiable_batched_{W}", "worlds": W, "bodies": int(sum(sizes)),
                   "bodies_per_world": f"log-uniform in [{BATCH_MIN}, {BATCH_MAX}] (seed {SEED})",
                   "world": "mixed workload scaled to the world's body count, seed 42 + world",
                   "steps": DIFF_BATCH_STEPS, "dt": DIFF_BATCH_DT, "solver_iterations": ITERATIONS,
                   "checkpoint_every": DIFF_BATCH_CHECKPOINT,
                   "manifold_capacity_per_body": DIFF_BATCH_MANIFOLDS_PER_BODY,
                   "loss": "sum over worlds of |final centre of mass - target|^2, targets seeded within 5 m",
                   "gradients": "initial velocities, masses, frictions, restitutions (torch.autograd)"},
        "loss": loss, "gradients_finite": finite,
        "device_memory": {"rollout_bytes": device_bytes,
                          "device_bytes_used_after_first_rollout": int(free0 - free1)},
        "e2e": {"value": ws / e2e_s, "unit": "world-steps/s", "h2d_bytes_per_step": h2d / DIFF_BATCH_STEPS,
                "d2h_bytes_per_step": (4 * roll.n * 6 + 4) / DIFF_BATCH_STEPS},
        "gpu_launches": 2 * reps,
        "plain_loop": {"value": plain, "unit": "world-steps/s",
                       "sample": f"every 64th world ({len(worlds)} worlds), {plain_steps} forward steps each, wall "
                                 f"clock of the single-world engine's step"},
        "speedup_vs_plain_loop": value / plain,
    }


SLEEP_DT = 1.0 / 120.0
SLEEP_WARMUP = 240
SLEEP_ITERATIONS = 8
# The reference's settled-box figures, sleeping enabled / disabled, Apple M2
# (benchmarks/results/sleeping-release.txt:36-38 of bkuangs/phys-engine).
SLEEP_REF_MS = {"enabled": 0.2372, "disabled": 1.8131}


def timed_steps(w, steps, dt, stream, flush):
    """Device time (ms) of `steps` steps, CUDA events on the world's stream, L2
    flushed before each."""
    import torch

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    launches = 0
    torch.cuda.synchronize()
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.add_(1.0)
        starts[k].record(stream)
        w.step(dt)
        ends[k].record(stream)
        launches += int(w.stats()["kernel_launches"])
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in zip(starts, ends)), launches


def run_sleeping(args, local_rank, flush):
    """Sleeping islands: the reference's settled-box profile scene (512 unit
    boxes in two-high stacks on a static floor, dt = 1/120, 8 iterations, 240
    warm-up steps) and 128 copies of it side by side (65,536 boxes), stepped
    with sleeping enabled and disabled; body-steps/s counts the dynamic bodies."""
    import torch

    from oracle import cpu
    from phys_gb300 import engine, scenes

    out = {}
    for name, tiles in (("stacks_512", (1, 1)), ("stacks_65536", (16, 8))):
        sc = scenes.box_stacks(*tiles)
        bodies = int(sc.count - sc.is_static.sum())
        res = {}
        for enabled in (True, False):
            w = engine.GpuWorld(device=local_rank, algo=engine.SAP, iterations=SLEEP_ITERATIONS,
                                order=engine.ORDER_COLOR)
            w.set_sleeping_enabled(enabled)
            w.load_scene(sc)
            for _ in range(SLEEP_WARMUP):
                w.step(SLEEP_DT)
            stream = torch.cuda.ExternalStream(w.stream(), device=torch.device("cuda", local_rank))
            ms, launches = timed_steps(w, args.sleep_steps, SLEEP_DT, stream, flush)
            st = w.stats()
            res["enabled" if enabled else "disabled"] = {
                "ms_per_step": ms / args.sleep_steps, "value": bodies * args.sleep_steps / (ms / 1000.0),
                "sleeping_bodies": int(st["sleeping_body_count"]), "awake_bodies": int(st["awake_body_count"]),
                "contacts": int(st["contact_count"]), "solved_contacts": int(st["solved_contact_count"]),
                "gpu_launches": launches}
            w.close()
        e, d = res["enabled"], res["disabled"]
        out[name] = {"metric": "body-steps/s, settled box stacks, sleeping enabled", "value": e["value"],
                     "unit": UNIT, "bodies": bodies, "steps": args.sleep_steps, "warmup": SLEEP_WARMUP,
                     "enabled": e, "disabled": d, "speedup_vs_disabled": d["ms_per_step"] / e["ms_per_step"]}
    # CPU: the oracle port on the 512-box scene, both ways
    sc = scenes.box_stacks()
    port = {}
    for enabled in (True, False):
        ow = cpu.OracleWorld(algo=0, iterations=SLEEP_ITERATIONS, order_mode=0)
        ow.set_sleeping_enabled(enabled)
        ow.load_scene(sc)
        for _ in range(SLEEP_WARMUP):
            ow.step(SLEEP_DT)
        t0 = time.perf_counter()
        for _ in range(args.sleep_steps):
            ow.step(SLEEP_DT)
        port["enabled" if enabled else "disabled"] = (time.perf_counter() - t0) * 1000.0 / args.sleep_steps
    out["cpu_baseline"] = {"kind": "port", "cores": 1, "workload": "stacks_512",
                           "sample": f"{args.sleep_steps} steps after {SLEEP_WARMUP} warm-up steps, oracle "
                                     "restatement (reference order, SAP, 8 iterations), one host thread",
                           "ms_per_step_enabled": port["enabled"], "ms_per_step_disabled": port["disabled"]}
    out["reference_published"] = {"ms_per_step_enabled": SLEEP_REF_MS["enabled"],
                                  "ms_per_step_disabled": SLEEP_REF_MS["disabled"], "hardware": "Apple M2",
                                  "broadphase": "dynamic AABB tree",
                                  "source": "benchmarks/results/sleeping-release.txt"}
    return out


# The reference's published mean step times on its own benchmark scene
# (phys_collision_bench, mixed field, SAP, 120 Hz, 240 warm-up + 1,200 measured
# steps, Apple M2): one worker per stage, and 4 + 4 + 4 workers at 10k
# (benchmarks/results/mixed-sustained-sap-release.txt:161,285,347,
# benchmarks/results/parallel-sap-sweep-release.txt:47-53).
REF_FIELD_MS = {1000: 2.33, 5000: 13.10, 10000: 27.32}
REF_FIELD_MS_4WORKERS = {5000: 4.17, 10000: 8.90}


def run_reference_field(args, local_rank, flush):
    """The reference's own benchmark scene (scenes.mixed_field: half spheres,
    half unit boxes in two layers over a floor) at 1k, 5k and 10k bodies, SAP,
    8 iterations, dt 1/120, 240 warm-up steps, then the timed steps; next to the
    reference's published M2 times and the oracle port on the host cores."""
    import torch

    from oracle import cpu
    from phys_gb300 import engine, scenes

    out = {}
    threads = os.cpu_count() or 1
    for n in (1000, 5000, 10000):
        sc = scenes.mixed_field(n, SEED)
        w = engine.GpuWorld(device=local_rank, algo=engine.SAP, iterations=SLEEP_ITERATIONS, order=engine.ORDER_COLOR)
        w.load_scene(sc)
        for _ in range(240):
            w.step(SLEEP_DT)
        stream = torch.cuda.ExternalStream(w.stream(), device=torch.device("cuda", local_rank))
        ms, launches = timed_steps(w, args.field_steps, SLEEP_DT, stream, flush)
        st = w.stats()
        w.close()
        entry = {"bodies": n, "steps": args.field_steps, "ms_per_step": ms / args.field_steps,
                 "value": n * args.field_steps / (ms / 1000.0), "unit": UNIT, "gpu_launches": launches,
                 "contacts": int(st["contact_count"]), "candidate_pairs": int(st["candidate_pairs"]),
                 "reference_m2_ms_per_step": REF_FIELD_MS[n]}
        if n in REF_FIELD_MS_4WORKERS:
            entry["reference_m2_4x3_workers_ms_per_step"] = REF_FIELD_MS_4WORKERS[n]
        if n == 10000 and not args.no_cpu_baseline:
            ow = cpu.OracleWorld(algo=0, iterations=SLEEP_ITERATIONS, order_mode=0, threads=threads)
            ow.load_scene(sc)
            for _ in range(240):
                ow.step(SLEEP_DT)
            t0, k = time.perf_counter(), 0
            while k < 120 and time.perf_counter() - t0 < 10.0:
                ow.step(SLEEP_DT)
                k += 1
            entry["cpu_port_ms_per_step"] = (time.perf_counter() - t0) * 1000.0 / k
            entry["cpu_port_cores"] = threads
        out[f"mixed_field_{n}"] = entry
    return out


PROFILE_WORKLOADS = ("mixed100k", "stacks", "spheres1000", "field", "stacking_convex")


def run_workload(args):
    """Steps one named workload on the GPU (no timing) and prints its step
    counters as JSON; the profiles under profiles/ are taken on these runs.
    `mixed100k` is the benchmark world; `stacks` the reference's settled-box
    profile scene (benchmarks/cpu_profile.cpp:20-41) repeated --tiles X Z times;
    `spheres1000` 1,000 spheres dropped on a floor (SAP, 10 iterations, dt 1/60);
    `field` the reference's own benchmark scene (benchmarks/bench_scenes.cpp:11-63,
    SAP, 8 iterations, dt 1/120) with --bodies bodies; `stacking_convex` the 256
    box pyramids plus 20,000 hulls (20 iterations, dt 1/60), or --pyramids per side,
    with the hulls lowered by --drop metres.
    `launches` (engine kernels over all steps) and `last_step_launches` let a
    profiler skip to the last steps of the run."""
    from phys_gb300 import engine, scenes

    algo = {"sap": engine.SAP, "grid": engine.GRID, "tree": engine.TREE}
    name = args.workload
    if name == "mixed100k":
        sc = workload_scene()
        bp = args.broadphase or "grid"
        w = engine.GpuWorld(device=0, algo=algo[bp], iterations=ITERATIONS,
                            cell_size=cell_size(sc) if bp == "grid" else 0.0)
        dt = DT
    elif name == "field":
        sc = scenes.mixed_field(args.bodies, SEED)
        bp = args.broadphase or "sap"
        w = engine.GpuWorld(device=0, algo=algo[bp], iterations=SLEEP_ITERATIONS)
        dt = SLEEP_DT
    elif name == "spheres1000":
        sc = scenes.generate(scenes.SPHERES_ON_FLOOR, SPHERES_BODIES, SEED)
        bp = args.broadphase or "sap"
        w = engine.GpuWorld(device=0, algo=algo[bp], iterations=ITERATIONS)
        dt = DT
    elif name == "stacking_convex":
        sc = scenes.generate(scenes.PYRAMIDS, args.pyramids, SEED)
        sc.pos[sc.shape == 2, 1] -= np.float32(args.drop)
        bp = args.broadphase or "sap"
        w = engine.GpuWorld(device=0, algo=algo[bp], iterations=STACK_ITERATIONS)
        dt = DT
    else:
        sc = scenes.box_stacks(*args.tiles)
        bp = args.broadphase or "sap"
        w = engine.GpuWorld(device=0, algo=algo[bp], iterations=SLEEP_ITERATIONS)
        dt = SLEEP_DT
    w.set_sleeping_enabled(args.sleeping)
    w.load_scene(sc)
    launches = 0
    for _ in range(args.profile_steps):
        w.step(dt)
        launches += int(w.stats()["kernel_launches"])
    st = w.stats()
    out = {"workload": name, "broadphase": bp, "bodies": sc.count, "steps": args.profile_steps,
           "launches": launches, "last_step_launches": int(st["kernel_launches"])}
    for f in ("candidate_pairs", "contact_count", "contact_points", "solved_contact_count", "awake_body_count",
              "sleeping_body_count", "total_ms", "integrate_ms", "broadphase_ms", "narrowphase_ms", "solver_ms",
              "pose_ms"):
        out[f] = st[f].item()
    w.close()
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the batched-world and differentiable-rollout measurements")
    ap.add_argument("--batch-worlds", type=int, default=BATCH_WORLDS, help="worlds of the batched measurement")
    ap.add_argument("--diff-worlds", type=int, default=DIFF_WORLDS, help="worlds of the differentiable rollout")
    ap.add_argument("--sleep-steps", type=int, default=200, help="timed steps of the sleeping measurement")
    ap.add_argument("--no-sleeping", action="store_true", help="skip the sleeping-island measurement")
    ap.add_argument("--field-steps", type=int, default=1200, help="timed steps of the reference-scene measurement")
    ap.add_argument("--no-field", action="store_true", help="skip the reference's own benchmark scene")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the 1,000-sphere and the pyramids-with-hulls whole-run measurements")
    ap.add_argument("--spheres-steps", type=int, default=SPHERES_STEPS, help="steps of the 1,000-sphere run")
    ap.add_argument("--stack-steps", type=int, default=STACK_STEPS, help="steps of the pyramids-with-hulls run")
    ap.add_argument("--workload", choices=PROFILE_WORKLOADS, default=None,
                    help="step one named workload untimed and print its counters (profiling runs)")
    ap.add_argument("--profile-steps", type=int, default=8, help="steps of the --workload run")
    ap.add_argument("--bodies", type=int, default=10000, help="bodies of the --workload field scene")
    ap.add_argument("--pyramids", type=int, default=16, help="pyramids per side of --workload stacking_convex")
    ap.add_argument("--drop", type=float, default=0.0,
                    help="--workload stacking_convex: lower the hulls by this many metres (contacts from the first steps)")
    ap.add_argument("--broadphase", choices=("grid", "sap", "tree"), default=None, help="--workload broadphase")
    ap.add_argument("--tiles", type=int, nargs=2, default=(1, 1), help="--workload stacks: copies along x and z")
    ap.add_argument("--sleeping", action="store_true", help="--workload: sleeping islands enabled")
    args = ap.parse_args()
    if args.workload:
        run_workload(args)
        return
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")

    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world_size)
        return
    if world_size > 1:
        import torch

        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    try:
        run_gpu(args, rank, world_size, local_rank)
    finally:
        if world_size > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
