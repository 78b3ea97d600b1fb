"""Steps one named workload on the GPU and prints its step counters as JSON.

    python -m phys_gb300.run_workload mixed100k [--broadphase grid|sap|tree] [--steps N]
    python -m phys_gb300.run_workload stacks [--tiles X Z] [--sleeping] [--steps N]
    python -m phys_gb300.run_workload spheres1000 [--broadphase sap|grid|tree] [--steps N]
    python -m phys_gb300.run_workload field [--bodies N] [--broadphase ...] [--steps N]

`mixed100k` is the benchmark world (100,000 spheres and boxes in a 200 x 100 x
200 m volume, dt 1/60, 10 solver iterations); `stacks` is the reference's
settled-box profile scene (benchmarks/cpu_profile.cpp:20-41, 512 boxes in
two-high stacks on a floor, dt 1/120, 8 iterations) repeated X x Z times;
`spheres1000` is 1,000 spheres dropped onto a static floor (dt 1/60, 10
iterations, SAP); `field` is the reference's own benchmark scene
(benchmarks/bench_scenes.cpp:11-63: spheres and unit boxes in two layers over a
floor, dt 1/120, 8 iterations, SAP).
The printed `launches` (engine kernels over all steps) and `last_step_launches`
let a profiler skip to the last steps of the run.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import engine, scenes


def mixed100k_cell(scene) -> float:
    """2 x the largest collider extent (sphere radius, box half diagonal)."""
    sph = scene.shape == 0
    ext = np.where(sph, scene.dims[:, 0], np.linalg.norm(scene.dims * 0.5, axis=1))
    return float(2.0 * ext.max())


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("workload", choices=("mixed100k", "stacks", "spheres1000", "field"))
    ap.add_argument("--bodies", type=int, default=10000)
    ap.add_argument("--broadphase", choices=("grid", "sap", "tree"), default=None)
    ap.add_argument("--tiles", type=int, nargs=2, default=(1, 1))
    ap.add_argument("--sleeping", action="store_true")
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    algo = {"sap": engine.SAP, "grid": engine.GRID, "tree": engine.TREE}
    if args.workload == "mixed100k":
        sc = scenes.generate(scenes.MIXED_VOLUME, 100_000, 42)
        bp = args.broadphase or "grid"
        w = engine.GpuWorld(device=args.device, algo=algo[bp], iterations=10,
                            cell_size=mixed100k_cell(sc) if bp == "grid" else 0.0)
        dt = 1.0 / 60.0
    elif args.workload == "field":
        sc = scenes.mixed_field(args.bodies, 42)
        bp = args.broadphase or "sap"
        w = engine.GpuWorld(device=args.device, algo=algo[bp], iterations=8)
        dt = 1.0 / 120.0
    elif args.workload == "spheres1000":
        sc = scenes.generate(scenes.SPHERES_ON_FLOOR, 1000, 42)
        bp = args.broadphase or "sap"
        w = engine.GpuWorld(device=args.device, algo=algo[bp], iterations=10)
        dt = 1.0 / 60.0
    else:
        sc = scenes.box_stacks(*args.tiles)
        bp = args.broadphase or "sap"
        w = engine.GpuWorld(device=args.device, algo=algo[bp], iterations=8)
        dt = 1.0 / 120.0
    w.set_sleeping_enabled(args.sleeping)
    w.load_scene(sc)
    launches = 0
    for _ in range(args.steps):
        w.step(dt)
        launches += int(w.stats()["kernel_launches"])
    st = w.stats()
    out = {"workload": args.workload, "broadphase": bp, "bodies": sc.count, "steps": args.steps,
           "launches": launches, "last_step_launches": int(st["kernel_launches"])}
    for f in ("candidate_pairs", "contact_count", "solved_contact_count", "awake_body_count", "sleeping_body_count",
              "total_ms", "integrate_ms", "broadphase_ms", "narrowphase_ms", "solver_ms", "pose_ms"):
        out[f] = st[f].item()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
