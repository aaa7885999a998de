"""Float32 against float64 on the coupled-bodies channel at reduced size: test infrastructure
(CPU only, the oracle alone).

The scene is ``fsi.scenes.coupled_bodies(nx=96, ny=48, nz=48, bodies=4, cube_edge=8,
sphere_radius=4.0)``: the geometry of the coupled benchmark (velocity inlet 0.05 / pressure
outlet in x, walls in y and z, cubes and balls with per-body Young's modulus, 10 substeps per
lattice step). The float32 run uses the device's polar iteration and the cell-ordered sums,
the configuration whose every field the GPU's FP32 sorted scatter reproduces bit for bit
(tests/test_gpu_config_geometry.py); the float64 run is the reference of the error table.
Both advance in lockstep; at the listed steps the script records the relative L2 error of
the fluid density and velocity, of the body drag (sum of the particles' coupling forces) and
of the particle displacement from the start.

With the reference's inlet the horizon is 200 steps. From about step 250 this channel grows
a disturbance at the inlet face next to a wall corner, cell (0, 42, 42), with or without the
bodies and in both precisions: max |u| 0.060 at step 250, 0.098 at step 450, 0.99 at step
500, NaN by step 550 (the lattice alone, float64). The face conditions are the reference's
literally (fsi/lbm3d.py:363-407): its velocity inlet, updated in place in q order, is what
grows. ``--inlet simultaneous`` uses the opt-in inlet that reads every population from before
the update (BoundaryConfig.velocity_update), which stays bounded; with it the table runs to
the 2,000 steps of the benchmark's configuration.

    python oracle/error_table_bodies.py --steps 200 --out table.json
    python oracle/error_table_bodies.py --inlet simultaneous --steps 2000 \
        --at 100,250,500,1000,1500,2000 --out table.json
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path[:0] = [str(ROOT), str(ROOT / "taichi-mpm-lbm_gb300")]

from fsi import scenes  # noqa: E402
from oracle import oracle as O  # noqa: E402


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--at", default="25,50,100,150,200",
                    help="steps at which the errors are recorded")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=None, help="JSON file for the table")
    ap.add_argument("--inlet", choices=("sequential", "simultaneous"), default="sequential",
                    help="velocity inlet update (BoundaryConfig.velocity_update)")
    args = ap.parse_args()
    marks = sorted({int(s) for s in args.at.split(",") if 0 < int(s) <= args.steps} | {args.steps})

    cfg, solid, pos, young = scenes.coupled_bodies(nx=96, ny=48, nz=48, bodies=4, cube_edge=8,
                                                   sphere_radius=4.0)
    if args.inlet != "sequential":
        inlet = dataclasses.replace(cfg.lbm.x_left, velocity_update=args.inlet)
        cfg = dataclasses.replace(cfg, lbm=dataclasses.replace(cfg.lbm, x_left=inlet))
    f32 = O.FSISimulation(cfg, dtype=np.float32, nthreads=args.threads, polar="device",
                          cell_order=True)
    f64 = O.FSISimulation(cfg, dtype=np.float64, nthreads=args.threads)
    for s in (f32, f64):
        s.initialize_lbm(solid)
        s.initialize_mpm_from_numpy(pos, youngs_modulus=young, poisson_ratio=0.3)
    x0 = np.asarray(pos, np.float64)
    rows = []
    t0 = time.time()
    for k in range(1, args.steps + 1):
        f32.coupler.step(cfg.lbm_dt)
        f64.coupler.step(cfg.lbm_dt)
        if k in marks:
            d32 = np.asarray(f32.coupler.total_particle_coupling_force(), np.float64)
            d64 = np.asarray(f64.coupler.total_particle_coupling_force(), np.float64)
            x64 = np.asarray(f64.mpm.positions_numpy(), np.float64)
            row = {"step": k,
                   "rho": rel_l2(f32.lbm.rho, f64.lbm.rho),
                   "u": rel_l2(f32.lbm.v, f64.lbm.v),
                   "drag": rel_l2(d32, d64),
                   "displacement": rel_l2(f32.mpm.positions_numpy() - x0, x64 - x0),
                   "max_u": float(np.abs(f64.lbm.v).max()),
                   "mean_displacement": float(np.linalg.norm(x64 - x0, axis=1).mean()),
                   "drag_f64": d64.tolist(),
                   "elapsed_s": round(time.time() - t0, 1)}
            rows.append(row)
            print(json.dumps(row), flush=True)
    table = {"workload": "coupled bodies channel 96x48x48, 4 bodies, "
                         f"{len(pos)} particles, 10 substeps per step",
             "float32": "oracle, device polar iteration, cell-ordered sums",
             "float64": "oracle", "inlet": args.inlet, "threads": args.threads, "rows": rows}
    if args.out:
        Path(args.out).write_text(json.dumps(table, indent=1))


if __name__ == "__main__":
    main()
