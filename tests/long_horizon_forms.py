"""Error of every lattice form against the float64 oracle over a long coupled run (test
infrastructure; a standalone script, not collected by pytest: the oracle's float64 run takes
minutes).

The scene is the coupled benchmark's geometry at reduced size, ``fsi.scenes.coupled_bodies(
nx=96, ny=48, nz=48, bodies=4, cube_edge=8, sphere_radius=4.0)``, with the opt-in velocity
inlet that reads every population from before its update (the reference's in-place inlet
grows without bound on this channel after a few hundred steps). Each GPU form (FP32 exact,
FP32 fast, FP16 and BF16 deviation storage; atomic scatter) runs the given number of
coupled steps; the float64 oracle runs the same steps on the host. At the listed steps the
script prints the relative L2 error of density, velocity, body drag (sum of the particles'
coupling forces) and particle displacement.

    python tests/long_horizon_forms.py --steps 2000 --at 1000,2000
"""
from __future__ import annotations

import argparse
import dataclasses
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path[:0] = [str(ROOT), str(ROOT / "taichi-mpm-lbm_gb300")]

from fsi import scenes  # noqa: E402
from fsi.simulation import FSISimulation  # noqa: E402
from oracle import oracle as O  # noqa: E402

FORMS = (("f32", "exact"), ("f32", "fast"), ("f16", "fast"), ("bf16", "fast"))


def rel(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def scene():
    cfg, solid, pos, young = scenes.coupled_bodies(nx=96, ny=48, nz=48, bodies=4, cube_edge=8,
                                                   sphere_radius=4.0)
    inlet = dataclasses.replace(cfg.lbm.x_left, velocity_update="simultaneous")
    return dataclasses.replace(cfg, lbm=dataclasses.replace(cfg.lbm, x_left=inlet)), solid, pos, young


def state(lbm_rho, lbm_u, x, drag):
    return {"rho": np.array(lbm_rho), "u": np.array(lbm_u), "x": np.array(x),
            "drag": np.asarray(drag, np.float64)}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--at", default="1000,2000")
    args = ap.parse_args()
    marks = sorted({int(s) for s in args.at.split(",") if 0 < int(s) <= args.steps})
    cfg, solid, pos, young = scene()
    x0 = np.asarray(pos, np.float64)

    gpu = {}
    for storage, arith in FORMS:
        c = dataclasses.replace(cfg, lbm=dataclasses.replace(
            cfg.lbm, population_storage=storage, collision_arithmetic=arith))
        sim = FSISimulation(c)
        sim.initialize_lbm(solid)
        sim.initialize_mpm_from_numpy(pos, youngs_modulus=young, poisson_ratio=0.3)
        for k in range(1, args.steps + 1):
            sim.coupler.step(c.lbm_dt)
            if k in marks:
                gpu[(storage, arith, k)] = state(
                    sim.lbm.density_numpy(), sim.lbm.velocity_numpy(), sim.mpm.positions_numpy(),
                    sim.coupler.total_particle_coupling_force())
        del sim

    ref = O.FSISimulation(cfg, dtype=np.float64, nthreads=os.cpu_count() or 1)
    ref.initialize_lbm(solid)
    ref.initialize_mpm_from_numpy(pos, youngs_modulus=young, poisson_ratio=0.3)
    print("| Form | Step | rho rel-L2 | u rel-L2 | body drag | particle displacement |")
    print("|---|---|---|---|---|---|")
    for k in range(1, args.steps + 1):
        ref.coupler.step(cfg.lbm_dt)
        if k not in marks:
            continue
        r = state(ref.lbm.rho, ref.lbm.v, ref.mpm.positions_numpy(),
                  ref.coupler.total_particle_coupling_force())
        for storage, arith in FORMS:
            g = gpu[(storage, arith, k)]
            print(f"| {storage} {arith} | {k} | {rel(g['rho'], r['rho']):.1e} | "
                  f"{rel(g['u'], r['u']):.1e} | {rel(g['drag'], r['drag']):.1e} | "
                  f"{rel(g['x'] - x0, r['x'] - x0):.1e} |", flush=True)


if __name__ == "__main__":
    main()
