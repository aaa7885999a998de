"""Benchmark of the GB300 coupled LBM-MPM timestep (LBMMpmCoupler.step / FSISimulation.step).

Headline workload (seeded, synthetic; the coupled configuration at scale):
  384x192x192 D3Q19 MRT channel, tau 0.55, velocity inlet 0.05 at x = 0, pressure outlet at
  x = nx-1, walls in y and z (mask planes); 48 elastic bodies (24 cubes of edge 12, 24 balls of
  radius 6) at 8 particles per cell, 502,304 particles, Young's modulus U[0.02, 0.1] per body
  (seed 3); 10 MPM substeps per lattice step, penalty coupling gamma 0.1.
A timed "step" is one coupled lattice step (10 coupling + MPM substeps, force assembly, lattice
step): value = coupled MLUPS (all lattice cells per second), with particle-steps/s beside it.
The standalone kernels at scale (256^3 lattice, 2,097,152-particle MPM), the coupled smoke
workload, the precision forms, the batched scenes and the learned closure are timed as extras.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 (under torchrun) runs independent replicas, one per GPU ("replicas only": the path has
no exchange step); value is the sum over ranks, time the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "taichi-mpm-lbm_gb300"))

LBM_BYTES_PER_CELL = 181     # algorithmic bytes per FP32 fluid cell update (pops 152, mask 1, force 12, rho+u 16)
SOLID_CELL_BYTES = 4         # a solid cell costs the step its flag word only
KERNEL_BYTES_PER_CELL = 168  # what the fused step moves: pops 152, flag word 4, force 12
MPM_BYTES_PER_PARTICLE = 200  # algorithmic bytes per particle-substep (standalone)
COUPLED_BYTES_PER_PARTICLE = 224  # per particle-substep with the coupling force written and read
MPM_BYTES_PER_NODE = 32       # per touched grid node per substep
# Kernel launches per call of each entry point the timed regions use.
LAUNCHES = {"fsi_coupling_forces": 1, "fsi_mpm_substep": 3, "fsi_mpm_substep_sorted": 10,
            "fsi_coupled_substep": 10, "fsi_coupled_substep_tiled": 4,
            "fsi_coupling_assemble": 1, "fsi_contact": 1,
            "fsi_lbm_update_macro": 1, "fsi_lbm_macro_diagnostics": 1, "fsi_lbm_reduce": 1,
            "fsi_coupled_diagnostics": 1, "fsi_lbm_force_op": 1, "fsi_mpm_reduce": 1,
            "fsi_coupling_reduce": 1}
# DRAM bytes per fluid cell and step kernel launch, from the ncu captures of the 192^3 scene
# (dram__bytes_read.sum + dram__bytes_write.sum, odd/even launch average).
TRAFFIC_PER_FLUID_CELL = {"f32/exact": 177.4, "f16/fast": 96.1}
# DRAM bytes of one coupled step of the headline scene (dram__bytes_read.sum +
# dram__bytes_write.sum summed over the step's launches, ncu capture of the third coupled step).
TRAFFIC_PER_COUPLED_STEP = 5_661_000_000
METRIC = "MLUPS & particle-steps/s on 1 GB300: plain vs FP16/learned, <=1% drag error"


def lattice_bytes(fluid_cells: int, solid_cells: int, per_fluid: int = LBM_BYTES_PER_CELL) -> int:
    """Algorithmic bytes of one lattice step: the per-cell figure for each fluid cell and the
    flag word for each solid cell (whose populations the step does not touch)."""
    return per_fluid * fluid_cells + SOLID_CELL_BYTES * solid_cells


def touched_nodes(base: np.ndarray, dims) -> int:
    """Grid nodes in the union of the particles' 27-node stencils (inside the grid)."""
    nx, ny, nz = dims
    b = base.astype(np.int64)
    cells = np.unique(b[np.all((b >= -2) & (b < np.array(dims)), axis=1)], axis=0)
    out = []
    for di in range(3):
        for dj in range(3):
            for dk in range(3):
                n = cells + np.array([di, dj, dk])
                n = n[np.all((n >= 0) & (n < np.array(dims)), axis=1)]
                out.append((n[:, 0] * ny + n[:, 1]) * nz + n[:, 2])
    return int(np.unique(np.concatenate(out)).size) if out else 0


def launches_since(before, lbm_step_launches: int = 1, tiled_substep_launches: int = 4) -> int:
    """Kernel launches of the library entry points called since the snapshot `before`
    (fsi_lbm_step launches its face kernel too when the lattice has x faces; the tiled coupled
    substep launches 3 kernels with the coupling inside P2G, 4 with its own kernel, 5 with
    separate force and spread kernels)."""
    from fsi import _native as nat
    table = dict(LAUNCHES, fsi_lbm_step=lbm_step_launches,
                 fsi_coupled_substep_tiled=tiled_substep_launches)
    total = 0
    for name, count in nat.CALLS.items():
        total += (count - before.get(name, 0)) * table.get(name, 1)
    return total


def load_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows: list[list[str]] = []
        self._proc = None
        self._thread = None

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._thread = threading.Thread(target=self._read, daemon=True)
            self._thread.start()
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
            self._thread.join(timeout=5)

    def summary(self) -> dict:
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[0]) for r in self.rows if num(r[0]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for name, v in zip(names, r[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": num(self.rows[0][1]), "reasons": sorted(reasons),
                "samples": len(self.rows),
                "power_w_max": max((num(r[2]) or 0.0) for r in self.rows)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int) -> None:
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    if torch.cuda.is_available():  # the timed GPU arm always has a device; gloo tests do not
        torch.cuda.synchronize()


# ------------------------------------------------------------------ GPU arm

FORM_BYTES = {  # (algorithmic, moved by the fused step) bytes per cell update
    ("f32", "exact"): (LBM_BYTES_PER_CELL, KERNEL_BYTES_PER_CELL),
    ("f32", "fast"): (LBM_BYTES_PER_CELL, KERNEL_BYTES_PER_CELL),
    ("f16", "fast"): (LBM_BYTES_PER_CELL - 76, KERNEL_BYTES_PER_CELL - 76),
    ("bf16", "fast"): (LBM_BYTES_PER_CELL - 76, KERNEL_BYTES_PER_CELL - 76),
}


def time_lbm_forms(lcfg, mask, args, world, stream) -> dict:
    """MLUPS of the lattice step in the other storage / arithmetic forms on the same scene."""
    import dataclasses

    import torch
    from fsi.lbm3d import LBMSolver3D

    peak, _ = load_peaks()
    out = {}
    for (storage, arithmetic), (alg, moved) in FORM_BYTES.items():
        if f"{storage}/{arithmetic}" == args.lbm_form:
            continue
        cfg = dataclasses.replace(lcfg, population_storage=storage, collision_arithmetic=arithmetic)
        lbm = LBMSolver3D(cfg)
        lbm.initialize(mask)
        for _ in range(args.warmup):
            lbm.step()
        barrier(world)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.steps):
            lbm.step()
        b.record(stream)
        barrier(world)
        ms = max_over_ranks(a.elapsed_time(b), world) / args.steps
        cells = lbm.n_cells
        achieved = alg * cells / (ms * 1e-3) / 1e9
        out[f"{storage}/{arithmetic}"] = {
            "value": round(cells / (ms * 1e-3) / 1e6 * world, 3), "unit": "MLUPS",
            "ms_per_step": round(ms, 5), "algorithmic_bytes_per_cell": alg,
            "kernel_bytes_per_cell": moved, "achieved_gbs": round(achieved, 1),
            "frac": round(achieved / peak, 4),
        }
        del lbm
        torch.cuda.empty_cache()
    return out


def time_coupled_extras(args, world, stream, at_scale: bool) -> dict:
    """The coupled smoke workload (48x32x32, one 8^3-cell cube of 4096 particles, 10
    substeps; eager and CUDA-graph steps) and, on the headline scene, the graph-replayed
    steps and the sorted (deterministic) scatter."""
    import dataclasses

    import torch
    from fsi import scenes
    from fsi.simulation import FSISimulation

    out = {}
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn, steps):
        barrier(world)
        a.record(stream)
        fn(steps)
        b.record(stream)
        barrier(world)
        return max_over_ranks(a.elapsed_time(b), world) / steps

    cases = [("smoke_48x32x32", "atomic"), ("smoke_48x32x32", "sorted")]
    if at_scale:
        cases += [("bodies_384x192x192", "atomic"), ("bodies_384x192x192", "sorted")]
    for name, mode in cases:
        if name.startswith("smoke"):
            cfg, solid, pos = scenes.coupled_smoke(100)
            young, steps = None, 100
        else:
            cfg, solid, pos, young = scenes.coupled_bodies()
            steps = args.steps
        cfg = dataclasses.replace(cfg, mpm=dataclasses.replace(cfg.mpm, p2g_mode=mode))
        sim = FSISimulation(cfg)
        sim.initialize_lbm(solid)
        sim.initialize_mpm_from_numpy(pos, youngs_modulus=young,
                                      poisson_ratio=None if young is None else 0.3)
        for _ in range(3):
            sim.coupler.step(cfg.lbm_dt)
        eager_ms = timed(lambda k: [sim.coupler.step(cfg.lbm_dt) for _ in range(k)], steps)
        sim.coupler.step_many(cfg.lbm_dt, 4)
        graph_ms = timed(lambda k: sim.coupler.step_many(cfg.lbm_dt, k), steps)
        sub = cfg.coupling.mpm_substeps_per_lbm_step
        cells = cfg.lbm.nx * cfg.lbm.ny * cfg.lbm.nz
        out[f"{name}_{mode}"] = {
            "p2g_mode": mode, "cells": cells, "particles": int(len(pos)), "substeps": sub,
            "eager_ms_per_step": round(eager_ms, 4), "graph_ms_per_step": round(graph_ms, 4),
            "coupled_steps_per_s": round(1e3 / min(eager_ms, graph_ms) * world, 2),
            "mlups": round(cells / (min(eager_ms, graph_ms) * 1e-3) / 1e6 * world, 2),
            "particle_steps_per_s": round(len(pos) * sub / (min(eager_ms, graph_ms) * 1e-3) * world, 1),
            "graph": "step_many: replays of a captured CUDA graph of two coupled steps "
                     "(capture included)",
        }
        del sim
        torch.cuda.empty_cache()
    return out


def time_headline(args, world, stream) -> dict:
    """The coupled configuration at scale: device-timed coupled steps (state resident), the
    lattice phase alone on the same lattice, and FSISimulation.step end to end."""
    import torch
    from fsi import _native as nat
    from fsi import scenes
    from fsi.simulation import FSISimulation

    from fsi import autotune

    cfg, solid, pos, young = scenes.coupled_bodies()
    sim = FSISimulation(cfg)
    sim.initialize_lbm(solid)
    sim.initialize_mpm_from_numpy(pos, youngs_modulus=young, poisson_ratio=0.3)
    faces = 2 if (sim.lbm.bc_x_left_mode or sim.lbm.bc_x_right_mode) else 1
    sim.coupler.step(cfg.lbm_dt)
    # substep launch parameters by the project's autotuner (state restored afterwards)
    tuning = autotune.tune_coupled(sim, steps=2, use_cache=False)
    for _ in range(args.warmup):
        sim.coupler.step(cfg.lbm_dt)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    before = dict(nat.CALLS)
    a.record(stream)
    for _ in range(args.steps):
        sim.coupler.step(cfg.lbm_dt)
    b.record(stream)
    barrier(world)
    launches = launches_since(before, faces, {1: 3, 2: 4, 3: 5}[tuning["best"][1]])
    step_ms = max_over_ranks(a.elapsed_time(b), world) / args.steps
    base = sim.mpm.base_cells_numpy()
    touched = touched_nodes(base, (cfg.lbm.nx, cfg.lbm.ny, cfg.lbm.nz))
    # the lattice phase alone (same lattice, force and parity cycle)
    barrier(world)
    a.record(stream)
    for _ in range(args.steps):
        sim.lbm.step()
    b.record(stream)
    barrier(world)
    lattice_ms = max_over_ranks(a.elapsed_time(b), world) / args.steps
    # end to end: FSISimulation.step with this step's driving force from pinned host memory
    # and its 18 diagnostics back on the host
    g_host = torch.tensor(cfg.lbm.force, dtype=torch.float32).pin_memory()
    for _ in range(2):
        sim.step(body_force=g_host.numpy())
    barrier(world)
    t0 = time.perf_counter()
    diag = None
    for _ in range(args.steps):
        diag = sim.step(body_force=g_host.numpy())
    barrier(world)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    n_particles = sim.mpm.particle_count()
    out = {
        "step_ms": step_ms, "lattice_ms": lattice_ms, "e2e_s": e2e_s, "launches": launches,
        "tuning": {"threads_per_block": tuning["best"][0],
                   "coupling": {1: "in P2G", 2: "own kernel",
                                3: "force and spread kernels"}[tuning["best"][1]],
                   "candidates_ms_per_step": {k: round(v, 4) for k, v in tuning["ms"].items()}},
        "cells": sim.lbm.n_cells, "fluid_cells": int((solid == 0).sum()),
        "solid_cells": int((solid != 0).sum()), "particles": n_particles, "touched": touched,
        "substeps": cfg.coupling.mpm_substeps_per_lbm_step,
        "last_diagnostics": {k: (v.tolist() if hasattr(v, "tolist") else v)
                             for k, v in (diag or {}).items()},
    }
    del sim
    torch.cuda.empty_cache()
    return out


def time_batched(args, world, stream) -> dict:
    """The batched workload: 256 independent coupled scenes (lattice edges 32-96, 1-4 bodies,
    seed 4) in FP16 deviation storage, advanced together by SceneBatch.run (one launch per
    phase over all scenes, CUDA graph) after autotuning, and by SceneBatch.run_persistent (all
    steps in one persistent cooperative launch); beside it the same per-scene work done one
    scene at a time (FSISimulation, eager) on the first 8 scenes."""
    import torch
    from fsi import scenes
    from fsi.batch import SceneBatch
    from fsi.simulation import FSISimulation

    items = scenes.batch_scenes(count=args.batch_scenes)
    cfgs = [c for c, _, _, _ in items]
    batch = SceneBatch(cfgs)
    batch.initialize([m for _, m, _, _ in items], [p for _, _, p, _ in items],
                     youngs_modulus=[e for _, _, _, e in items],
                     poisson_ratio=[0.3] * len(items))
    rec = batch.autotune(steps=3)
    batch.run(4)
    steps = 10
    barrier(world)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    batch.run(steps)
    b.record(stream)
    barrier(world)
    ms = max_over_ranks(a.elapsed_time(b), world) / steps
    # the same steps as one persistent cooperative launch (grid-wide barriers between phases)
    batch.run_persistent(2)
    barrier(world)
    a.record(stream)
    batch.run_persistent(steps)
    b.record(stream)
    barrier(world)
    persist_ms = max_over_ranks(a.elapsed_time(b), world) / steps
    cells = batch.lattice.cells
    particles = sum(batch.particle_counts)
    sub = batch.substeps
    # one scene at a time (eager FSISimulation steps) on a sample of the same scenes
    sample = items[:8]
    single_ms = 0.0
    single_cells = 0
    for cfg, mask, pos, young in sample:
        sim = FSISimulation(cfg)
        sim.initialize_lbm(mask)
        sim.initialize_mpm_from_numpy(pos, youngs_modulus=young, poisson_ratio=0.3)
        for _ in range(2):
            sim.coupler.step(cfg.lbm_dt)
        a.record(stream)
        for _ in range(3):
            sim.coupler.step(cfg.lbm_dt)
        b.record(stream)
        torch.cuda.synchronize()
        single_ms += a.elapsed_time(b) / 3
        single_cells += cfg.lbm.nx * cfg.lbm.ny * cfg.lbm.nz
        del sim
    single_mlups = single_cells / (single_ms * 1e-3) / 1e6
    out = {
        "scenes": len(items), "cells": cells, "particles": particles, "substeps": sub,
        "storage": "f16", "ms_per_coupled_step": round(ms, 4),
        "scene_steps_per_s": round(len(items) * 1e3 / ms * world, 1),
        "mlups": round(cells / (ms * 1e-3) / 1e6 * world, 1),
        "particle_steps_per_s": round(particles * sub / (ms * 1e-3) * world, 1),
        "autotune": {"best_step_tile_cells": rec["best"][0], "best_variant": rec["best"][1]},
        "one_at_a_time": {"scenes": len(sample), "mlups": round(single_mlups, 1),
                          "mode": "FSISimulation coupler.step, eager, one scene after another"},
        "speedup_vs_one_at_a_time": round(cells / (ms * 1e-3) / 1e6 / single_mlups, 2),
        "gpu_launches": steps * (4 * sub + 3),
        "persistent": {"ms_per_coupled_step": round(persist_ms, 4),
                       "mlups": round(cells / (persist_ms * 1e-3) / 1e6 * world, 1),
                       "launches": 1, "steps_per_launch": steps,
                       "mode": "SceneBatch.run_persistent: one cooperative launch of all steps"},
    }
    del batch
    torch.cuda.empty_cache()
    return out


def time_closure(args, world, stream, snapshots: int = 40, every: int = 3,
                 cell_fraction: float = 0.1, train_steps: int = 4000,
                 rollout_rounds: int = 0) -> dict:
    """Learned coarse-grid closure: steps/s of the coarse 192x96x96 lattice with the fused
    tcgen05 inference and correction after every step, against the plain fine 384x192x192
    lattice (2 fine steps = 1 coarse step of simulated time), on the bodies channel geometry
    (static body masks); and the accuracy protocol of the closure workload at reduced size:
    a network trained here on restricted fine runs of 200 channel scenes (seeds 100-299:
    walls, g_x drive, four static balls, fine 48x24x24 -> coarse 24x12x12; a seeded 10 % of
    each snapshot's cells), evaluated on the 32 held-out scenes of seeds 300-331 for velocity,
    flow rate, body drag and the guards' fallback rate."""
    import torch
    from fsi import closure as cl
    from fsi import scenes
    from fsi.lbm3d import LBMSolver3D

    # --- training and accuracy (reduced-size scenes) ------------------------------
    train_seeds, held_seeds = range(100, 300), range(300, 332)
    t0 = time.perf_counter()
    net = cl.ClosureMLP(seed=0)
    trainer = cl.ClosureTrainer(net)
    train = [scenes.closure_channel(seed) for seed in train_seeds]
    # the 200 fine runs advance as one autotuned LatticeBatch; snapshots over the
    # 120-fine-step window the evaluation covers, from rest
    batch_rec = trainer.add_batch([c for c, _, _ in train], [m for _, m, _ in train],
                                  warmup=0, snapshots=snapshots, every=every,
                                  cell_fraction=cell_fraction, seeds=list(train_seeds))
    del train
    rows = trainer.build()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    hist = trainer.fit(steps=train_steps, batch=16384, lr=2e-3, halvings=5.0)
    b.record(stream)
    torch.cuda.synchronize()
    train_ms = a.elapsed_time(b) / train_steps
    # solver in the loop: pairs along the network's own closure trajectories, then refit
    for r in range(rollout_rounds):
        for seed in train_seeds:
            cfg, mask, _ = scenes.closure_channel(seed)
            trainer.add_rollout_run(cfg, mask, coarse_steps=60, every=3,
                                    cell_fraction=cell_fraction, seed=1000 * (r + 1) + seed)
        rows = trainer.merge()
        hist += trainer.fit(steps=train_steps, batch=16384, lr=1e-3, halvings=5.0, seed=r + 1)
    data_s = time.perf_counter() - t0
    del trainer
    torch.cuda.empty_cache()
    held = []
    for seed in held_seeds:
        cfg, mask, body = scenes.closure_channel(seed)
        held.append(cl.evaluate(cfg, mask, net, coarse_steps=60, body_mask=body, check_every=10))
    acc = {"seeds": f"{held_seeds.start}-{held_seeds.stop - 1}", "scenes": len(held),
           "coarse_steps": 60, "fine_lattice": [48, 24, 24], "coarse_lattice": [24, 12, 12]}
    for h in held:
        h["drag_error_closure_links_only"] = (abs(h["drag_closure_links_only"] - h["drag_fine"])
                                              / abs(h["drag_fine"]))
    for k in ("velocity_l2_plain", "velocity_l2_closure", "flow_rate_error_plain",
              "flow_rate_error_closure", "drag_error_plain", "drag_error_closure",
              "drag_error_closure_links_only", "drag_fine", "drag_plain", "drag_closure",
              "drag_closure_links_only"):
        vals = [h[k] for h in held]
        acc[k + "_mean"] = round(float(np.mean(vals)), 5)
        acc[k + "_max"] = round(float(np.max(vals)), 5)
    acc["fallback_rate"] = sum(h["fallback"] is not None for h in held) / len(held)
    acc["fallback_reasons"] = sorted({h["fallback"] for h in held if h["fallback"]})

    # --- speed on the bodies channel geometry ------------------------------------
    bcfg, bsolid, _, _ = scenes.coupled_bodies()
    fine_cfg = scenes.LBMConfig(nx=bcfg.lbm.nx, ny=bcfg.lbm.ny, nz=bcfg.lbm.nz,
                                viscosity=bcfg.lbm.viscosity, force=(1e-5, 0.0, 0.0),
                                **scenes.PERIODIC_FACES)
    fine = LBMSolver3D(fine_cfg)
    fine.initialize(bsolid)
    sim = cl.ClosureSimulation(fine_cfg, bsolid, net, check_every=0)
    for _ in range(3):
        fine.step()
        sim.step()
    steps = 10
    a.record(stream)
    for _ in range(2 * steps):
        fine.step()
    b.record(stream)
    torch.cuda.synchronize()
    fine_ms = a.elapsed_time(b) / steps  # per coarse-step interval of simulated time
    a.record(stream)
    for _ in range(steps):
        sim.step()
    b.record(stream)
    torch.cuda.synchronize()
    coarse_ms = a.elapsed_time(b) / steps
    net.check()
    cells_c = sim.coarse.n_cells
    mlp_flops = 2.0 * (656 * 64 + 64 * 64 * 2 + 64 * 32) * cells_c
    out = {
        "fine_lattice": [fine_cfg.nx, fine_cfg.ny, fine_cfg.nz],
        "coarse_lattice": [fine_cfg.nx // 2, fine_cfg.ny // 2, fine_cfg.nz // 2],
        "fine_ms_per_2_steps": round(fine_ms, 4), "closure_ms_per_step": round(coarse_ms, 4),
        "speedup_vs_fine": round(fine_ms / coarse_ms, 2),
        "mlp_tflops_per_s_in_step": round(mlp_flops / (coarse_ms * 1e-3) / 1e12, 1),
        "training": {"rows": rows, "scenes": len(train_seeds),
                     "seeds": f"{train_seeds.start}-{train_seeds.stop - 1}",
                     "snapshots_per_scene": snapshots, "cell_fraction": cell_fraction,
                     "rollout_rounds": rollout_rounds,
                     "steps": train_steps, "batch": 16384,
                     "lr": "2e-3 halving 5 times over the run",
                     "occupancy_feature": "solid fraction" if net.use_fraction else "0/1",
                     "ms_per_step": round(train_ms, 3),
                     "loss_first": round(hist[0], 5), "loss_last": round(hist[-1], 5),
                     "wall_s_incl_data": round(data_s, 1),
                     "data": "ClosureTrainer.add_batch: the fine runs as one LatticeBatch "
                             "whose step launch the batch autotuner picked on these scenes",
                     "batch_tuning": {"best_step_tile_cells": (batch_rec["tuning"]["best"]
                                                               or [None])[0],
                                      "candidates_ms_per_step": {
                                          k: round(v, 4) for k, v in
                                          batch_rec["tuning"]["ms"].items()}}},
        "accuracy_heldout": {k: (round(v, 6) if isinstance(v, float) else v)
                             for k, v in acc.items()},
        "gpu_launches": steps * 3 + 2 * steps,
    }
    del fine, sim
    torch.cuda.empty_cache()
    return out


def run_gpu(args) -> dict:
    import torch
    from fsi import scenes
    from fsi.lbm3d import LBMSolver3D
    from fsi.mpm3d import MPMSolver3D

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    peak, peak_kind = load_peaks()

    clocks = ClockSampler(local)
    with clocks:
        time.sleep(0.3)  # let the sampler start before the timed region
        # --- headline: coupled steps at scale --------------------------------------
        head = time_headline(args, world, stream)
        # --- standalone kernels at scale: 256^3 lattice, 2M-particle solid ----------
        import dataclasses
        lcfg, mask = scenes.channel_spheres_lbm(n=args.n)
        storage, arithmetic = args.lbm_form.split("/")
        alg_bytes, moved_bytes = FORM_BYTES[(storage, arithmetic)]
        lbm = LBMSolver3D(dataclasses.replace(lcfg, population_storage=storage,
                                              collision_arithmetic=arithmetic))
        lbm.initialize(mask)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for _ in range(args.warmup):
            lbm.step()
        barrier(world)
        e0.record(stream)
        for _ in range(args.steps):
            lbm.step()
        e1.record(stream)
        barrier(world)
        lbm_ms = max_over_ranks(e0.elapsed_time(e1), world) / args.steps
        cells = lbm.n_cells
        fluid_cells = int((mask == 0).sum())
        del lbm
        torch.cuda.empty_cache()
        mpm_out = {}
        mcfg, pos = scenes.cubes_mpm(n=args.n)
        for mode in ("atomic", "sorted"):
            mpm = MPMSolver3D(dataclasses.replace(mcfg, p2g_mode=mode))
            mpm.initialize_particles_from_numpy(pos)
            for _ in range(args.warmup):
                mpm.substep()
            barrier(world)
            e0.record(stream)
            for _ in range(args.steps):
                mpm.substep()
            e1.record(stream)
            barrier(world)
            mpm_ms = max_over_ranks(e0.elapsed_time(e1), world) / args.steps
            touched = touched_nodes(mpm.base_cells_numpy(), (args.n,) * 3)
            alg = MPM_BYTES_PER_PARTICLE * len(pos) + MPM_BYTES_PER_NODE * touched
            mpm_out[mode] = {"value": round(len(pos) / (mpm_ms * 1e-3) * world, 1),
                             "ms_per_substep": round(mpm_ms, 5),
                             "algorithmic_gbs": round(alg / (mpm_ms * 1e-3) / 1e9, 1),
                             "frac": round(alg / (mpm_ms * 1e-3) / 1e9 / peak, 4)}
            del mpm
            torch.cuda.empty_cache()
        # --- the lattice in the other storage / arithmetic forms ----------------
        forms = time_lbm_forms(lcfg, mask, args, world, stream) if not args.no_forms else {}
        # --- coupled smoke workload, graph replays, sorted scatter ------------------
        coupled = (time_coupled_extras(args, world, stream, not args.no_coupled_scale)
                   if not args.no_coupled else {})
        # --- many scenes at once ------------------------------------------------
        batched = time_batched(args, world, stream) if args.batch_scenes > 0 else {}
        # --- learned coarse-grid closure ------------------------------------------
        learned = time_closure(args, world, stream) if not args.no_closure else {}

    h = head
    step_ms = h["step_ms"]
    lat_bytes = lattice_bytes(h["fluid_cells"], h["solid_cells"])
    mpm_bytes = h["substeps"] * (COUPLED_BYTES_PER_PARTICLE * h["particles"]
                                 + MPM_BYTES_PER_NODE * h["touched"])
    step_bytes = lat_bytes + mpm_bytes
    achieved = step_bytes / (step_ms * 1e-3) / 1e9
    sub_ms = step_ms - h["lattice_ms"]
    lat_alone = lattice_bytes(fluid_cells, cells - fluid_cells, alg_bytes)
    result = {
        "metric": METRIC,
        "value": round(h["cells"] / (step_ms * 1e-3) / 1e6 * world, 3),
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(step_ms, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded scene generators; no dataset)",
        "config": {
            "workload": "coupled at scale: 384x192x192 channel, 48 elastic bodies "
                        f"({h['particles']} particles), 10 MPM substeps per lattice step",
            "step": "LBMMpmCoupler.step: 10 x (coupling + MPM substep), force assembly, "
                    "lattice step (FP32 exact, velocity inlet / pressure outlet faces)",
            "p2g_mode": "atomic",
            "substep_tuning": h["tuning"],
            "lattice": [384, 192, 192], "tau": 0.55, "inflow": 0.05,
            "fluid_cells": h["fluid_cells"], "particles": h["particles"], "substeps": h["substeps"],
            "l2": "inputs larger than L2 (populations 1.08 GB, particles 60 MB, grid 0.23 GB)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
        },
        "particle_steps_per_s": round(h["particles"] * h["substeps"] / (step_ms * 1e-3) * world, 1),
        "coupled_steps_per_s": round(1e3 / step_ms * world, 2),
        "phases_ms": {"lattice_step": round(h["lattice_ms"], 4),
                      "substeps_and_assembly": round(sub_ms, 4)},
        "roofline": {
            "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": TRAFFIC_PER_COUPLED_STEP,
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum summed over the "
                               "launches of one coupled step (the third) of this scene"),
            "kernel": "coupled step (all launches of LBMMpmCoupler.step)",
            "peak_source": peak_kind,
            "algorithmic_bytes_per_step": step_bytes,
            "bytes_basis": ("lattice: 181 B per fluid cell + 4 B per solid cell; per substep: "
                            "224 B per particle + 32 B per touched grid node"),
            "lattice_step": {
                "achieved": round(lat_bytes / (h["lattice_ms"] * 1e-3) / 1e9, 1),
                "frac": round(lat_bytes / (h["lattice_ms"] * 1e-3) / 1e9 / peak, 4)},
            "substeps": {
                "achieved": round(mpm_bytes / (sub_ms * 1e-3) / 1e9, 1),
                "frac": round(mpm_bytes / (sub_ms * 1e-3) / 1e9 / peak, 4)},
        },
        "e2e": {
            "value": round(h["cells"] * args.steps / h["e2e_s"] / 1e6 * world, 3), "unit": "MLUPS",
            "h2d_bytes_per_step": 12, "d2h_bytes_per_step": 264,
            "api": "FSISimulation.step(body_force=g): the step's driving force from pinned host "
                   "memory in, the 18 diagnostics (one 264-byte device record) out",
            "last_diagnostics": h["last_diagnostics"],
        },
        "lattice": {
            "workload": "standalone 256^3 channel, ~10 % static spheres (seed 1), g_x 1e-6",
            "form": args.lbm_form,
            "value": round(cells / (lbm_ms * 1e-3) / 1e6 * world, 3), "unit": "MLUPS",
            "fluid_mlups": round(fluid_cells / (lbm_ms * 1e-3) / 1e6 * world, 3),
            "ms_per_step": round(lbm_ms, 5),
            "achieved_gbs": round(lat_alone / (lbm_ms * 1e-3) / 1e9, 1),
            "frac": round(lat_alone / (lbm_ms * 1e-3) / 1e9 / peak, 4),
            "bytes_basis": f"{alg_bytes} B per fluid cell + 4 B per solid cell",
            "traffic": (round(TRAFFIC_PER_FLUID_CELL[args.lbm_form] * fluid_cells)
                        if args.lbm_form in TRAFFIC_PER_FLUID_CELL else None),
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch of the "
                               "192^3 capture (odd/even average per fluid cell), scaled to this "
                               "lattice's fluid cells"),
        },
        "mpm": {"metric": "particle-steps/s",
                "workload": "64 elastic cubes of 16^3 cells (2,097,152 particles), 256^3 grid",
                **mpm_out},
        "lbm_forms": forms,
        "coupled": coupled,
        "batched": batched,
        "learned_closure": learned,
        "gpu_launches": h["launches"],
        "gpu_launches_basis": "kernel launches of the timed coupled steps (the headline)",
        "clocks": clocks.summary(),
    }
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return result if rank == 0 else None


# --------------------------------------------------------------- CPU leg

# The reference arm times full coupled steps of the headline scene while the whole run stays
# within a few minutes (about 2.5 s per step on 16 Arm cores); longer runs time a bounded sample.
FULL_REFERENCE_STEPS = 40
SAMPLE_SCENE = dict(nx=96, bodies=12)  # the first quarter of the channel, a quarter of the bodies


def cpu_coupled_sample(steps: int, warmup: int, nthreads: int, **scene_kw) -> dict:
    """The oracle (C++ OpenMP restatement of the reference kernels; P2G and the coupling as
    parallel loops with atomic adds, like the reference's parallel Taichi loops) timed on
    coupled steps of the headline scene (scene_kw selects a smaller sample of it)."""
    from fsi import scenes
    from oracle import oracle as O

    cfg, solid, pos, young = scenes.coupled_bodies(**scene_kw)
    sim = O.FSISimulation(cfg, nthreads=nthreads, polar="device", deterministic=False)
    sim.initialize_lbm(solid)
    sim.initialize_mpm_from_numpy(pos)
    for _ in range(warmup):
        sim.coupler.step(cfg.lbm_dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.coupler.step(cfg.lbm_dt)
    dt = (time.perf_counter() - t0) / max(steps, 1)
    cells = cfg.lbm.nx * cfg.lbm.ny * cfg.lbm.nz
    sub = cfg.coupling.mpm_substeps_per_lbm_step
    return {"mlups": cells / dt / 1e6, "s_per_step": dt, "cells": cells,
            "particles": int(len(pos)), "particle_steps_per_s": len(pos) * sub / dt,
            "cores": nthreads, "lattice": [cfg.lbm.nx, cfg.lbm.ny, cfg.lbm.nz]}


def cpu_baseline_entry(nthreads: int) -> dict:
    s = cpu_coupled_sample(steps=2, warmup=1, nthreads=nthreads)
    return {"value": round(s["mlups"], 3), "unit": "MLUPS", "cores": s["cores"], "kind": "port",
            "sample": (f"oracle (C++ OpenMP float32 restatement; Taichi is not installable) on 2 "
                       f"coupled steps of the headline scene ({s['cells']} cells, "
                       f"{s['particles']} particles, 10 substeps each) after 1 warm-up step"),
            "particle_steps_per_s": round(s["particle_steps_per_s"], 1)}


def run_reference(args) -> dict | None:
    world, rank, _ = dist_env()
    if rank != 0:
        return None
    from oracle import oracle as O
    nthreads = O.max_threads()
    full = args.steps + args.warmup <= FULL_REFERENCE_STEPS
    s = cpu_coupled_sample(args.steps, args.warmup, nthreads, **({} if full else SAMPLE_SCENE))
    sample = ("full coupled steps of the headline scene" if full else
              f"coupled steps of a {s['lattice'][0]}x192x192 slab of the headline channel with "
              f"{s['particles']} particles (a bounded sample for long runs)")
    return {
        "impl": "reference",
        "metric": METRIC, "value": round(s["mlups"], 3), "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(s["s_per_step"] * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generators; no dataset)",
        "config": {"workload": "coupled at scale: 384x192x192 channel, 48 elastic bodies, "
                               "10 MPM substeps per lattice step",
                   "sample": sample},
        "particle_steps_per_s": round(s["particle_steps_per_s"], 1),
        "cpu_baseline": {"value": round(s["mlups"], 3), "unit": "MLUPS", "cores": nthreads,
                         "kind": "port",
                         "sample": "reference's Taichi CPU path unavailable (taichi not "
                                   "installable); the oracle restatement of it, all host "
                                   "threads, " + sample},
        "e2e": {"value": round(s["mlups"], 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=256, help="lattice edge (default 256)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lbm-form", default="f32/exact",
                    choices=["f32/exact", "f32/fast", "f16/fast", "bf16/fast"],
                    help="population storage / collision arithmetic of the headline lattice")
    ap.add_argument("--no-coupled", action="store_true", help="skip the extra coupled-step timings")
    ap.add_argument("--no-closure", action="store_true", help="skip the learned-closure section")
    ap.add_argument("--batch-scenes", type=int, default=256,
                    help="scenes of the batched workload (0 skips it)")
    ap.add_argument("--no-coupled-scale", action="store_true",
                    help="skip the extra timings of the headline scene (graph, sorted scatter)")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip timing the FP32-fast / FP16 / BF16 lattice forms")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        out = run_reference(args)
    else:
        out = run_gpu(args)
        world, rank, _ = dist_env()
        if out is not None and world == 1 and not args.no_cpu_baseline:
            from oracle import oracle as O
            out["cpu_baseline"] = cpu_baseline_entry(O.max_threads())
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
