"""Benchmark of the GB300 coupled LBM-MPM kernels on the standalone-at-scale workload.

Workload (seeded, synthetic):
  lattice: 256^3 D3Q19 MRT channel, tau 0.6, g_x = 1e-6, walls in y and z (mask planes),
           ~10% volume of non-overlapping static spheres with radii U[4, 12] (seed 1);
  solid:   64 elastic cubes of 16^3 cells at 8 particles per cell = 2,097,152 particles at
           random positions (seed 2) in a 256^3 grid, gravity -1e-4, dt 0.1.
A timed "step" is one lattice step (value: MLUPS over all cells); the solid is timed the same
way per MPM substep (particle-steps/s) and reported beside it.

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

LBM_BYTES_PER_CELL = 181     # algorithmic bytes per FP32 cell update (pops 152, mask 1, force 12, rho+u 16)
KERNEL_BYTES_PER_CELL = 168  # what the fused step moves: pops 152, flag word 4, force 12
MPM_BYTES_PER_PARTICLE = 200  # algorithmic bytes per particle-substep (standalone)
MPM_BYTES_PER_NODE = 32       # per touched grid node per substep
# DRAM bytes per fluid cell and step kernel launch, from the ncu captures of the 192^3 scene
# (dram__bytes_read.sum + dram__bytes_write.sum, odd/even launch average).
TRAFFIC_PER_FLUID_CELL = {"f32/exact": 177.4, "f16/fast": 96.1}
METRIC = "MLUPS & particle-steps/s on 1 GB300: plain vs FP16/learned, <=1% drag error"


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


def time_coupled(args, world, stream) -> dict:
    """Coupled LBM-MPM steps (LBMMpmCoupler.step) on the coupled smoke workload (48x32x32,
    4096 particles) and the coupled workload at scale (384x192x192, 48 bodies), FP32 exact."""
    import torch
    from fsi import scenes
    from fsi.simulation import FSISimulation

    out = {}
    cases = [("smoke_48x32x32", 100)]
    if not args.no_coupled_scale:
        cases.append(("bodies_384x192x192", 20))
    for name, steps in cases:
        if name.startswith("smoke"):
            cfg, solid, pos = scenes.coupled_smoke(steps)
            young = None
        else:
            cfg, solid, pos, young = scenes.coupled_bodies()
        sim = FSISimulation(cfg)
        sim.initialize_lbm(solid)
        sim.initialize_mpm_from_numpy(pos, youngs_modulus=young,
                                      poisson_ratio=None if young is None else 0.3)
        for _ in range(3):
            sim.coupler.step(cfg.lbm_dt)
        barrier(world)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            sim.coupler.step(cfg.lbm_dt)
        b.record(stream)
        barrier(world)
        eager_ms = max_over_ranks(a.elapsed_time(b), world) / steps
        # the same steps replayed from a captured CUDA graph (capture outside the timed region)
        sim.coupler.step_many(cfg.lbm_dt, 4)
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a.record(stream)
        sim.coupler.step_many(cfg.lbm_dt, steps)
        b.record(stream)
        barrier(world)
        torch.cuda.synchronize()
        graph_wall_ms = (time.perf_counter() - t0) * 1e3 / steps
        ms = max_over_ranks(a.elapsed_time(b), world) / steps
        sub = cfg.coupling.mpm_substeps_per_lbm_step
        cells = cfg.lbm.nx * cfg.lbm.ny * cfg.lbm.nz
        out[name] = {
            "coupled_steps_per_s": round(1e3 / ms * world, 2), "ms_per_step": round(ms, 4),
            "eager_ms_per_step": round(eager_ms, 4),
            "graph_wall_ms_per_step": round(graph_wall_ms, 4),
            "mode": "step_many (CUDA graph of two coupled steps, capture included)",
            "mlups": round(cells / (ms * 1e-3) / 1e6 * world, 2),
            "particle_steps_per_s": round(len(pos) * sub / (ms * 1e-3) * world, 1),
            "cells": cells, "particles": int(len(pos)), "substeps": sub, "timed_steps": steps,
            # per substep: coupling forces + P2G + G2P + block clear; per step: force assembly,
            # lattice step and, with x-face conditions, the face kernel
            "gpu_launches": 2 * steps * (4 * sub + 2 + (1 if sim.lbm.bc_x_left_mode
                                                        or sim.lbm.bc_x_right_mode else 0)),
        }
        del sim
        torch.cuda.empty_cache()
    return out


def time_batched(args, world, stream) -> dict:
    """The batched workload: 256 independent coupled scenes (lattice edges 32-96, 1-4 bodies,
    seed 4) in FP16 deviation storage, advanced together by SceneBatch.run (one launch per
    phase over all scenes, CUDA graph), after autotuning; beside it the same per-scene work
    done one scene at a time (FSISimulation, eager) on the first 8 scenes."""
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
    }
    del batch
    torch.cuda.empty_cache()
    return out


def time_closure(args, world, stream) -> dict:
    """Learned coarse-grid closure: steps/s of the coarse 192x96x96 lattice with the fused
    tcgen05 inference and correction after every step, against the plain fine 384x192x192
    lattice (2 fine steps = 1 coarse step of simulated time), on the bodies channel geometry
    (static body masks); and the accuracy of a network trained here on restricted fine runs
    of small channel scenes (seeds 100-115), evaluated on held-out scenes (seeds 300-302)."""
    import torch
    from fsi import closure as cl
    from fsi import scenes
    from fsi.lbm3d import LBMSolver3D

    # --- training and accuracy on small scenes --------------------------------
    def channel(seed, n=(48, 24, 24)):
        rng = np.random.default_rng(seed)
        nx, ny, nz = n
        mask = scenes.wall_mask(nx, ny, nz)
        for _ in range(4):
            c = [rng.uniform(5, nx - 5), rng.uniform(6, ny - 6), rng.uniform(6, nz - 6)]
            scenes.add_sphere(mask, c, rng.uniform(2.5, 4.5))
        cfg = scenes.LBMConfig(nx=nx, ny=ny, nz=nz, viscosity=(0.6 - 0.5) / 3.0,
                               force=(2e-5, 0.0, 0.0), **scenes.PERIODIC_FACES)
        return cfg, mask

    t0 = time.perf_counter()
    net = cl.ClosureMLP(seed=0)
    trainer = cl.ClosureTrainer(net)
    for seed in range(100, 116):
        cfg, mask = channel(seed)
        # snapshots over the whole 120-fine-step window the evaluation covers, from rest
        trainer.add_run(cfg, mask, warmup=0, snapshots=40, every=3)
    rows = trainer.build()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    train_steps = 3000
    hist = trainer.fit(steps=train_steps, batch=16384, lr=2e-3, halvings=5.0)
    b.record(stream)
    torch.cuda.synchronize()
    train_ms = a.elapsed_time(b) / train_steps
    train_s = time.perf_counter() - t0
    held = [cl.evaluate(*channel(seed), net, coarse_steps=60) for seed in (300, 301, 302)]
    acc = {"seeds": [300, 301, 302], "coarse_steps": 60}
    for k in ("velocity_l2_plain", "velocity_l2_closure", "flow_rate_error_plain", "flow_rate_error_closure"):
        acc[k] = [round(h[k], 5) for h in held]
        acc[k + "_mean"] = round(float(np.mean([h[k] for h in held])), 5)
    acc["fallback"] = [h["fallback"] for h in held]

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
        "training": {"rows": rows, "scenes": 16, "steps": train_steps, "batch": 16384,
                     "lr": "2e-3 halving 5 times over the run",
                     "occupancy_feature": "solid fraction" if net.use_fraction else "0/1",
                     "ms_per_step": round(train_ms, 3),
                     "loss_first": round(hist[0], 5), "loss_last": round(hist[-1], 5),
                     "wall_s_incl_data": round(train_s, 1)},
        "accuracy_heldout_48x24x24": {k: (round(v, 5) if isinstance(v, float) else v)
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

    import dataclasses
    lcfg, mask = scenes.channel_spheres_lbm(n=args.n)
    storage, arithmetic = args.lbm_form.split("/")
    head_cfg = dataclasses.replace(lcfg, population_storage=storage, collision_arithmetic=arithmetic)
    alg_bytes, moved_bytes = FORM_BYTES[(storage, arithmetic)]
    lbm = LBMSolver3D(head_cfg)
    lbm.initialize(mask)
    cells = lbm.n_cells
    fluid_cells = int((mask == 0).sum())

    mcfg, pos = scenes.cubes_mpm(n=args.n)
    mpm = MPMSolver3D(mcfg)
    mpm.initialize_particles_from_numpy(pos)
    particles = mpm.particle_count()

    stream = torch.cuda.current_stream()
    # --- lattice, device-resident -------------------------------------------------
    for _ in range(args.warmup):
        lbm.step()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    m0, m1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    with clocks:
        time.sleep(0.3)  # let the sampler start before the timed region
        e0.record(stream)
        for _ in range(args.steps):
            lbm.step()
        e1.record(stream)
        barrier(world)
        # --- solid, device-resident -----------------------------------------------
        for _ in range(args.warmup):
            mpm.substep()
        barrier(world)
        m0.record(stream)
        for _ in range(args.steps):
            mpm.substep()
        m1.record(stream)
        barrier(world)
        # --- the lattice in the other storage / arithmetic forms ----------------
        forms = time_lbm_forms(lcfg, mask, args, world, stream) if not args.no_forms else {}
        # --- coupled steps -------------------------------------------------------
        coupled = time_coupled(args, world, stream) if not args.no_coupled else {}
        # --- many scenes at once ------------------------------------------------
        batched = time_batched(args, world, stream) if args.batch_scenes > 0 else {}
        # --- learned coarse-grid closure ------------------------------------------
        learned = time_closure(args, world, stream) if not args.no_closure else {}
    lbm_ms = max_over_ranks(e0.elapsed_time(e1), world) / args.steps
    lbm_launches = args.steps
    mpm_ms = max_over_ranks(m0.elapsed_time(m1), world) / args.steps
    base = mpm.base_cells_numpy().astype(np.int64)
    # grid nodes touched per substep: the union of the particles' 27-node stencils
    occupied = np.unique((base[:, 0] * args.n + base[:, 1]) * args.n + base[:, 2])
    oi, oj, ok = occupied // (args.n * args.n), (occupied // args.n) % args.n, occupied % args.n
    stencil = np.unique(np.concatenate([((oi + di) * args.n + oj + dj) * args.n + ok + dk
                                        for di in range(3) for dj in range(3) for dk in range(3)]))
    touched = int(len(stencil))

    # --- end to end through the public API (host input, host result each step) ----
    g_host = np.array(lcfg.force, dtype=np.float32)
    for _ in range(2):
        lbm.set_uniform_force(g_host)
        lbm.step()
        lbm.total_mass()
    barrier(world)
    t0 = time.perf_counter()
    diag = None
    for _ in range(args.steps):
        lbm.set_uniform_force(g_host)   # 12 B of step input from the host
        lbm.step()
        diag = (lbm.total_mass(), lbm.max_velocity_norm())  # 16 B of step result to the host
    barrier(world)
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)

    peak, peak_kind = load_peaks()
    achieved = alg_bytes * cells / (lbm_ms * 1e-3) / 1e9
    mlups = cells / (lbm_ms * 1e-3) / 1e6
    result = {
        "metric": METRIC,
        "value": round(mlups * world, 3),
        "unit": "MLUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(lbm_ms, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if storage == "f32" else f"{storage} storage, f32 arithmetic",
        "data": "synthetic (seeded scene generators; no dataset)",
        "config": {
            "workload": "standalone lattice 256^3 channel + 64 elastic cubes (2,097,152 particles)",
            "lbm_form": args.lbm_form,
            "lattice": [args.n] * 3, "tau": 0.6, "g_x": 1e-6,
            "solid_fraction": round(float(mask.mean()), 4),
            "fluid_cells": fluid_cells,
            "particles": particles, "mpm_dt": 0.1, "gravity_y": -1e-4,
            "l2": "inputs larger than L2 (populations 1.27 GB, particles 0.25 GB)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
        },
        "fluid_mlups": round(fluid_cells / (lbm_ms * 1e-3) / 1e6 * world, 3),
        "mpm": {
            "metric": "particle-steps/s",
            "value": round(particles / (mpm_ms * 1e-3) * world, 1),
            "ms_per_substep": round(mpm_ms, 5),
            "algorithmic_gbs": round((MPM_BYTES_PER_PARTICLE * particles
                                      + MPM_BYTES_PER_NODE * touched) / (mpm_ms * 1e-3) / 1e9, 1),
        },
        "roofline": {
            "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4),
            "traffic": (round(TRAFFIC_PER_FLUID_CELL[args.lbm_form] * fluid_cells)
                        if args.lbm_form in TRAFFIC_PER_FLUID_CELL else None),
            "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch of the "
                               "192^3 capture (odd/even average per fluid cell), scaled to this "
                               "lattice's fluid cells"),
            "kernel": "lbm_step_kernel", "peak_source": peak_kind,
            "algorithmic_bytes_per_cell": alg_bytes,
            "kernel_bytes_per_cell": moved_bytes,
        },
        "e2e": {
            "value": round(cells * args.steps / e2e_s / 1e6 * world, 3), "unit": "MLUPS",
            "h2d_bytes_per_step": 12, "d2h_bytes_per_step": 16,
            "api": "LBMSolver3D.set_uniform_force + step + total_mass + max_velocity_norm",
            "last_diagnostics": [float(diag[0]), float(diag[1])] if diag else None,
        },
        "lbm_forms": forms,
        "coupled": coupled,
        "batched": batched,
        "learned_closure": learned,
        # lattice steps + 3 MPM launches per substep + 3 launches per end-to-end step
        # (force op, step, fused macro + diagnostics) + one step per form per step + coupled
        "gpu_launches": (lbm_launches + 3 * args.steps + 3 * args.steps + len(forms) * args.steps
                         + sum(c["gpu_launches"] for c in coupled.values())
                         + batched.get("gpu_launches", 0) + learned.get("gpu_launches", 0)),
        "clocks": clocks.summary(),
    }
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return result if rank == 0 else None


# --------------------------------------------------------------- CPU leg

def cpu_sample(steps: int, warmup: int, nthreads: int, n: int = 256, slab: int = 32,
               cubes: int = 8) -> dict:
    """The oracle (C++ OpenMP restatement of the reference) on a bounded sample of the same
    workload: a slab of `slab` x n x n cells of the lattice and `cubes` of the 64 cubes."""
    from fsi import scenes
    from oracle import oracle as O

    lcfg, mask = scenes.channel_spheres_lbm(n=n)
    sub = mask[:slab].copy()
    from dataclasses import replace
    scfg = replace(lcfg, nx=slab)
    lbm = O.LBMSolver3D(scfg, nthreads=nthreads)
    lbm.initialize(sub)
    for _ in range(warmup):
        lbm.step()
    t0 = time.perf_counter()
    for _ in range(steps):
        lbm.step()
    lbm_s = time.perf_counter() - t0
    mcfg, pos = scenes.cubes_mpm(n=n)
    per_cube = len(pos) // 64
    pos = pos[: cubes * per_cube]
    mpm = O.MPMSolver3D(replace(mcfg, max_particles=len(pos)), nthreads=nthreads,
                        deterministic=False)
    mpm.initialize_particles_from_numpy(pos)
    for _ in range(max(1, warmup // 2)):
        mpm.substep()
    t1 = time.perf_counter()
    for _ in range(steps):
        mpm.substep()
    mpm_s = time.perf_counter() - t1
    cells = slab * n * n
    return {"mlups": cells * steps / lbm_s / 1e6, "lbm_s_per_step": lbm_s / steps,
            "particle_steps_per_s": len(pos) * steps / mpm_s, "mpm_s_per_substep": mpm_s / steps,
            "cells": cells, "particles": len(pos), "cores": nthreads}


def cpu_baseline_entry(nthreads: int) -> dict:
    s = cpu_sample(steps=3, warmup=1, nthreads=nthreads)
    return {"value": round(s["mlups"], 3), "unit": "MLUPS", "cores": s["cores"], "kind": "port",
            "sample": (f"oracle (C++ OpenMP float32 restatement; Taichi is not installable) on a "
                       f"32x256x256 slab of the lattice ({s['cells']} cells, 3 steps) and 8 of the "
                       f"64 cubes ({s['particles']} particles, 3 substeps)"),
            "particle_steps_per_s": round(s["particle_steps_per_s"], 1)}


def run_reference(args) -> dict | None:
    world, rank, _ = dist_env()
    if rank != 0:
        return None
    from oracle import oracle as O
    nthreads = O.max_threads()
    s = cpu_sample(steps=args.steps, warmup=args.warmup, nthreads=nthreads)
    return {
        "impl": "reference",
        "metric": METRIC, "value": round(s["mlups"], 3), "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(s["lbm_s_per_step"] * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generators; no dataset)",
        "config": {"workload": "standalone lattice 256^3 channel + 64 elastic cubes (2,097,152 particles)",
                   "sample": "32x256x256 lattice slab per step; 8 of 64 cubes per substep"},
        "mpm": {"metric": "particle-steps/s", "value": round(s["particle_steps_per_s"], 1)},
        "cpu_baseline": {"value": round(s["mlups"], 3), "unit": "MLUPS", "cores": nthreads,
                         "kind": "port",
                         "sample": "reference's Taichi CPU path unavailable (taichi not installable); "
                                   "the oracle restatement of it, all host threads"},
        "e2e": {"value": round(s["mlups"], 3), "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=256, help="lattice edge (default 256)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lbm-form", default="f32/exact",
                    choices=["f32/exact", "f32/fast", "f16/fast", "bf16/fast"],
                    help="population storage / collision arithmetic of the headline lattice")
    ap.add_argument("--no-coupled", action="store_true", help="skip the coupled-step timings")
    ap.add_argument("--no-closure", action="store_true", help="skip the learned-closure section")
    ap.add_argument("--batch-scenes", type=int, default=256,
                    help="scenes of the batched workload (0 skips it)")
    ap.add_argument("--no-coupled-scale", action="store_true",
                    help="time only the small coupled workload")
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
