"""Autotuners of launch parameters (no reference counterpart): the batched lattice step
(``tune_lattice_batch``) and the coupled substep of one scene (``tune_coupled``).

Batched step: candidates are (cells per thread block, register-cap variant) pairs of
``fsi_batch_tune``.
Each is timed with CUDA events over a few lattice steps of the actual batch, from a
snapshot of the batch's state that is restored afterwards, so tuning leaves the
simulation where it was. The fastest choice is applied and stored, with every candidate's
timing, in a JSON cache keyed by the GPU, the storage / arithmetic form and the batch's
lattice sizes, so a later batch of the same shape starts tuned.

Coupled substep: candidates are (threads per block of P2G and G2P, coupling placement) pairs
of the tiled scatter's descriptor fields (``fsi_mpm_desc.launch_threads``, ``coupling_fold``),
timed on whole coupled steps of the simulation from a snapshot of its state that is restored
afterwards, cached under the GPU, grid shape, particle count, scatter mode and storage.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

import torch

from . import _native as nat


def cache_path() -> Path:
    return Path(os.environ.get("FSI_AUTOTUNE_CACHE",
                               Path.home() / ".cache" / "fsi_gb300" / "autotune.json"))


def _signature(batch) -> str:
    c0 = batch.configs[0]
    shapes = sorted(batch.shapes)
    text = json.dumps([torch.cuda.get_device_name(), c0.population_storage,
                       c0.resolved_arithmetic(), shapes])
    return hashlib.sha1(text.encode()).hexdigest()


def candidates(batch) -> list[tuple[int, int]]:
    lanes = 2 if batch.configs[0].resolved_arithmetic() == "fast" else 1
    tiles = [t for t in (128, 256, 512, 1024) if t % (128 * lanes) == 0]
    return [(t, v) for t in tiles for v in (0, 1, 2)]


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(key: str, record: dict) -> None:
    path = cache_path()
    data = _load()
    data[key] = record
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(data, indent=1))
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home only loses the cache


def apply(batch, tile_cells: int, variant: int) -> None:
    nat.call("fsi_batch_tune", batch._handle, int(tile_cells), int(variant))
    batch.tuning = {"step_tile_cells": int(tile_cells), "variant": int(variant)}


def tune_lattice_batch(batch, steps: int = 4, use_cache: bool = True) -> dict:
    """Choose and apply the fastest step launch parameters for ``batch`` (a LatticeBatch);
    returns the record {"best": [tile_cells, variant], "ms": {candidate: ms per step}}."""
    if not batch._initialized:
        raise RuntimeError("initialize the batch before tuning it.")
    key = _signature(batch)
    if use_cache:
        rec = _load().get(key)
        if rec:
            apply(batch, *rec["best"])
            return rec
    snap = batch.snapshot()
    timings = {}
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for tile, variant in candidates(batch):
        apply(batch, tile, variant)
        batch.restore(snap)
        batch.step()  # warm-up (first launch of this variant)
        torch.cuda.synchronize()
        start.record()
        for _ in range(steps):
            batch.step()
        end.record()
        torch.cuda.synchronize()
        timings[f"{tile}/{variant}"] = start.elapsed_time(end) / steps
    best = min(timings, key=timings.get)
    tile, variant = (int(x) for x in best.split("/"))
    apply(batch, tile, variant)
    batch.restore(snap)
    rec = {"best": [tile, variant], "ms": timings, "steps": steps}
    _store(key, rec)
    return rec


# ------------------------------------------------------------- coupled scene
def coupled_signature(sim) -> str:
    """Cache key of a coupled simulation's substep tuning: the GPU, the lattice / grid shape,
    the particle count (rounded to 1/16 of a power of two: nearby counts share a record), the
    scatter mode and the lattice storage."""
    n = max(int(sim.mpm.particle_count()), 1)
    bucket = 1 << max(n.bit_length() - 5, 0)
    c = sim.config
    text = json.dumps([torch.cuda.get_device_name(), "coupled", [c.lbm.nx, c.lbm.ny, c.lbm.nz],
                       (n + bucket - 1) // bucket * bucket, c.mpm.p2g_mode,
                       c.lbm.population_storage])
    return hashlib.sha1(text.encode()).hexdigest()


def coupled_candidates(sim) -> list[tuple[int, int]]:
    """(threads per block of P2G / G2P, coupling placement) pairs of the tiled (atomic)
    scatter: 128, 256 or 512 particles share a shared-memory tile; the coupling force is formed
    inside P2G (1), by its own kernel first (2), or by a force kernel and a spread kernel (3).
    The sorted scatter has no such choice."""
    if sim.config.mpm.p2g_mode == "sorted":
        return []
    return [(t, f) for t in (128, 256, 512) for f in (1, 2, 3)]


def apply_coupled(sim, threads: int, fold: int) -> None:
    d = sim.mpm.desc
    d.launch_threads, d.coupling_fold = int(threads), int(fold)
    sim.mpm.tuning = {"launch_threads": int(threads), "coupling_fold": int(fold)}


def tune_coupled(sim, steps: int = 2, use_cache: bool = True) -> dict:
    """Choose and apply the fastest substep launch parameters for ``sim`` (an initialised
    FSISimulation) by timing ``steps`` coupled steps per candidate from a snapshot of the
    simulation's state, restored afterwards (the simulation continues from where it was).
    Returns {"best": [threads, fold], "ms": {candidate: ms per coupled step}}."""
    cands = coupled_candidates(sim)
    if not cands:
        return {"best": None, "ms": {}}
    key = coupled_signature(sim)
    if use_cache:
        rec = _load().get(key)
        if rec and rec.get("best"):
            apply_coupled(sim, *rec["best"])
            return rec
    snap = sim.state_dict()
    dt = sim.config.lbm_dt
    timings = {}
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for threads, fold in cands:
        apply_coupled(sim, threads, fold)
        sim.load_state_dict(snap)
        sim.coupler.step(dt)  # warm-up (first launch of this variant)
        torch.cuda.synchronize()
        start.record()
        for _ in range(steps):
            sim.coupler.step(dt)
        end.record()
        torch.cuda.synchronize()
        timings[f"{threads}/{fold}"] = start.elapsed_time(end) / steps
    best = min(timings, key=timings.get)
    threads, fold = (int(x) for x in best.split("/"))
    apply_coupled(sim, threads, fold)
    sim.load_state_dict(snap)
    rec = {"best": [threads, fold], "ms": timings, "steps": steps}
    _store(key, rec)
    return rec
