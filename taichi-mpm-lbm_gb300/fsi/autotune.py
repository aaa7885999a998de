"""Autotuner of the batched lattice step's launch parameters (no reference counterpart).

Candidates are (cells per thread block, register-cap variant) pairs of ``fsi_batch_tune``.
Each is timed with CUDA events over a few lattice steps of the actual batch, from a
snapshot of the batch's state that is restored afterwards, so tuning leaves the
simulation where it was. The fastest choice is applied and stored, with every candidate's
timing, in a JSON cache keyed by the GPU, the storage / arithmetic form and the batch's
lattice sizes, so a later batch of the same shape starts tuned.
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
