"""Host logic of the batched-step autotuner (no GPU): candidate launch parameters per
arithmetic form, the JSON cache (round trip, damaged or unwritable file), the cache key and
the cached path that applies a stored choice without timing anything."""
from __future__ import annotations

import json
from types import SimpleNamespace

import pytest

from fsi import autotune


class _Cfg:
    def __init__(self, storage="f32", arithmetic="exact"):
        self.population_storage = storage
        self._arith = arithmetic

    def resolved_arithmetic(self):
        return self._arith


def _batch(shapes=((16, 8, 8), (8, 8, 8)), **cfg):
    return SimpleNamespace(configs=[_Cfg(**cfg) for _ in shapes], shapes=list(shapes),
                           _initialized=True, _handle=object(), tuning=None)


@pytest.fixture
def cache(tmp_path, monkeypatch):
    path = tmp_path / "tune" / "autotune.json"
    monkeypatch.setenv("FSI_AUTOTUNE_CACHE", str(path))
    monkeypatch.setattr(autotune.torch.cuda, "get_device_name", lambda *a: "GB300 (fake)")
    return path


def test_candidates_follow_the_cells_per_thread_of_the_form():
    exact = autotune.candidates(_batch(arithmetic="exact"))
    fast = autotune.candidates(_batch(arithmetic="fast"))
    assert exact == [(t, v) for t in (128, 256, 512, 1024) for v in (0, 1, 2)]
    # two cells per thread: tiles must hold whole 256-cell passes
    assert fast == [(t, v) for t in (256, 512, 1024) for v in (0, 1, 2)]


def test_cache_round_trip_and_damaged_file(cache):
    assert autotune._load() == {}
    autotune._store("k1", {"best": [256, 1]})
    autotune._store("k2", {"best": [512, 0]})
    assert json.loads(cache.read_text()) == {"k1": {"best": [256, 1]}, "k2": {"best": [512, 0]}}
    cache.write_text("{ not json")
    assert autotune._load() == {}


def test_unwritable_cache_only_loses_the_cache(tmp_path, monkeypatch):
    blocker = tmp_path / "file"
    blocker.write_text("x")
    monkeypatch.setenv("FSI_AUTOTUNE_CACHE", str(blocker / "sub" / "autotune.json"))
    autotune._store("k", {"best": [128, 0]})  # parent is a file: no exception
    assert autotune._load() == {}


def test_signature_ignores_scene_order_and_tracks_form_and_sizes(cache):
    a = autotune._signature(_batch(shapes=((16, 8, 8), (8, 8, 8))))
    b = autotune._signature(_batch(shapes=((8, 8, 8), (16, 8, 8))))
    assert a == b
    assert a != autotune._signature(_batch(storage="f16", arithmetic="fast"))
    assert a != autotune._signature(_batch(shapes=((16, 8, 8), (8, 8, 16))))


def test_cached_choice_is_applied_without_timing(cache, monkeypatch):
    calls = []
    monkeypatch.setattr(autotune.nat, "call", lambda name, *args: calls.append((name, args[1:])))
    batch = _batch()
    batch.snapshot = lambda: pytest.fail("a cached choice must not time candidates")
    rec = {"best": [512, 2], "ms": {"512/2": 1.0}, "steps": 4}
    autotune._store(autotune._signature(batch), rec)
    assert autotune.tune_lattice_batch(batch) == rec
    assert calls == [("fsi_batch_tune", (512, 2))]
    assert batch.tuning == {"step_tile_cells": 512, "variant": 2}


def test_tuning_needs_an_initialized_batch(cache):
    batch = _batch()
    batch._initialized = False
    with pytest.raises(RuntimeError):
        autotune.tune_lattice_batch(batch)


def _sim(p2g_mode="atomic", particles=4096, shape=(48, 32, 32)):
    from fsi import _native as nat
    lbm = SimpleNamespace(nx=shape[0], ny=shape[1], nz=shape[2], population_storage="f32")
    cfg = SimpleNamespace(lbm=lbm, mpm=SimpleNamespace(p2g_mode=p2g_mode), lbm_dt=1.0)
    mpm = SimpleNamespace(desc=nat.MpmDesc(), tuning=None, particle_count=lambda: particles)
    return SimpleNamespace(config=cfg, mpm=mpm)


def test_coupled_candidates_and_signature(cache):
    assert autotune.coupled_candidates(_sim()) == [(t, f) for t in (128, 256, 512) for f in (1, 2, 3)]
    assert autotune.coupled_candidates(_sim(p2g_mode="sorted")) == []
    a = autotune.coupled_signature(_sim(particles=502304))
    # nearby particle counts share a record, other shapes and modes do not
    assert autotune.coupled_signature(_sim(particles=502000)) == a
    assert autotune.coupled_signature(_sim(particles=251000)) != a
    assert autotune.coupled_signature(_sim(particles=502304, shape=(48, 32, 16))) != a
    assert autotune.coupled_signature(_sim(particles=502304, p2g_mode="sorted")) != a


def test_coupled_tuning_from_the_cache_applies_without_timing(cache):
    sim = _sim()
    autotune._store(autotune.coupled_signature(sim), {"best": [512, 2], "ms": {}})
    rec = autotune.tune_coupled(sim)  # no GPU: only the cached path can run
    assert rec["best"] == [512, 2]
    assert (sim.mpm.desc.launch_threads, sim.mpm.desc.coupling_fold) == (512, 2)
    assert sim.mpm.tuning == {"launch_threads": 512, "coupling_fold": 2}
    assert autotune.tune_coupled(_sim(p2g_mode="sorted")) == {"best": None, "ms": {}}
