"""Launch tuning of the coupled substep on the GPU (fsi.autotune.tune_coupled): every candidate
(threads per block of P2G / G2P, coupling formed inside P2G or by its own kernel) gives the
default launch's results to the float32 order noise of the atomic grid sums, and tuning leaves
the simulation's state where it found it."""
from __future__ import annotations

import numpy as np
import pytest

from fsi import autotune, scenes
from fsi.simulation import FSISimulation
from helpers import rel_l2

pytestmark = pytest.mark.gpu

CANDIDATES = [(t, f) for t in (128, 256, 512) for f in (1, 2, 3)]


def smoke():
    cfg, solid, pos = scenes.coupled_smoke(10)
    sim = FSISimulation(cfg)
    sim.initialize_lbm(solid)
    sim.initialize_mpm_from_numpy(pos)
    return cfg, sim


@pytest.mark.parametrize("threads,fold", CANDIDATES)
def test_every_candidate_matches_the_default_launch(threads, fold):
    cfg, ref = smoke()
    _, sim = smoke()
    autotune.apply_coupled(sim, threads, fold)
    for _ in range(10):
        ref.coupler.step(cfg.lbm_dt)
        sim.coupler.step(cfg.lbm_dt)
    assert rel_l2(sim.mpm.positions_numpy(), ref.mpm.positions_numpy()) < 1e-6
    assert rel_l2(sim.mpm.velocities_numpy(), ref.mpm.velocities_numpy()) < 1e-3
    assert rel_l2(sim.lbm.density_numpy(), ref.lbm.density_numpy()) < 1e-6
    assert rel_l2(sim.lbm.velocity_numpy(), ref.lbm.velocity_numpy()) < 1e-3
    a, b = sim.coupler.coupling_diagnostics(), ref.coupler.coupling_diagnostics()
    for key in ("unsupported_particle_count", "partial_support_particle_count",
                "clipped_particle_count"):
        assert a[key] == b[key], key


def test_tuning_restores_the_state_and_caches_the_choice(tmp_path, monkeypatch):
    monkeypatch.setenv("FSI_AUTOTUNE_CACHE", str(tmp_path / "autotune.json"))
    cfg, sim = smoke()
    for _ in range(3):
        sim.coupler.step(cfg.lbm_dt)
    x0 = sim.mpm.positions_numpy()
    f0 = sim.lbm.distribution_numpy()
    k0 = (sim.coupler.coupled_step, sim.lbm.steps_done)
    rec = autotune.tune_coupled(sim, steps=2)
    assert sorted(rec["ms"]) == sorted(f"{t}/{f}" for t, f in CANDIDATES)
    assert all(v > 0 for v in rec["ms"].values())
    assert tuple(rec["best"]) in CANDIDATES
    assert (sim.mpm.desc.launch_threads, sim.mpm.desc.coupling_fold) == tuple(rec["best"])
    np.testing.assert_array_equal(sim.mpm.positions_numpy(), x0)
    np.testing.assert_array_equal(sim.lbm.distribution_numpy(), f0)
    assert (sim.coupler.coupled_step, sim.lbm.steps_done) == k0
    _, other = smoke()
    assert autotune.tune_coupled(other)["best"] == rec["best"]  # from the cache
    assert other.mpm.tuning == sim.mpm.tuning
