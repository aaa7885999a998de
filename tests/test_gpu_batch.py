"""Batched lattices (fsi.batch.LatticeBatch) against standalone LBMSolver3D runs of the same
configurations: bit-identical in the exact form (shared per-cell code), within float32
rounding in the fast forms (the pairing of cells into packed lanes differs)."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest

from fsi.batch import LatticeBatch
from fsi.config import LBMConfig
from fsi.lbm3d import LBMSolver3D, dhumieres_rates
from helpers import PERIODIC, channel_mask, rel_l2

pytestmark = pytest.mark.gpu


def scenes(storage="f32", arithmetic="auto"):
    rng = np.random.default_rng(4)
    cfgs, masks = [], []
    for n, tau, gx in ((12, 0.6, 1e-5), (9, 0.8, 3e-6), (16, 0.55, 7e-6), (10, 0.7, 0.0)):
        shape = (n, n - 2, n + 1)
        cfg = LBMConfig(nx=shape[0], ny=shape[1], nz=shape[2], viscosity=(tau - 0.5) / 3.0,
                        force=(gx, 0.0, 1e-6), initial_velocity=(1e-3, 0.0, 0.0),
                        population_storage=storage, collision_arithmetic=arithmetic, **PERIODIC)
        m = channel_mask(*shape)
        m[tuple(rng.integers(2, s - 2) for s in shape)] = 1
        cfgs.append(cfg)
        masks.append(m)
    cfgs[3] = dataclasses.replace(cfgs[3], mrt_rates=dhumieres_rates(0.7))
    return cfgs, masks


def run_both(cfgs, masks, steps):
    batch = LatticeBatch(cfgs)
    batch.initialize(masks)
    singles = []
    for c, m in zip(cfgs, masks):
        s = LBMSolver3D(c)
        s.initialize(m)
        singles.append(s)
    for _ in range(steps):
        batch.step()
        for s in singles:
            s.step()
    return batch, singles


@pytest.mark.parametrize("steps", [1, 6, 11])
def test_exact_batch_is_bit_identical(steps):
    cfgs, masks = scenes()
    batch, singles = run_both(cfgs, masks, steps)
    for i, s in enumerate(singles):
        np.testing.assert_array_equal(batch.distribution_numpy(i), s.distribution_numpy())
        np.testing.assert_array_equal(batch.velocity_numpy(i), s.velocity_numpy())
        np.testing.assert_array_equal(batch.density_numpy(i), s.density_numpy())
    diag = batch.mass_and_speed()
    for i, s in enumerate(singles):
        # float32 warp partial sums, float64 across warps: summation order differs
        assert diag[i, 0] == pytest.approx(s.total_mass(), rel=1e-7)
        assert diag[i, 1] == pytest.approx(s.max_velocity_norm(), rel=1e-6)


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
def test_fast_batch_matches_standalone(storage):
    cfgs, masks = scenes(storage, "fast")
    batch, singles = run_both(cfgs, masks, 9)
    for i, s in enumerate(singles):
        assert rel_l2(batch.distribution_numpy(i), s.distribution_numpy()) < 1e-6
        assert rel_l2(batch.velocity_numpy(i), s.velocity_numpy()) < 1e-3


def test_batch_rejects_mixed_forms_and_faces():
    cfgs, _ = scenes()
    with pytest.raises(ValueError):
        LatticeBatch([cfgs[0], dataclasses.replace(cfgs[1], population_storage="f16")])
    from fsi.config import BoundaryConfig
    with pytest.raises(NotImplementedError):
        LatticeBatch([dataclasses.replace(cfgs[0], x_left=BoundaryConfig("velocity"))])


def coupled_scenes():
    from fsi import scenes as sc
    from fsi.config import CouplingConfig, MPMConfig, SimulationConfig
    rng = np.random.default_rng(5)
    cfgs, masks, pos, young = [], [], [], []
    for n, tau, gx, E in ((20, 0.6, 1e-5, 0.05), (16, 0.7, 4e-6, 0.08), (24, 0.55, 7e-6, 0.03)):
        shape = (n + 4, n, n - 2)
        lbm = LBMConfig(nx=shape[0], ny=shape[1], nz=shape[2], viscosity=(tau - 0.5) / 3.0,
                        force=(gx, 0.0, 0.0), **PERIODIC)
        mpm = MPMConfig(nx=shape[0], ny=shape[1], nz=shape[2], max_particles=4096,
                        particles_per_cell=2, dx=1.0, dt=0.1, density=1.5, youngs_modulus=E,
                        poisson_ratio=0.3, gravity=(0.0, 0.0, 0.0), boundary_width=3)
        cfgs.append(SimulationConfig(num_steps=10, lbm_dt=1.0, lbm=lbm, mpm=mpm,
                                     coupling=CouplingConfig(gamma=0.1, mpm_substeps_per_lbm_step=4,
                                                             gamma_ramp_steps=3)))
        masks.append(sc.wall_mask(*shape))
        lo = rng.integers(5, 8, size=3)
        pos.append(sc.cube_particles(lo, 5, 2, rng))
        young.append(E)
    return cfgs, masks, pos, young


@pytest.mark.parametrize("graph", [False, True])
def test_scene_batch_matches_standalone_simulations(graph):
    from fsi.batch import SceneBatch
    from fsi.simulation import FSISimulation
    cfgs, masks, pos, _ = coupled_scenes()
    steps = 9
    batch = SceneBatch(cfgs)
    batch.initialize(masks, pos)
    batch.run(steps, graph=graph)
    assert batch.step_index == steps
    counters = batch.counters_numpy()
    for s, (c, m, p) in enumerate(zip(cfgs, masks, pos)):
        sim = FSISimulation(c)
        sim.initialize_lbm(m)
        sim.initialize_mpm_from_numpy(p)
        for _ in range(steps):
            sim.coupler.step(c.lbm_dt)
        assert rel_l2(batch.density_numpy(s), sim.lbm.density_numpy()) < 1e-5
        # u: float32 order noise of the atomic grid sums (2.5e-4 at 100 steps of the smoke
        # workload, larger relative to the smaller velocities after 9 steps)
        assert rel_l2(batch.velocity_numpy(s), sim.lbm.velocity_numpy()) < 1e-3
        assert rel_l2(batch.positions_numpy(s), sim.mpm.positions_numpy()) < 1e-5
        assert rel_l2(batch.velocities_numpy(s), sim.mpm.velocities_numpy()) < 1e-3
        d = sim.coupler.coupling_diagnostics()
        assert counters[s, 0] == d["unsupported_particle_count"]
        assert counters[s, 1] == d["partial_support_particle_count"]


def test_scene_batch_per_particle_stiffness():
    """Per-scene Young's modulus given to initialize() equals the scenes' own configuration."""
    from fsi.batch import SceneBatch
    cfgs, masks, pos, young = coupled_scenes()
    a = SceneBatch(cfgs)
    a.initialize(masks, pos)
    b = SceneBatch(cfgs)
    b.initialize(masks, pos, youngs_modulus=young, poisson_ratio=[0.3] * 3)
    a.run(4, graph=False)
    b.run(4, graph=False)
    for s in range(3):
        assert rel_l2(b.positions_numpy(s), a.positions_numpy(s)) < 1e-6


def test_autotune_keeps_state_and_results(tmp_path, monkeypatch):
    monkeypatch.setenv("FSI_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    cfgs, masks = scenes()
    a, b = LatticeBatch(cfgs), LatticeBatch(cfgs)
    a.initialize(masks)
    b.initialize(masks)
    for _ in range(3):
        a.step()
        b.step()
    rec = a.autotune(steps=2)
    assert len(rec["ms"]) == 12 and all(v > 0 for v in rec["ms"].values())
    assert a.tuning == {"step_tile_cells": rec["best"][0], "variant": rec["best"][1]}
    for _ in range(5):
        a.step()
        b.step()
    for i in range(len(cfgs)):  # exact form: launch parameters do not change the results
        np.testing.assert_array_equal(a.distribution_numpy(i), b.distribution_numpy(i))
    c = LatticeBatch(cfgs)
    c.initialize(masks)
    assert c.autotune()["best"] == rec["best"]  # from the cache


def test_batch_scene_generator_runs_in_fp16(tmp_path, monkeypatch):
    from fsi import scenes as sc
    from fsi.batch import SceneBatch
    monkeypatch.setenv("FSI_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    items = sc.batch_scenes(count=5, seed=4, edges=(32, 48), substeps=4)
    batch = SceneBatch([c for c, _, _, _ in items])
    batch.initialize([m for _, m, _, _ in items], [p for _, _, p, _ in items],
                     youngs_modulus=[e for _, _, _, e in items], poisson_ratio=[0.3] * 5)
    batch.autotune(steps=2)
    batch.run(6, graph=True)
    for s, (_, _, p, _) in enumerate(items):
        x = batch.positions_numpy(s)
        assert np.all(np.isfinite(x)) and rel_l2(x, p) < 1e-2
        assert np.all(np.isfinite(batch.velocity_numpy(s)))
        rho = batch.density_numpy(s)
        assert abs(float(rho.mean()) - 1.0) < 1e-2


@pytest.mark.parametrize("storage,ib", [("f32", False), ("f16", False), ("f32", True)])
def test_persistent_run_matches_per_phase_steps(storage, ib):
    """SceneBatch.run_persistent (one cooperative launch per run, grid-wide barriers between
    the phases) against the same scenes stepped one launch per phase: the same per-item code
    in the same phase order, so the states agree to the float32 order noise of the atomic grid
    and coupling sums; counters and step bookkeeping are equal."""
    from fsi.batch import SceneBatch
    cfgs, masks, pos, _ = coupled_scenes()
    cfgs = [dataclasses.replace(c, lbm=dataclasses.replace(c.lbm, population_storage=storage),
                                coupling=dataclasses.replace(c.coupling,
                                                             immersed_boundary_enabled=ib,
                                                             immersed_boundary_drag=0.05 * ib))
            for c in cfgs]
    steps = 9
    a, b = SceneBatch(cfgs), SceneBatch(cfgs)
    for x in (a, b):
        x.initialize(masks, pos)
    a.run(steps, graph=False)
    b.run_persistent(steps, max_steps_per_launch=4)
    assert b.step_index == a.step_index == steps
    assert b.lattice.steps_done == a.lattice.steps_done
    np.testing.assert_array_equal(b.counters_numpy()[:, :3], a.counters_numpy()[:, :3])
    if ib:  # immersed-boundary active / clipped cell counts
        np.testing.assert_array_equal(b.counters_numpy()[:, 5:7], a.counters_numpy()[:, 5:7])
    for s in range(len(cfgs)):
        assert rel_l2(b.density_numpy(s), a.density_numpy(s)) < 1e-5
        assert rel_l2(b.velocity_numpy(s), a.velocity_numpy(s)) < 1e-3
        assert rel_l2(b.positions_numpy(s), a.positions_numpy(s)) < 1e-5
        assert rel_l2(b.velocities_numpy(s), a.velocities_numpy(s)) < 1e-3
    # both continue in step: a per-phase step after persistent launches, and the reverse
    a.run_persistent(2)
    b.run(2, graph=False)
    for s in range(len(cfgs)):
        assert rel_l2(b.positions_numpy(s), a.positions_numpy(s)) < 1e-5


def test_persistent_run_reports_a_barrier_wait_that_gave_up():
    """With a wait limit of a few clock cycles the blocks of the persistent launch give up at
    the first grid barrier: the launch ends with FSI_ERR_TIMEOUT in the error word, which
    run_persistent turns into an exception; the device stays usable and a fresh batch runs."""
    from fsi import _native as nat
    from fsi.batch import SceneBatch
    cfgs, masks, pos, _ = coupled_scenes()
    a = SceneBatch(cfgs)
    a.initialize(masks, pos)
    a.step()
    with pytest.raises(nat.NativeError, match="gave up"):
        a.run_persistent(3, wait_cycles=1)
    assert int(a._error.item()) == 0  # cleared after the report
    b, c = SceneBatch(cfgs), SceneBatch(cfgs)
    for x in (b, c):
        x.initialize(masks, pos)
    b.run_persistent(3)
    c.run(3, graph=False)
    for s in range(len(cfgs)):
        assert rel_l2(b.positions_numpy(s), c.positions_numpy(s)) < 1e-5
