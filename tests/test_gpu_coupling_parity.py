"""GPU coupling vs the CPU oracle, the reference's coupling tests, and the goldens.

Single-particle coupling evaluations are bit-exact (each node receives one
contribution, so atomic ordering cannot matter). The 48x32x32 coupled smoke
workload with the sorted scatter (p2g_mode="sorted") against the oracle summing in
the same cell order is bit-identical for ten steps and within relative L2 1e-5 for
density, velocity, particle positions and velocities after 100; with the default
atomic scatter, against the serial oracle, density and positions are within 1e-5
and velocity within its float32 order noise. Masks and counters match exactly.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np
import pytest

import fsi.reference_cases as rc
import fsi.validation_cases as vc
from fsi.config import CouplingConfig, SimulationConfig
from fsi.coupling import LBMMpmCoupler
from fsi.lbm3d import LBMSolver3D
from fsi.mpm3d import MPMSolver3D
from fsi.simulation import FSISimulation
from helpers import coupled_smoke_config, periodic_lbm, rel_l2, small_mpm
from oracle import oracle as O

pytestmark = pytest.mark.gpu
NTHREADS = os.cpu_count() or 1


def pair(cfg: CouplingConfig, *, lbm_velocity=(1.0, 0.0, 0.0), position=(4.0, 4.0, 4.0),
         velocity=(0.0, 0.0, 0.0), mass=1.0, volume=1.0, solid=None):
    out = []
    for L, M, C in ((LBMSolver3D, MPMSolver3D, LBMMpmCoupler),
                    (O.LBMSolver3D, O.MPMSolver3D, O.LBMMpmCoupler)):
        lbm = L(periodic_lbm(initial_velocity=lbm_velocity))
        lbm.initialize(solid)
        mpm = M(small_mpm())
        mpm.initialize_particles_from_numpy(np.array([position], np.float32),
                                            np.array([velocity], np.float32), mass, volume)
        out.append(C(cfg, lbm, mpm))
    return out


def assert_coupling_equal(g, o):
    np.testing.assert_array_equal(g.mpm.particle_forces_numpy(), o.mpm.particle_forces_numpy())
    np.testing.assert_array_equal(g.coupling_force_numpy(), o.coupling_force_numpy())
    np.testing.assert_array_equal(g.solid_volume_fraction_numpy(), o.solid_volume_fraction_numpy())
    np.testing.assert_array_equal(g.particle_valid_weights_numpy(), o.particle_valid_weights_numpy())
    np.testing.assert_array_equal(g.particle_coupling_mask_numpy(), o.particle_coupling_mask_numpy())
    np.testing.assert_array_equal(g.particle_contact_mask_numpy(), o.particle_contact_mask_numpy())
    np.testing.assert_array_equal(g.immersed_boundary_force_numpy(), o.immersed_boundary_force_numpy())
    np.testing.assert_array_equal(g.mpm.velocities_numpy(), o.mpm.velocities_numpy())
    dg, do = g.coupling_diagnostics(), o.coupling_diagnostics()
    for key in ("unsupported_particle_count", "partial_support_particle_count",
                "clipped_particle_count", "ib_active_cell_count", "ib_clipped_cell_count",
                "contact_candidate_count", "contact_damped_particle_count"):
        assert dg[key] == do[key], key
    assert dg["ib_total_force_x"] == pytest.approx(do["ib_total_force_x"], rel=1e-5, abs=1e-12)
    assert dg["effective_gamma"] == pytest.approx(do["effective_gamma"])


SOLID_1 = np.zeros((8, 8, 8), np.int32)
SOLID_1[4, 4, 4] = 1
SOLID_BLOCK = np.zeros((8, 8, 8), np.int32)
SOLID_BLOCK[3:6, 3:6, 3:6] = 1


@pytest.mark.parametrize("cfg,kw", [
    (CouplingConfig(gamma=0.05), dict(lbm_velocity=(1e-4, 0, 0), mass=2.0)),
    (CouplingConfig(gamma=100.0, force_limit=0.05), {}),
    (CouplingConfig(gamma=10.0, relative_velocity_limit=0.01), dict(mass=2.0)),
    (CouplingConfig(gamma=10.0, gamma_ramp_steps=4), {}),
    (CouplingConfig(gamma=1.0), dict(position=(-0.75, 4.0, 4.0))),
    (CouplingConfig(gamma=1.0), dict(solid=SOLID_1)),
    (CouplingConfig(gamma=1.0), dict(solid=SOLID_BLOCK)),
    (CouplingConfig(gamma=0.0, immersed_boundary_enabled=True, immersed_boundary_drag=0.5,
                    immersed_boundary_fraction_threshold=0.01),
     dict(lbm_velocity=(1e-3, 0, 0), volume=4.0)),
    (CouplingConfig(gamma=0.0, immersed_boundary_enabled=True, immersed_boundary_drag=100.0,
                    immersed_boundary_fraction_threshold=0.01, immersed_boundary_max_force=1e-5),
     dict(lbm_velocity=(1e-3, 0, 0), volume=4.0)),
    (CouplingConfig(gamma=0.0, contact_enabled=True, contact_velocity_damping=0.25,
                    contact_fraction_threshold=0.01),
     dict(lbm_velocity=(1e-3, 0, 0), velocity=(0.1, 0, 0), solid=SOLID_BLOCK)),
])
def test_single_particle_coupling_bit_exact(cfg, kw):
    g, o = pair(cfg, **kw)
    g.compute_coupling_forces(dt_ratio=1.0)
    o.compute_coupling_forces(dt_ratio=1.0)
    assert_coupling_equal(g, o)


def test_reference_coupling_assertions():
    """The reference's tests/test_coupling*.py and IB/contact assertions."""
    g, _ = pair(CouplingConfig(gamma=0.05), lbm_velocity=(1e-4, 0, 0), mass=2.0)
    g.compute_coupling_forces(dt_ratio=1.0)
    fp, ff = g.total_particle_coupling_force(), g.total_fluid_coupling_force()
    assert fp[0] > 0 and ff[0] < 0
    np.testing.assert_allclose(fp + ff * g.cell_volume, 0.0, rtol=1e-5, atol=1e-7)
    g, _ = pair(CouplingConfig(gamma=10.0, gamma_ramp_steps=4))
    assert g.effective_gamma() == pytest.approx(2.5)
    g, _ = pair(CouplingConfig(gamma=4.0, gamma_ramp_steps=4, force_limit=0.1),
                lbm_velocity=(1e-3, 0, 0))
    assert g.effective_gamma() == pytest.approx(1.0)
    for _ in range(4):
        g.step(lbm_dt=1.0e-3)
    assert g.effective_gamma() == pytest.approx(4.0)
    with pytest.raises(ValueError):
        g.step(lbm_dt=0.0)
    lbm = LBMSolver3D(periodic_lbm())
    mpm = MPMSolver3D(small_mpm(nx=9))
    with pytest.raises(ValueError):
        LBMMpmCoupler(CouplingConfig(), lbm, mpm)
    mpm = MPMSolver3D(small_mpm())
    mpm.initialize_particles_from_numpy(np.array([[4.0, 4.0, 4.0]], np.float32))
    with pytest.raises(RuntimeError):
        LBMMpmCoupler(CouplingConfig(), lbm, mpm).compute_coupling_forces()
    g, _ = pair(CouplingConfig(gamma=0.0, contact_enabled=True, contact_velocity_damping=0.25,
                               contact_fraction_threshold=0.01),
                velocity=(0.1, 0, 0), solid=SOLID_BLOCK)
    g.compute_coupling_forces(dt_ratio=1.0)
    assert np.linalg.norm(g.mpm.velocities_numpy()[0]) == pytest.approx(0.075)


@pytest.mark.parametrize("cfg", [
    CouplingConfig(gamma=0.01, mpm_substeps_per_lbm_step=2),
    CouplingConfig(enabled=False, gamma=0.05, mpm_substeps_per_lbm_step=2),
    CouplingConfig(gamma=50.0, force_limit=0.1, relative_velocity_limit=0.01, gamma_ramp_steps=3,
                   mpm_substeps_per_lbm_step=1),
    CouplingConfig(gamma=0.01, mpm_substeps_per_lbm_step=1, immersed_boundary_enabled=True,
                   immersed_boundary_drag=0.1, immersed_boundary_fraction_threshold=0.01,
                   immersed_boundary_max_force=1e-3, contact_enabled=True,
                   contact_velocity_damping=0.1, contact_fraction_threshold=0.01),
])
def test_coupled_steps_single_particle_match_oracle(cfg):
    g, o = pair(cfg, lbm_velocity=(1e-3, 0, 0), volume=2.0)
    for _ in range(3):
        g.step(lbm_dt=1.0e-3)
        o.step(lbm_dt=1.0e-3)
    assert rel_l2(g.mpm.positions_numpy(), o.mpm.positions_numpy()) < 1e-7
    assert rel_l2(g.lbm.velocity_numpy(), o.lbm.v) < 1e-5
    assert rel_l2(g.lbm.density_numpy(), o.lbm.rho) < 1e-7
    assert np.isfinite(g.lbm.velocity_numpy()).all()


def _smoke_pair(steps, *, p2g_mode="sorted"):
    """The 48x32x32 coupled smoke workload on the GPU and on the oracle. The sorted scatter
    is paired with the oracle summing in the same cell order; the atomic scatter (default)
    with the oracle's serial particle order."""
    cfg, solid, pos = coupled_smoke_config(steps=steps)
    cfg = dataclasses.replace(cfg, mpm=dataclasses.replace(cfg.mpm, p2g_mode=p2g_mode))
    sim = FSISimulation(cfg)
    sim.initialize_lbm(solid)
    sim.initialize_mpm_from_numpy(pos)
    ref = O.FSISimulation(cfg, nthreads=NTHREADS, polar="device",
                          cell_order=p2g_mode == "sorted")
    ref.initialize_lbm(solid)
    ref.initialize_mpm_from_numpy(pos)
    np.testing.assert_array_equal(sim.mpm.base_cells_numpy(),
                                  ((pos * np.float32(1.0)) - np.float32(0.5)).astype(np.int32))
    return cfg, sim, ref


def _assert_masks_and_counters(sim, ref):
    np.testing.assert_array_equal(sim.lbm.solid_numpy(), ref.lbm.solid)
    np.testing.assert_array_equal(sim.coupler.particle_coupling_mask_numpy(),
                                  ref.coupler.particle_coupling_mask_numpy())
    dg, do = sim.coupler.coupling_diagnostics(), ref.coupler.coupling_diagnostics()
    for key in ("unsupported_particle_count", "partial_support_particle_count",
                "clipped_particle_count"):
        assert dg[key] == do[key]


@pytest.mark.slow
def test_coupled_smoke_workload_100_steps():
    """48x32x32 tau=0.6 channel, one 8^3 elastic cube of 4096 particles, 10 substeps, 100
    coupled steps: density, velocity and positions within relative L2 1e-5 of the oracle."""
    cfg, sim, ref = _smoke_pair(100)
    for _ in range(100):
        sim.coupler.step(cfg.lbm_dt)
        ref.coupler.step(cfg.lbm_dt)
    errs = {
        "rho": rel_l2(sim.lbm.density_numpy(), ref.lbm.rho),
        "u": rel_l2(sim.lbm.velocity_numpy(), ref.lbm.v),
        "x": rel_l2(sim.mpm.positions_numpy(), ref.mpm.positions_numpy()),
        "v": rel_l2(sim.mpm.velocities_numpy(), ref.mpm.velocities_numpy()),
    }
    assert max(errs.values()) <= 1e-5, errs
    _assert_masks_and_counters(sim, ref)
    assert np.abs(ref.lbm.v).max() > 1e-4


def test_coupled_smoke_steps_bit_exact():
    """Ten coupled smoke steps are bit-identical to the oracle in the cell order: lattice
    populations, fluid fields, coupling accumulator and every particle field."""
    cfg, sim, ref = _smoke_pair(10)
    for k in range(10):
        sim.coupler.step(cfg.lbm_dt)
        ref.coupler.step(cfg.lbm_dt)
        np.testing.assert_array_equal(sim.lbm.distribution_numpy(), ref.lbm.distribution_numpy(),
                                      err_msg=f"step {k}")
    np.testing.assert_array_equal(sim.lbm.density_numpy(), ref.lbm.rho)
    np.testing.assert_array_equal(sim.lbm.velocity_numpy(), ref.lbm.v)
    np.testing.assert_array_equal(sim.coupler.coupling_force_numpy(),
                                  ref.coupler.coupling_force_numpy())
    np.testing.assert_array_equal(sim.coupler.solid_volume_fraction_numpy(),
                                  ref.coupler.solid_volume_fraction_numpy())
    np.testing.assert_array_equal(sim.mpm.positions_numpy(), ref.mpm.positions_numpy())
    np.testing.assert_array_equal(sim.mpm.velocities_numpy(), ref.mpm.velocities_numpy())
    np.testing.assert_array_equal(sim.mpm.deformation_gradients_numpy(),
                                  ref.mpm.deformation_gradients_numpy())
    np.testing.assert_array_equal(sim.mpm.particle_forces_numpy(),
                                  ref.mpm.particle_forces_numpy())
    _assert_masks_and_counters(sim, ref)


@pytest.mark.slow
def test_coupled_smoke_workload_atomic_scatter():
    """The atomic scatter (p2g_mode="atomic") against the oracle's serial particle order.
    Its grid and reaction sums arrive in scheduling order, and on this workload float32
    order differences alone move u by 2.06e-4 (relative L2) after 100 steps (two oracle runs
    differing only in P2G order); density and positions stay within 1e-5."""
    cfg, sim, ref = _smoke_pair(100, p2g_mode="atomic")
    for _ in range(100):
        sim.coupler.step(cfg.lbm_dt)
        ref.coupler.step(cfg.lbm_dt)
    assert rel_l2(sim.lbm.density_numpy(), ref.lbm.rho) <= 1e-5
    assert rel_l2(sim.mpm.positions_numpy(), ref.mpm.positions_numpy()) <= 1e-5
    assert rel_l2(sim.lbm.velocity_numpy(), ref.lbm.v) <= 2.5e-4
    _assert_masks_and_counters(sim, ref)


@pytest.fixture()
def gpu_cases():
    return vc


def test_validation_suite_on_gpu(gpu_cases):
    for r in gpu_cases.run_validation_suite():
        assert r.passed, r.to_dict()


def test_goldens_on_gpu():
    reports = rc.run_reference_validation_suite()
    assert len(reports) == 6
    for rep in reports:
        assert rep.passed, rep.to_dict()


def test_simulation_runner_bookkeeping(tmp_path):
    cfg = SimulationConfig(num_steps=3, lbm_dt=1e-3,
                           lbm=periodic_lbm(initial_velocity=(1e-5, 0, 0)), mpm=small_mpm(),
                           coupling=CouplingConfig(gamma=0.01, mpm_substeps_per_lbm_step=1))
    sim = FSISimulation(cfg)
    with pytest.raises(RuntimeError):
        sim.run(steps=1)
    with pytest.raises(ValueError):
        sim.initialize()
    sim.initialize(mpm_box_lower=(3.0, 3.0, 3.0), mpm_box_upper=(5.0, 5.0, 5.0), mpm_box_spacing=1.0)
    assert sim.lbm._initialized and sim.mpm._initialized and sim.mpm.particle_count() > 0
    d = sim.step()
    assert d["step"] == 1 and d["time"] == pytest.approx(1e-3)
    assert np.isfinite(d["lbm_total_mass"]) and np.isfinite(d["mpm_center_of_mass"]).all()
    hist = sim.run()
    assert len(hist) == 3 and sim.step_index == 4
    with pytest.raises(ValueError):
        sim.run(steps=0)
    fr = sim.coupler.solid_volume_fraction_numpy()
    assert fr.min() >= 0.0 and fr.max() <= 1.0


def test_runner_diagnostics_are_device_resident():
    """FSISimulation.step() returns the reference's 18 diagnostics from device reductions
    with a single host synchronisation and no tensor copied to the host by .cpu()/.item();
    the values agree with the per-accessor host path (float64 sums vs float32 numpy)."""
    import torch

    cfg, solid, pos = coupled_smoke_config(steps=5)
    cfg = dataclasses.replace(cfg, coupling=dataclasses.replace(
        cfg.coupling, immersed_boundary_enabled=True, immersed_boundary_drag=0.1,
        immersed_boundary_fraction_threshold=0.05, contact_enabled=True,
        contact_fraction_threshold=0.5, contact_velocity_damping=0.01))
    sim = FSISimulation(cfg)
    sim.initialize_lbm(solid)
    sim.initialize_mpm_from_numpy(pos)
    for _ in range(2):
        sim.step()
    counts = {"sync": 0, "cpu": 0, "item": 0}
    real_sync, real_cpu, real_item = torch.cuda.Stream.synchronize, torch.Tensor.cpu, torch.Tensor.item

    def sync(self, *a, **k):
        counts["sync"] += 1
        return real_sync(self, *a, **k)

    def cpu(self, *a, **k):
        counts["cpu"] += 1
        return real_cpu(self, *a, **k)

    def item(self, *a, **k):
        counts["item"] += 1
        return real_item(self, *a, **k)

    torch.cuda.Stream.synchronize, torch.Tensor.cpu, torch.Tensor.item = sync, cpu, item
    try:
        d = sim.step(body_force=(2.0e-5, 0.0, 0.0))
    finally:
        torch.cuda.Stream.synchronize, torch.Tensor.cpu, torch.Tensor.item = real_sync, real_cpu, real_item
    assert counts == {"sync": 1, "cpu": 0, "item": 0}, counts
    assert list(d) == [k for k in (
        "step", "time", "lbm_total_mass", "lbm_max_velocity_norm", "mpm_particle_count",
        "mpm_center_of_mass", "mpm_max_velocity_norm", "total_particle_coupling_force",
        "total_fluid_coupling_force", "coupling_unsupported_particle_count",
        "coupling_partial_support_particle_count", "coupling_clipped_particle_count",
        "coupling_effective_gamma", "coupling_ib_active_cell_count",
        "coupling_ib_clipped_cell_count", "coupling_ib_total_force_norm",
        "coupling_contact_candidate_count", "coupling_contact_damped_particle_count")]
    cd = sim.coupler.coupling_diagnostics()
    assert d["lbm_total_mass"] == pytest.approx(sim.lbm.total_mass(), rel=1e-12)
    assert d["lbm_max_velocity_norm"] == pytest.approx(sim.lbm.max_velocity_norm(), rel=1e-12)
    np.testing.assert_allclose(d["mpm_center_of_mass"], sim.mpm.center_of_mass(), rtol=1e-6)
    assert d["mpm_max_velocity_norm"] == pytest.approx(sim.mpm.max_velocity_norm(), rel=1e-6)
    np.testing.assert_allclose(d["total_particle_coupling_force"],
                               sim.coupler.total_particle_coupling_force(), rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(d["total_fluid_coupling_force"],
                               sim.coupler.total_fluid_coupling_force(), rtol=1e-5, atol=1e-12)
    for key in ("unsupported_particle_count", "partial_support_particle_count",
                "clipped_particle_count", "ib_active_cell_count", "ib_clipped_cell_count",
                "contact_candidate_count", "contact_damped_particle_count"):
        assert d["coupling_" + key] == cd[key], key
    assert d["coupling_ib_total_force_norm"] == pytest.approx(cd["ib_total_force_norm"], rel=1e-6)
    assert d["coupling_ib_active_cell_count"] > 0 and d["coupling_contact_candidate_count"] > 0
    assert sim._diag_fused  # the fluid reaction came from the step's force assembly


@pytest.mark.parametrize("ib", [False, True])
def test_assembly_with_reaction_sum_is_the_plain_assembly(ib):
    """fsi_coupling_assemble_sum writes the force field (and IB field and counters) of
    fsi_coupling_assemble bit for bit, and its fluid-reaction sum is total_fluid_coupling_force
    of the accumulator it read. The sorted scatter makes the two runs' states comparable bit
    for bit."""
    import torch

    cfg, solid, pos = coupled_smoke_config(steps=5)
    cfg = dataclasses.replace(cfg, mpm=dataclasses.replace(cfg.mpm, p2g_mode="sorted"))
    if ib:
        cfg = dataclasses.replace(cfg, coupling=dataclasses.replace(
            cfg.coupling, immersed_boundary_enabled=True, immersed_boundary_drag=0.1,
            immersed_boundary_fraction_threshold=0.05))
    sims = []
    for fused in (False, True):
        sim = FSISimulation(cfg)
        sim.initialize_lbm(solid)
        sim.initialize_mpm_from_numpy(pos)
        if fused:
            sim.coupler._reaction_out = torch.zeros(3, dtype=torch.float64, device="cuda")
        sims.append(sim)
    plain, fused = sims
    for _ in range(4):
        for sim in sims:
            sim.coupler.step(cfg.lbm_dt)
        assert fused.coupler._reaction_fresh and not plain.coupler._reaction_fresh
        np.testing.assert_allclose(fused.coupler._reaction_out.cpu().numpy(),
                                   fused.coupler.total_fluid_coupling_force(),
                                   rtol=1e-5, atol=1e-12)
    np.testing.assert_array_equal(fused.lbm.distribution_numpy(), plain.lbm.distribution_numpy())
    np.testing.assert_array_equal(fused.coupler.immersed_boundary_force_numpy(),
                                  plain.coupler.immersed_boundary_force_numpy())
    df, dp = fused.coupler.immersed_boundary_diagnostics(), plain.coupler.immersed_boundary_diagnostics()
    assert df.keys() == dp.keys()
    for key in df:  # the IB force totals are float atomic sums, the counts exact
        assert df[key] == pytest.approx(dp[key], rel=1e-5, abs=1e-12), key
    if ib:
        assert df["ib_active_cell_count"] > 0


def test_body_force_per_step_matches_config_force():
    """step(body_force=g) with g equal to LBMConfig.force repeats the plain step bit for bit."""
    cfg, solid, pos = coupled_smoke_config(steps=3)
    sims = []
    for bf in (None, cfg.lbm.force):
        sim = FSISimulation(cfg)
        sim.initialize_lbm(solid)
        sim.initialize_mpm_from_numpy(pos)
        for _ in range(3):
            sim.step(body_force=bf)
        sims.append(sim)
    np.testing.assert_array_equal(sims[0].lbm.distribution_numpy(), sims[1].lbm.distribution_numpy())
    np.testing.assert_array_equal(sims[0].mpm.positions_numpy(), sims[1].mpm.positions_numpy())
    with pytest.raises(ValueError):
        sims[0].step(body_force=(1.0, 2.0))


def test_coupled_large_launch_matches_oracle():
    """A coupled step with enough particles (85,184) for the coupling's own shared-memory
    kernel on the tiled scatter: lattice and particle fields within relative L2 1e-5 of the
    oracle after two steps, coupling masks and counters exact, the coupling force within the
    atomic scatter's float32 noise."""
    from fsi import scenes

    nx, ny, nz = 48, 40, 40
    lbm = periodic_lbm(nx=nx, ny=ny, nz=nz, viscosity=(0.6 - 0.5) / 3.0, force=(1e-5, 0.0, 0.0))
    mpm = small_mpm(nx=nx, ny=ny, nz=nz, max_particles=90_000, dt=0.25, density=1.5,
                    youngs_modulus=0.05, poisson_ratio=0.3, boundary_width=3)
    cfg = SimulationConfig(num_steps=2, lbm_dt=1.0, lbm=lbm, mpm=mpm,
                           coupling=CouplingConfig(gamma=0.1, mpm_substeps_per_lbm_step=4))
    solid = scenes.wall_mask(nx, ny, nz)
    pos = scenes.cube_particles(np.array([10.0, 9.0, 9.0]), 22, 2, np.random.default_rng(5))
    assert len(pos) == 85_184
    sim = FSISimulation(cfg)
    ref = O.FSISimulation(cfg, nthreads=NTHREADS, polar="device")
    for s in (sim, ref):
        s.initialize_lbm(solid)
        s.initialize_mpm_from_numpy(pos)
    for _ in range(2):
        sim.coupler.step(cfg.lbm_dt)
        ref.coupler.step(cfg.lbm_dt)
    assert rel_l2(sim.lbm.density_numpy(), ref.lbm.rho) <= 1e-5
    assert rel_l2(sim.lbm.velocity_numpy(), ref.lbm.v) <= 1e-5
    assert rel_l2(sim.mpm.positions_numpy(), ref.mpm.positions_numpy()) <= 1e-5
    assert rel_l2(sim.mpm.particle_forces_numpy(), ref.mpm.particle_forces_numpy()) <= 1e-4
    assert rel_l2(sim.coupler.coupling_force_numpy(), ref.coupler.coupling_force_numpy()) <= 1e-4
    _assert_masks_and_counters(sim, ref)
