"""Parity on reduced versions of the configurations at scale, built by the same seeded scene
generators (fsi.scenes) as the benchmark.

  standalone kernels: a 64^3 channel with static spheres (~10 % solid) and walls, 100 lattice
  steps, bit-identical to the oracle; four elastic cubes of 8^3 cells (8 particles per cell)
  in a 64^3 grid under gravity, 100 substeps: the sorted scatter bit-identical to the oracle's
  cell order, the atomic scatter within float32 order noise of the serial oracle;
  coupled at scale: a 96x48x48 channel with a velocity inlet (0.05) and a pressure outlet,
  walls in y and z, two cubes and two balls with per-body Young's modulus, 10 substeps per
  step, 100 coupled steps with the sorted scatter: lattice, fluid fields, coupling fields,
  particles, masks and counters bit-identical to the oracle's cell order.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np
import pytest

from fsi import scenes
from fsi.lbm3d import LBMSolver3D
from fsi.mpm3d import MPMSolver3D
from fsi.simulation import FSISimulation
from helpers import rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu
NTHREADS = os.cpu_count() or 1


def test_standalone_lattice_spheres_channel_100_steps():
    cfg, mask = scenes.channel_spheres_lbm(n=64)
    assert 0.1 <= mask.mean() <= 0.4
    g, o = LBMSolver3D(cfg), O.LBMSolver3D(cfg, nthreads=NTHREADS)
    g.initialize(mask)
    o.initialize(mask)
    for _ in range(100):
        g.step()
        o.step()
    np.testing.assert_array_equal(g.solid_numpy(), o.solid)
    np.testing.assert_array_equal(g.distribution_numpy(), o.distribution_numpy())
    np.testing.assert_array_equal(g.density_numpy(), o.rho)
    np.testing.assert_array_equal(g.velocity_numpy(), o.v)
    assert np.abs(o.v).max() > 1e-6


@pytest.mark.parametrize("mode", ["sorted", "atomic"])
def test_standalone_cubes_100_substeps(mode):
    mcfg, pos = scenes.cubes_mpm(n=64, cubes=4, edge=8)
    mcfg = dataclasses.replace(mcfg, p2g_mode=mode)
    g = MPMSolver3D(mcfg)
    o = O.MPMSolver3D(mcfg, polar="device", cell_order=mode == "sorted")
    for s in (g, o):
        s.initialize_particles_from_numpy(pos)
    for _ in range(100):
        g.substep()
        o.substep()
    np.testing.assert_array_equal(g.base_cells_numpy(),
                                  (o.positions_numpy() - np.float32(0.5)).astype(np.int32))
    if mode == "sorted":
        np.testing.assert_array_equal(g.positions_numpy(), o.positions_numpy())
        np.testing.assert_array_equal(g.velocities_numpy(), o.velocities_numpy())
        np.testing.assert_array_equal(g.deformation_gradients_numpy(), o.deformation_gradients_numpy())
    else:
        assert rel_l2(g.positions_numpy(), o.positions_numpy()) <= 1e-6
        assert rel_l2(g.velocities_numpy(), o.velocities_numpy()) <= 1e-3
        assert rel_l2(g.deformation_gradients_numpy(), o.deformation_gradients_numpy()) <= 1e-5
    assert o.velocities_numpy()[:, 1].mean() < -1e-4  # the cubes fall


@pytest.mark.slow
def test_coupled_bodies_channel_100_steps():
    cfg, solid, pos, young = scenes.coupled_bodies(nx=96, ny=48, nz=48, bodies=4, cube_edge=8,
                                                   sphere_radius=4.0)
    cfg = dataclasses.replace(cfg, mpm=dataclasses.replace(cfg.mpm, p2g_mode="sorted"))
    sim = FSISimulation(cfg)
    ref = O.FSISimulation(cfg, nthreads=NTHREADS, polar="device", cell_order=True)
    for s in (sim, ref):
        s.initialize_lbm(solid)
        s.initialize_mpm_from_numpy(pos, youngs_modulus=young, poisson_ratio=0.3)
    assert len(np.unique(young)) == 4
    for k in range(100):
        sim.coupler.step(cfg.lbm_dt)
        ref.coupler.step(cfg.lbm_dt)
        if k % 25 == 24:
            np.testing.assert_array_equal(sim.lbm.distribution_numpy(),
                                          ref.lbm.distribution_numpy(), err_msg=f"step {k}")
    np.testing.assert_array_equal(sim.lbm.solid_numpy(), ref.lbm.solid)
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
    np.testing.assert_array_equal(sim.coupler.particle_coupling_mask_numpy(),
                                  ref.coupler.particle_coupling_mask_numpy())
    dg, do = sim.coupler.coupling_diagnostics(), ref.coupler.coupling_diagnostics()
    for key in ("unsupported_particle_count", "partial_support_particle_count",
                "clipped_particle_count"):
        assert dg[key] == do[key], key
    # the inlet drives the channel and the bodies move
    assert np.abs(ref.lbm.v).max() > 1e-2
    assert np.abs(ref.mpm.positions_numpy() - pos).max() > 1e-4
