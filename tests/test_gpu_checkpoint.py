"""Checkpoint / restart of the solvers and the runner (absent in the reference, which only
writes snapshots): a restored run continues exactly as the uninterrupted one."""
from __future__ import annotations

import numpy as np
import pytest

from fsi.config import CouplingConfig, SimulationConfig
from fsi.lbm3d import LBMSolver3D
from fsi.simulation import FSISimulation
from helpers import channel_mask, periodic_lbm, rel_l2, small_mpm

pytestmark = pytest.mark.gpu


def test_lattice_restart_is_bit_exact():
    cfg = periodic_lbm(nx=12, ny=10, nz=9, force=(1e-5, 0.0, 2e-6))
    solid = channel_mask(12, 10, 9)
    a = LBMSolver3D(cfg)
    a.initialize(solid)
    for _ in range(5):
        a.step()
    state = a.state_dict()
    for _ in range(7):
        a.step()
    b = LBMSolver3D(cfg)
    b.load_state_dict(state)
    for _ in range(7):
        b.step()
    np.testing.assert_array_equal(a.distribution_numpy(), b.distribution_numpy())
    np.testing.assert_array_equal(a.velocity_numpy(), b.velocity_numpy())


def test_coupled_restart_from_file(tmp_path):
    cfg = SimulationConfig(
        num_steps=3, lbm_dt=1.0,
        lbm=periodic_lbm(nx=12, ny=10, nz=10, viscosity=1 / 30, force=(1e-5, 0.0, 0.0)),
        mpm=small_mpm(nx=12, ny=10, nz=10, max_particles=64, dt=0.1, density=1.5,
                      youngs_modulus=0.05, poisson_ratio=0.3),
        coupling=CouplingConfig(gamma=0.1, mpm_substeps_per_lbm_step=4, gamma_ramp_steps=5))
    pos = (4.0 + 2.0 * np.random.default_rng(1).uniform(0, 1, (64, 3))).astype(np.float32)
    a = FSISimulation(cfg)
    a.initialize_lbm(channel_mask(12, 10, 10))
    a.initialize_mpm_from_numpy(pos)
    a.run(steps=3)
    path = tmp_path / "ckpt.pt"
    a.save_checkpoint(path)
    a.run(steps=3)
    b = FSISimulation(cfg)
    b.load_checkpoint(path)
    assert b.step_index == 3 and b.coupler.coupled_step == 3
    b.run(steps=3)
    assert b.step_index == a.step_index and b.time == a.time
    assert b.coupler.effective_gamma() == a.coupler.effective_gamma()
    assert rel_l2(b.mpm.positions_numpy(), a.mpm.positions_numpy()) < 1e-6
    assert rel_l2(b.lbm.density_numpy(), a.lbm.density_numpy()) < 1e-6
    assert rel_l2(b.lbm.velocity_numpy(), a.lbm.velocity_numpy()) < 1e-3
