"""GPU lattice Boltzmann vs the CPU oracle: bit-exact on identical inputs.

The device kernel evaluates the reference's float32 operations in the same
order as the oracle (no contraction, generated MRT formulas), so populations,
density and velocity must agree to the last bit after any number of steps,
including the AA-pattern's odd/even storage, bounce-back, x-face conditions and
force changes between steps.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from fsi.config import BoundaryConfig, LBMConfig
from fsi.lbm3d import LBMSolver3D
from helpers import PERIODIC, channel_mask, periodic_lbm, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu
NTHREADS = os.cpu_count() or 1


def assert_same_state(gpu: LBMSolver3D, ref: O.LBMSolver3D, tag: str = "") -> None:
    f = gpu.distribution_numpy()
    np.testing.assert_array_equal(f, ref.f, err_msg=f"distribution {tag}")
    np.testing.assert_array_equal(gpu.density_numpy(), ref.rho, err_msg=f"rho {tag}")
    np.testing.assert_array_equal(gpu.velocity_numpy(), ref.v, err_msg=f"u {tag}")


def run_pair(cfg: LBMConfig, steps: int, solid=None, check_every: int | None = None):
    gpu, ref = LBMSolver3D(cfg), O.LBMSolver3D(cfg, nthreads=NTHREADS)
    gpu.initialize(solid)
    ref.initialize(solid)
    assert_same_state(gpu, ref, "init")
    for s in range(steps):
        gpu.step()
        ref.step()
        if check_every and (s + 1) % check_every == 0:
            assert_same_state(gpu, ref, f"step {s + 1}")
    assert_same_state(gpu, ref, f"step {steps}")
    return gpu, ref


def test_periodic_rest_20_steps():
    run_pair(periodic_lbm(), 20)


def test_periodic_forced_every_step_parity():
    # Checking after every step alternates the AA even/odd layouts of the accessor.
    run_pair(periodic_lbm(force=(1.0e-6, 2.0e-7, -3.0e-7)), 9, check_every=1)


def test_channel_with_obstacle_100_steps():
    """48x32x32 tau=0.6 channel: walls in y and z as mask planes, a static 8^3 block, g_x=1e-5."""
    cfg = LBMConfig(nx=48, ny=32, nz=32, viscosity=(0.6 - 0.5) / 3.0, force=(1.0e-5, 0.0, 0.0),
                    **PERIODIC)
    solid = channel_mask(48, 32, 32)
    solid[12:20, 12:20, 12:20] = 1
    gpu, ref = run_pair(cfg, 100, solid=solid)
    assert rel_l2(gpu.velocity_numpy(), ref.v) == 0.0
    assert np.abs(ref.v).max() > 1e-4  # the flow actually developed
    np.testing.assert_array_equal(gpu.velocity_numpy()[solid == 1], 0.0)


@pytest.mark.parametrize("left,right", [
    (BoundaryConfig("velocity", velocity=(0.02, 0.0, 0.0)), BoundaryConfig("pressure", rho=1.0)),
    (BoundaryConfig("pressure", rho=1.01), BoundaryConfig("pressure", rho=1.0)),
    (BoundaryConfig("periodic"), BoundaryConfig("velocity", velocity=(-0.01, 0.005, 0.0))),
    (BoundaryConfig("velocity", velocity=(0.02, 0.003, 0.0), velocity_update="simultaneous"),
     BoundaryConfig("pressure", rho=1.0)),
])
def test_x_face_conditions(left, right):
    faces = dict(PERIODIC, x_left=left, x_right=right)
    cfg = LBMConfig(nx=16, ny=8, nz=8, viscosity=0.05, **faces)
    solid = channel_mask(16, 8, 8)
    solid[0, 3, 3] = 1          # a solid face cell
    solid[1, 4, 4] = 1          # a solid inner neighbour of a face cell
    solid[14, 4, 3] = 1
    run_pair(cfg, 31, solid=solid, check_every=10)


def test_force_changes_between_steps_use_the_previous_force():
    """Changing the force after a step must not alter the macroscopic state the next
    collision sees (the reference stores u with the previous step's force)."""
    cfg = periodic_lbm(force=(1.0e-6, 0.0, 0.0))
    solid = np.zeros((8, 8, 8), np.int32)
    solid[3:5, 3:5, 3:5] = 1
    gpu, ref = LBMSolver3D(cfg), O.LBMSolver3D(cfg)
    gpu.initialize(solid)
    ref.initialize(solid)
    rng = np.random.default_rng(5)
    for s in range(12):
        if s % 3 == 1:
            local = rng.normal(0, 1e-6, (8, 8, 8, 3)).astype(np.float32)
            gpu.set_force_from_numpy(local)
            ref.set_force_from_numpy(local)
        elif s % 3 == 2:
            gpu.add_uniform_force((1e-7, 0.0, -2e-7))
            ref.add_uniform_force((1e-7, 0.0, -2e-7))
        if s == 6:
            gpu.reset_force()
            ref.reset_force()
            assert gpu.total_mass() > 0  # forces a macro refresh mid-run
        gpu.step()
        ref.step()
        np.testing.assert_array_equal(gpu.force_numpy(), ref.force)
    assert_same_state(gpu, ref)


def test_force_api_semantics():
    cfg = periodic_lbm(force=(1.0e-6, 2.0e-6, -3.0e-6))
    solid = np.zeros((8, 8, 8), np.int32)
    solid[3:5, 3:5, 3:5] = 1
    s = LBMSolver3D(cfg)
    s.initialize(solid)
    f = s.force_numpy()
    assert f.shape == (8, 8, 8, 3)
    np.testing.assert_array_equal(f[solid == 1], 0.0)
    np.testing.assert_allclose(s.total_force(), np.array([504e-6, 1008e-6, -1512e-6]), rtol=1e-5)
    s.clear_force()
    np.testing.assert_array_equal(s.force_numpy(), 0.0)
    s.set_uniform_force((1e-6, 2e-6, 0.0))
    s.add_uniform_force((3e-6, -1e-6, 4e-6))
    f = s.force_numpy()
    np.testing.assert_allclose(f[solid == 0][:, 0], 4e-6, rtol=1e-6)
    np.testing.assert_allclose(f[solid == 0][:, 1], 1e-6, rtol=1e-6)
    np.testing.assert_array_equal(f[solid == 1], 0.0)
    with pytest.raises(ValueError):
        s.set_uniform_force((1e-6, 0.0))
    with pytest.raises(ValueError):
        s.set_force_from_numpy(np.zeros((8, 8, 8), np.float32))


def test_reference_lbm_behaviour():
    """The reference's tests/test_lbm3d.py assertions on the GPU solver."""
    s = LBMSolver3D(periodic_lbm())
    with pytest.raises(RuntimeError):
        s.step()
    with pytest.raises(ValueError):
        s.initialize(np.zeros((8, 8, 7), np.int32))
    with pytest.raises(NotImplementedError):
        LBMSolver3D(periodic_lbm(use_sparse=True))
    with pytest.raises(NotImplementedError):
        LBMSolver3D(periodic_lbm(y_left=BoundaryConfig("pressure")))
    s.initialize()
    m0 = s.total_mass()
    for _ in range(20):
        s.step()
    assert s.total_mass() == pytest.approx(m0, rel=1e-5, abs=1e-5)
    assert np.isfinite(s.density_numpy()).all() and s.density_numpy().shape == (8, 8, 8)
    local = LBMSolver3D(periodic_lbm())
    local.initialize()
    lf = np.zeros((8, 8, 8, 3), np.float32)
    lf[2:6, :, :, 0] = 1e-6
    local.set_force_from_numpy(lf)
    np.testing.assert_allclose(local.total_force(), [256e-6, 0, 0], rtol=1e-5, atol=1e-9)
    local.step()
    v = local.velocity_numpy()
    assert v[2:6, :, :, 0].mean() > np.concatenate([v[0:2, ..., 0].ravel(), v[6:8, ..., 0].ravel()]).mean()


def test_load_solid_from_txt(tmp_path):
    mask = np.zeros((6, 5, 7), np.int32)
    mask[1:3, 2, 4:6] = 1
    path = tmp_path / "solid.txt"
    np.savetxt(path, mask.reshape(-1, order="F"))
    np.testing.assert_array_equal(LBMSolver3D.load_solid_from_txt(path, 6, 5, 7), mask)
