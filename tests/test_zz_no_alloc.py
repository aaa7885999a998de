"""The MPM substep entry point for callers that cannot allocate device memory.

Some hosts of this library may not call cudaMalloc (a real-time loop that cannot
take an allocation's device synchronisation, a plugin inside an application that
owns the device memory pool, a plain FFI caller without a device allocator).
``fsi_mpm_substep_noalloc`` serves them with the grid held in the library's static
device array. This test calls it through the C ABI on the same particles as the
allocating entry point ``fsi_mpm_substep`` and checks that two substeps in a row
agree within the tolerance of the other MPM parity tests (the grid sums are
accumulated by atomics, so the order and the last bits may differ). It lives in a
file of its own, collected last, and runs alone or after the other tests.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _solvers():
    from fsi.config import MPMConfig
    from fsi.mpm3d import MPMSolver3D

    cfg = MPMConfig(nx=24, ny=20, nz=16, max_particles=4096, dt=1.0e-2, youngs_modulus=400.0,
                    gravity=(0.0, -1.0e-3, 0.0), boundary_width=2)
    rng = np.random.default_rng(21)
    pos = np.stack(np.meshgrid(np.arange(6.0, 12.0, 0.5), np.arange(5.0, 9.0, 0.5),
                               np.arange(4.0, 8.0, 0.5), indexing="ij"), -1).reshape(-1, 3)
    pos = (pos + rng.uniform(0.0, 0.25, pos.shape)).astype(np.float32)
    vel = rng.normal(0.0, 1.0e-2, pos.shape).astype(np.float32)
    out = []
    for _ in range(2):
        s = MPMSolver3D(cfg)
        s.initialize_particles_from_numpy(pos, vel, particle_volume=0.125)
        out.append(s)
    return out


def test_noalloc_substep_matches_allocating_substep_twice():
    from fsi import _native as nat

    with_grid, without_grid = _solvers()
    for call in range(2):
        with_grid.substep()
        nat.call("fsi_mpm_substep_noalloc", without_grid.desc, without_grid.particles,
                 nat.stream_ptr())
        assert _rel_l2(without_grid.positions_numpy(), with_grid.positions_numpy()) < 1e-6, call
        assert _rel_l2(without_grid.velocities_numpy(), with_grid.velocities_numpy()) < 1e-4, call
        assert _rel_l2(without_grid.deformation_gradients_numpy(),
                       with_grid.deformation_gradients_numpy()) < 1e-5, call
        assert np.isfinite(without_grid.velocities_numpy()).all()


def test_noalloc_substep_rejects_grids_above_its_limit():
    from fsi import _native as nat
    from fsi.config import MPMConfig
    from fsi.mpm3d import MPMSolver3D

    big = MPMSolver3D(MPMConfig(nx=80, ny=64, nz=64, max_particles=8))
    big.initialize_particles_from_numpy(np.full((8, 3), 10.0, np.float32))
    with pytest.raises(ValueError, match="at most"):
        nat.call("fsi_mpm_substep_noalloc", big.desc, big.particles, nat.stream_ptr())


def _pair(nx, ny, nz, lo, hi, seed):
    """Two solvers on the same particles (a jittered sub-cell lattice in [lo, hi))."""
    from fsi.config import MPMConfig
    from fsi.mpm3d import MPMSolver3D

    cfg = MPMConfig(nx=nx, ny=ny, nz=nz, max_particles=20_000, dt=1.0e-2, youngs_modulus=400.0,
                    gravity=(0.0, -1.0e-3, 0.0), boundary_width=2)
    rng = np.random.default_rng(seed)
    axes = [np.arange(a, b, 0.5) for a, b in zip(lo, hi)]
    pos = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    pos = (pos + rng.uniform(0.0, 0.25, pos.shape)).astype(np.float32)
    vel = rng.normal(0.0, 1.0e-2, pos.shape).astype(np.float32)
    out = []
    for _ in range(2):
        s = MPMSolver3D(cfg)
        s.initialize_particles_from_numpy(pos, vel, particle_volume=0.125)
        out.append(s)
    return out


def _check_same(without_grid, with_grid, what):
    assert _rel_l2(without_grid.positions_numpy(), with_grid.positions_numpy()) < 1e-6, what
    assert _rel_l2(without_grid.velocities_numpy(), with_grid.velocities_numpy()) < 1e-4, what
    assert _rel_l2(without_grid.deformation_gradients_numpy(),
                   with_grid.deformation_gradients_numpy()) < 1e-5, what


def test_noalloc_grids_of_different_shape_one_after_another():
    """A large grid, then a smaller one of another shape, then the large one again: each call
    clears the part of the shared array it uses, so no call sees what the last one left."""
    from fsi import _native as nat

    big = _pair(48, 40, 36, (10.0, 8.0, 6.0), (30.0, 20.0, 16.0), 31)
    small = _pair(20, 30, 12, (4.0, 6.0, 3.0), (12.0, 16.0, 8.0), 32)
    for what, (with_grid, without_grid) in (("big", big), ("small", small), ("big again", big)):
        with_grid.substep()
        nat.call("fsi_mpm_substep_noalloc", without_grid.desc, without_grid.particles,
                 nat.stream_ptr())
        _check_same(without_grid, with_grid, what)


def test_noalloc_accepts_a_grid_at_its_limit():
    """64 x 64 x 64 nodes, the array's full capacity, is accepted and agrees."""
    from fsi import _native as nat

    with_grid, without_grid = _pair(64, 64, 64, (50.0, 52.0, 48.0), (60.0, 61.0, 61.0), 33)
    for call in range(2):
        with_grid.substep()
        nat.call("fsi_mpm_substep_noalloc", without_grid.desc, without_grid.particles,
                 nat.stream_ptr())
        _check_same(without_grid, with_grid, call)
