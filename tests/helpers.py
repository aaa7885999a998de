"""Shared builders for the parity tests (configs of the reference's own tests and workloads)."""
from __future__ import annotations

import numpy as np

from fsi.config import BoundaryConfig, CouplingConfig, LBMConfig, MPMConfig, SimulationConfig

PERIODIC = {n: BoundaryConfig("periodic")
            for n in ("x_left", "x_right", "y_left", "y_right", "z_left", "z_right")}


def periodic_lbm(**kw) -> LBMConfig:
    params = dict(nx=8, ny=8, nz=8, viscosity=0.1, rho0=1.0, force=(0.0, 0.0, 0.0),
                  initial_velocity=(0.0, 0.0, 0.0), **PERIODIC)
    params.update(kw)
    return LBMConfig(**params)


def small_mpm(**kw) -> MPMConfig:
    params = dict(nx=8, ny=8, nz=8, max_particles=128, dx=1.0, dt=1.0e-3, density=1.0,
                  youngs_modulus=100.0, poisson_ratio=0.25, gravity=(0.0, 0.0, 0.0),
                  boundary_width=1)
    params.update(kw)
    return MPMConfig(**params)


def channel_mask(nx: int, ny: int, nz: int) -> np.ndarray:
    """Solid wall planes at y = 0, ny-1 and z = 0, nz-1 (walls expressed as mask planes)."""
    s = np.zeros((nx, ny, nz), np.int32)
    s[:, 0, :] = s[:, -1, :] = 1
    s[:, :, 0] = s[:, :, -1] = 1
    return s


def coupled_smoke_config(steps: int = 100):
    """The 48x32x32 coupled smoke workload (fsi.scenes.coupled_smoke)."""
    from fsi import scenes
    return scenes.coupled_smoke(steps)


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))
