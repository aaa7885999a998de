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


def coupled_smoke_config(steps: int = 100) -> tuple[SimulationConfig, np.ndarray, np.ndarray]:
    """The 48x32x32 coupled smoke workload: MRT tau 0.6 channel with walls in y and z,
    g_x = 1e-5, one 8^3-cell elastic cube (E 0.05, nu 0.3, rho_s 1.5) centred at 16,
    2x2x2 particles per cell jittered in their sub-cells from seed 0, gamma 0.1,
    10 substeps, gravity off."""
    nx, ny, nz = 48, 32, 32
    lbm = LBMConfig(nx=nx, ny=ny, nz=nz, viscosity=(0.6 - 0.5) / 3.0, rho0=1.0,
                    force=(1.0e-5, 0.0, 0.0), **PERIODIC)
    mpm = MPMConfig(nx=nx, ny=ny, nz=nz, max_particles=4096, particles_per_cell=2, dx=1.0,
                    dt=0.1, density=1.5, youngs_modulus=0.05, poisson_ratio=0.3,
                    gravity=(0.0, 0.0, 0.0), boundary_width=3)
    cfg = SimulationConfig(num_steps=steps, lbm_dt=1.0, lbm=lbm, mpm=mpm,
                           coupling=CouplingConfig(gamma=0.1, mpm_substeps_per_lbm_step=10))
    rng = np.random.default_rng(0)
    idx = np.stack(np.meshgrid(np.arange(16), np.arange(16), np.arange(16), indexing="ij"),
                   axis=-1).reshape(-1, 3)
    pos = (12.0 + 0.5 * (idx + rng.uniform(0.0, 1.0, idx.shape))).astype(np.float32)
    return cfg, channel_mask(nx, ny, nz), pos


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))
