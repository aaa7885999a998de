"""Seeded scene generators: wall masks, sphere packings and particle cubes.

These build the occupancy masks and particle sets of the benchmark workloads
(the reference has no generators; its masks come from callers or
``LBMSolver3D.load_solid_from_txt``). Masks use the reference's convention: int32
0/1 of shape (nx, ny, nz) in C order; walls in y and z are expressed as solid
mask planes because the reference supports only periodic y/z faces
(fsi/lbm3d.py:98-108).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .config import BoundaryConfig, CouplingConfig, LBMConfig, MPMConfig, SimulationConfig

PERIODIC_FACES = {name: BoundaryConfig("periodic")
                  for name in ("x_left", "x_right", "y_left", "y_right", "z_left", "z_right")}


def viscosity_for_tau(tau: float) -> float:
    """nu = (tau - 1/2) / 3, the inverse of tau = 3 nu + 1/2 (fsi/lbm3d.py:141)."""
    return (tau - 0.5) / 3.0


def wall_mask(nx: int, ny: int, nz: int) -> np.ndarray:
    """Solid planes at y = 0, ny-1 and z = 0, nz-1."""
    s = np.zeros((nx, ny, nz), np.int32)
    s[:, 0, :] = s[:, -1, :] = 1
    s[:, :, 0] = s[:, :, -1] = 1
    return s


def add_sphere(mask: np.ndarray, center, radius: float) -> int:
    """Mark the cells whose centres lie within ``radius`` of ``center`` (cell units);
    returns the number of cells that became solid."""
    lo = [max(int(np.floor(c - radius)), 0) for c in center]
    hi = [min(int(np.ceil(c + radius)) + 1, n) for c, n in zip(center, mask.shape)]
    ii, jj, kk = np.meshgrid(*[np.arange(a, b) for a, b in zip(lo, hi)], indexing="ij")
    inside = ((ii - center[0]) ** 2 + (jj - center[1]) ** 2 + (kk - center[2]) ** 2) <= radius ** 2
    box = mask[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
    added = int(np.count_nonzero(inside & (box == 0)))
    box[inside] = 1
    return added


def sphere_packing(shape, fraction: float, rmin: float, rmax: float, seed: int,
                   margin: int = 1, max_tries: int = 200_000):
    """Non-overlapping spheres with radii U[rmin, rmax] and centres uniform in the interior,
    added by rejection sampling until they fill ``fraction`` of the volume.
    Returns (mask, centres, radii)."""
    rng = np.random.default_rng(seed)
    mask = np.zeros(shape, np.int32)
    centres, radii = [], []
    total = float(np.prod(shape))
    filled = 0
    tries = 0
    while filled < fraction * total and tries < max_tries:
        tries += 1
        r = float(rng.uniform(rmin, rmax))
        c = np.array([rng.uniform(margin + r, n - 1 - margin - r) for n in shape])
        if centres:
            d = np.linalg.norm(np.asarray(centres) - c, axis=1)
            if np.any(d < np.asarray(radii) + r):
                continue
        added = add_sphere(mask, c, r)
        if added == 0:
            continue
        filled += added
        centres.append(c)
        radii.append(r)
    return mask, np.asarray(centres), np.asarray(radii)


def cube_particles(lower_cells, edge_cells: int, ppc_axis: int, rng=None) -> np.ndarray:
    """Particles of a cube of edge ``edge_cells`` cells with lower corner ``lower_cells``:
    ``ppc_axis``^3 per cell on the sub-cell lattice, each jittered uniformly within its
    sub-cell when ``rng`` is given. Ordered cell by cell (C order), then sub-cell."""
    n = edge_cells * ppc_axis
    idx = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"),
                   axis=-1).reshape(-1, 3)
    cell = idx // ppc_axis
    sub = idx % ppc_axis
    order = np.lexsort((sub[:, 2], sub[:, 1], sub[:, 0], cell[:, 2], cell[:, 1], cell[:, 0]))
    idx = idx[order]
    jitter = rng.uniform(0.0, 1.0, idx.shape) if rng is not None else 0.5
    return (np.asarray(lower_cells, np.float64) + (idx + jitter) / ppc_axis).astype(np.float32)


def random_cubes(grid: int, count: int, edge: int, seed: int, margin: int = 4,
                 ppc_axis: int = 2) -> np.ndarray:
    """``count`` non-overlapping cubes of ``edge`` cells at random positions in a ``grid``^3
    domain (rejection sampling from ``seed``); returns their particles."""
    rng = np.random.default_rng(seed)
    corners = []
    tries = 0
    while len(corners) < count:
        tries += 1
        if tries > 1_000_000:
            raise RuntimeError("could not place the cubes without overlap")
        c = rng.integers(margin, grid - margin - edge, size=3)
        if any(np.all(np.abs(c - o) < edge + 1) for o in corners):
            continue
        corners.append(c)
    return np.concatenate([cube_particles(c, edge, ppc_axis, rng) for c in corners])


@dataclass
class Workload:
    name: str
    lbm: LBMConfig
    mpm: MPMConfig
    solid: np.ndarray
    particles: np.ndarray


def channel_spheres_lbm(n: int = 256, tau: float = 0.6, gx: float = 1.0e-6, seed: int = 1,
                        fraction: float = 0.10) -> tuple[LBMConfig, np.ndarray]:
    """The standalone lattice at scale: n^3 channel (walls in y and z), g_x force, and
    non-overlapping spheres of radius U[4, 12] filling ~10% of the volume (seed 1)."""
    mask, _, _ = sphere_packing((n, n, n), fraction, 4.0, 12.0, seed, margin=1)
    mask = np.maximum(mask, wall_mask(n, n, n))
    cfg = LBMConfig(nx=n, ny=n, nz=n, viscosity=viscosity_for_tau(tau), force=(gx, 0.0, 0.0),
                    **PERIODIC_FACES)
    return cfg, mask


def closure_channel(seed: int, nx: int = 48, ny: int = 24, nz: int = 24, tau: float = 0.6,
                    gx: float = 2.0e-5, balls: int = 4, rmin: float = 2.5,
                    rmax: float = 4.5) -> tuple[LBMConfig, np.ndarray, np.ndarray]:
    """A scene of the learned closure's data set: the standalone lattice's geometry (channel
    with walls in y and z, periodic in x, driven by g_x, static balls) at a reduced size:
    ``balls`` balls with centres uniform in the interior (x in [5, nx-5], y, z 6 cells off
    the walls) and radii U[rmin, rmax], drawn from ``seed`` (balls may overlap).
    Returns (config, solid mask incl. walls, body mask: the balls alone)."""
    rng = np.random.default_rng(seed)
    bodies = np.zeros((nx, ny, nz), np.int32)
    for _ in range(balls):
        c = [rng.uniform(5, nx - 5), rng.uniform(6, ny - 6), rng.uniform(6, nz - 6)]
        add_sphere(bodies, c, rng.uniform(rmin, rmax))
    mask = np.maximum(bodies, wall_mask(nx, ny, nz))
    cfg = LBMConfig(nx=nx, ny=ny, nz=nz, viscosity=viscosity_for_tau(tau), force=(gx, 0.0, 0.0),
                    **PERIODIC_FACES)
    return cfg, mask, bodies


def cubes_mpm(n: int = 256, cubes: int = 64, edge: int = 16, seed: int = 2,
              gravity: float = -1.0e-4, dt: float = 0.1) -> tuple[MPMConfig, np.ndarray]:
    """The standalone solid at scale: ``cubes`` elastic cubes of ``edge``^3 cells at 8
    particles per cell (2 per axis) at random positions (seed 2) in an n^3 grid.
    64 cubes of 16^3 cells give 2,097,152 particles."""
    pos = random_cubes(n, cubes, edge, seed)
    cfg = MPMConfig(nx=n, ny=n, nz=n, max_particles=len(pos), particles_per_cell=2, dx=1.0, dt=dt,
                    density=1.5, youngs_modulus=0.05, poisson_ratio=0.3,
                    gravity=(0.0, gravity, 0.0), boundary_width=3)
    return cfg, pos


def coupled_smoke(steps: int = 1000) -> tuple[SimulationConfig, np.ndarray, np.ndarray]:
    """The 48x32x32 coupled smoke workload: tau 0.6 channel (walls in y, z), g_x = 1e-5, one
    elastic 8^3-cell cube (E 0.05, nu 0.3, rho_s 1.5) with corner (12,12,12), 2x2x2 particles per
    cell jittered in their sub-cells from seed 0 (4096 particles), gamma 0.1, 10 substeps per
    lattice step, gravity off."""
    nx, ny, nz = 48, 32, 32
    lbm = LBMConfig(nx=nx, ny=ny, nz=nz, viscosity=viscosity_for_tau(0.6), rho0=1.0,
                    force=(1.0e-5, 0.0, 0.0), **PERIODIC_FACES)
    mpm = MPMConfig(nx=nx, ny=ny, nz=nz, max_particles=4096, particles_per_cell=2, dx=1.0,
                    dt=0.1, density=1.5, youngs_modulus=0.05, poisson_ratio=0.3,
                    gravity=(0.0, 0.0, 0.0), boundary_width=3)
    cfg = SimulationConfig(num_steps=steps, lbm_dt=1.0, lbm=lbm, mpm=mpm,
                           coupling=CouplingConfig(gamma=0.1, mpm_substeps_per_lbm_step=10))
    rng = np.random.default_rng(0)
    idx = np.stack(np.meshgrid(np.arange(16), np.arange(16), np.arange(16), indexing="ij"),
                   axis=-1).reshape(-1, 3)
    pos = (12.0 + 0.5 * (idx + rng.uniform(0.0, 1.0, idx.shape))).astype(np.float32)
    return cfg, wall_mask(nx, ny, nz), pos


def sphere_particles(center, radius: float, ppc_axis: int, rng=None) -> np.ndarray:
    """Particles of a ball: the sub-cell lattice of its bounding cube of cells, jittered like
    ``cube_particles``, kept where the particle lies within ``radius`` of ``center``."""
    edge = int(np.ceil(2 * radius))
    lower = np.floor(np.asarray(center, np.float64) - edge / 2)
    pts = cube_particles(lower, edge, ppc_axis, rng)
    keep = np.linalg.norm(pts.astype(np.float64) - np.asarray(center), axis=1) <= radius
    return pts[keep]


def coupled_bodies(nx: int = 384, ny: int = 192, nz: int = 192, bodies: int = 48,
                   cube_edge: int = 12, sphere_radius: float = 6.0, tau: float = 0.55,
                   inflow: float = 0.05, seed: int = 3, substeps: int = 10,
                   start_moving: bool = True):
    """The coupled workload at scale: an nx*ny*nz channel (walls in y and z as mask planes)
    with a velocity inlet of ``inflow`` in x at x = 0 and a pressure outlet (rho 1) at
    x = nx-1; ``bodies`` elastic bodies, half cubes of edge ``cube_edge`` cells and half
    balls of radius ``sphere_radius``, at non-overlapping positions from ``seed``, 8
    particles per cell, Young's modulus U[0.02, 0.1] per body, nu 0.3, rho_s 1.2. With
    ``start_moving`` the fluid starts at the inflow velocity everywhere (so the bodies are
    driven, deform and move from the first step), else at rest (the inlet's flow then takes
    ~x/0.6 steps to reach a body at x).
    Returns (config, solid mask, positions, per-particle Young's modulus)."""
    rng = np.random.default_rng(seed)
    lbm = LBMConfig(nx=nx, ny=ny, nz=nz, viscosity=viscosity_for_tau(tau), rho0=1.0,
                    initial_velocity=(inflow, 0.0, 0.0) if start_moving else (0.0, 0.0, 0.0),
                    x_left=BoundaryConfig("velocity", velocity=(inflow, 0.0, 0.0)),
                    x_right=BoundaryConfig("pressure", rho=1.0),
                    y_left=BoundaryConfig("periodic"), y_right=BoundaryConfig("periodic"),
                    z_left=BoundaryConfig("periodic"), z_right=BoundaryConfig("periodic"))
    half = max(cube_edge / 2, sphere_radius)
    margin = half + 4
    centres = []
    tries = 0
    while len(centres) < bodies:
        tries += 1
        if tries > 1_000_000:
            raise RuntimeError("could not place the bodies without overlap")
        c = np.array([rng.uniform(margin + 16, nx - margin - 16), rng.uniform(margin, ny - margin),
                      rng.uniform(margin, nz - margin)])
        if any(np.max(np.abs(c - o)) < 2 * half + 2 for o in centres):
            continue
        centres.append(c)
    pos, young = [], []
    for b, c in enumerate(centres):
        if b % 2 == 0:
            p = cube_particles(np.floor(c - cube_edge / 2), cube_edge, 2, rng)
        else:
            p = sphere_particles(c, sphere_radius, 2, rng)
        pos.append(p)
        young.append(np.full(len(p), rng.uniform(0.02, 0.1), np.float32))
    pos = np.concatenate(pos)
    young = np.concatenate(young)
    mpm = MPMConfig(nx=nx, ny=ny, nz=nz, max_particles=len(pos), particles_per_cell=2, dx=1.0,
                    dt=1.0 / substeps, density=1.2, youngs_modulus=0.05, poisson_ratio=0.3,
                    gravity=(0.0, 0.0, 0.0), boundary_width=3)
    cfg = SimulationConfig(num_steps=2000, lbm_dt=1.0, lbm=lbm, mpm=mpm,
                           coupling=CouplingConfig(gamma=0.1, mpm_substeps_per_lbm_step=substeps))
    return cfg, wall_mask(nx, ny, nz), pos, young


def batch_scenes(count: int = 256, seed: int = 4, edges=(32, 48, 64, 96), bodies=(1, 4),
                 size=(4, 10), storage: str = "f16", substeps: int = 10):
    """Independent coupled scenes for a batch: per scene a cubic lattice of edge drawn from
    ``edges`` (walls in y and z as mask planes, periodic x), g_x U[1e-6, 1e-5], tau
    U[0.55, 0.8], and 1 to 4 non-overlapping elastic bodies -- cubes of edge or balls of
    radius U{4..10} cells, 8 particles per cell, Young's modulus U[0.02, 0.1] per body,
    nu 0.3, rho_s 1.2 -- all drawn from ``seed``. Population storage ``storage``.
    Returns a list of (config, solid mask, positions, per-particle Young's modulus)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.choice(edges))
        tau = float(rng.uniform(0.55, 0.8))
        gx = float(rng.uniform(1e-6, 1e-5))
        lbm = LBMConfig(nx=n, ny=n, nz=n, viscosity=viscosity_for_tau(tau),
                        force=(gx, 0.0, 0.0), population_storage=storage, **PERIODIC_FACES)
        want = int(rng.integers(bodies[0], bodies[1] + 1))
        placed = []  # (centre, half extent)
        pos, young = [], []
        tries = 0
        while len(placed) < want and tries < 1000:
            tries += 1
            s_ = int(rng.integers(size[0], size[1] + 1))
            cube = bool(rng.integers(0, 2))
            half = s_ / 2 if cube else float(s_)
            lo_c, hi_c = 4 + half, n - 4 - half
            if hi_c <= lo_c:
                continue
            c = rng.uniform(lo_c, hi_c, size=3)
            if any(np.max(np.abs(c - o)) < half + h + 1 for o, h in placed):
                continue
            placed.append((c, half))
            p = (cube_particles(np.floor(c - s_ / 2), s_, 2, rng) if cube
                 else sphere_particles(c, float(s_), 2, rng))
            pos.append(p)
            young.append(np.full(len(p), rng.uniform(0.02, 0.1), np.float32))
        pos = np.concatenate(pos)
        mpm = MPMConfig(nx=n, ny=n, nz=n, max_particles=len(pos), particles_per_cell=2, dx=1.0,
                        dt=1.0 / substeps, density=1.2, youngs_modulus=0.05, poisson_ratio=0.3,
                        gravity=(0.0, 0.0, 0.0), boundary_width=3)
        cfg = SimulationConfig(num_steps=500, lbm_dt=1.0, lbm=lbm, mpm=mpm,
                               coupling=CouplingConfig(gamma=0.1, mpm_substeps_per_lbm_step=substeps))
        out.append((cfg, wall_mask(n, n, n), pos, np.concatenate(young)))
    return out
