"""CPU oracle of the reference's coupled LBM-MPM timestep.

TEST INFRASTRUCTURE ONLY: used by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py as the checker. Nothing in the product package
imports it.

The classes below restate the host logic of the reference's solver classes
(fsi/lbm3d.py, fsi/mpm3d.py, fsi/coupling.py, fsi/simulation.py) over numpy
arrays in the reference's own layouts, and call the C++ restatement of each
Taichi kernel (oracle/fsi_oracle.cpp) through ctypes. ``dtype`` selects the
float32 (reference precision) or float64 (error-table) instantiation.

The class names match the reference so the reference's validation scenarios
can be run on the oracle by substituting the classes.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from . import build as _build

_Q = 19
_LIB = None

# D3Q19 velocities, fsi/lbm3d.py:221-239.
E = np.array(
    [[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
     [1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 0, 1], [-1, 0, -1], [1, 0, -1],
     [-1, 0, 1], [0, 1, 1], [0, -1, -1], [0, 1, -1], [0, -1, 1]], dtype=np.int32)
LR = np.array([0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17], dtype=np.int32)


def mrt_matrix() -> np.ndarray:
    """The 19x19 MRT transform of fsi/lbm3d.py:30-54 (float32)."""
    rows = [
        [1] * 19,
        [-1, 0, 0, 0, 0, 0, 0] + [1] * 12,
        [1, -2, -2, -2, -2, -2, -2] + [1] * 12,
        [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
        [0, -2, 2, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
        [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1],
        [0, 0, 0, -2, 2, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1],
        [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1],
        [0, 0, 0, 0, 0, -2, 2, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1],
        [0, 2, 2, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
        [0, -2, -2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
        [0, 0, 0, 1, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
        [0, 0, 0, -1, -1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, -1, 1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, -1, 1, 1, -1],
    ]
    return np.array(rows, dtype=np.float32)


def lattice_tables(viscosity: float):
    """M, inv(M), S and w exactly as fsi/lbm3d.py:140-174 and 244-248 build them (float32)."""
    tau_f = 3.0 * viscosity + 0.5
    s_v = 1.0 / tau_f
    s_o = 8.0 * (2.0 - s_v) / (8.0 - s_v)
    S = np.array([0.0, s_v, s_v, 0.0, s_o, 0.0, s_o, 0.0, s_o, s_v, s_v, s_v, s_v, s_v, s_v,
                  s_v, s_o, s_o, s_o], dtype=np.float32)
    M = mrt_matrix()
    invM = np.linalg.inv(M).astype(np.float32)
    w = np.empty(_Q, dtype=np.float32)
    w[0] = 1.0 / 3.0
    w[1:7] = 1.0 / 18.0
    w[7:] = 1.0 / 36.0
    return M, invM, S, w


def lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        _LIB = ctypes.CDLL(str(path))
        _LIB.oracle_max_threads.restype = ctypes.c_int
    return _LIB


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _suffix(dtype) -> str:
    return "f32" if np.dtype(dtype) == np.float32 else "f64"


def _real(dtype):
    return ctypes.c_float if np.dtype(dtype) == np.float32 else ctypes.c_double


# Mode codes of fsi/lbm3d.py:16-27.
def boundary_mode(boundary) -> int:
    t = boundary.boundary_type
    if t == "periodic":
        return 0
    if t == "pressure":
        return 1
    if t == "velocity":
        # 3: the extension that reads every population from before the update
        return 3 if getattr(boundary, "velocity_update", "sequential") == "simultaneous" else 2
    if t == "wall":
        raise NotImplementedError("wall face boundaries are reserved; use solid masks.")
    raise ValueError(f"Unsupported boundary type: {t}.")


class LBMSolver3D:
    """Oracle of fsi/lbm3d.py:57-534 over numpy arrays."""

    def __init__(self, config, dtype=np.float32, nthreads: int = 1):
        config.validate()
        if config.use_sparse:
            raise NotImplementedError("Sparse LBM storage is not implemented.")
        for name, b in (("x_left", config.x_left), ("x_right", config.x_right)):
            if b.boundary_type not in ("periodic", "pressure", "velocity"):
                raise NotImplementedError(f"{name}={b.boundary_type!r} is not implemented.")
        for name, b in (("y_left", config.y_left), ("y_right", config.y_right),
                        ("z_left", config.z_left), ("z_right", config.z_right)):
            if b.boundary_type != "periodic":
                raise NotImplementedError(f"{name}={b.boundary_type!r} is not implemented.")
        self.config = config
        self.dtype = np.dtype(dtype)
        self.nthreads = nthreads
        self.nx, self.ny, self.nz = int(config.nx), int(config.ny), int(config.nz)
        self.q = _Q
        self.bc_x_left_mode = boundary_mode(config.x_left)
        self.bc_x_right_mode = boundary_mode(config.x_right)
        M, invM, S, w = lattice_tables(config.viscosity)
        # LBMConfig.mrt_rates (an extension with no reference counterpart) replaces single
        # entries of S; every other rate is the reference's rule above.
        for k, rate in (getattr(config, "mrt_rates", None) or {}).items():
            S[int(k)] = np.float32(rate)
        dt = self.dtype
        self.M, self.invM, self.S, self.w = (np.ascontiguousarray(a.astype(dt)) for a in (M, invM, S, w))
        shape = (self.nx, self.ny, self.nz)
        self.f = np.zeros((*shape, _Q), dt)
        self.F = np.zeros((*shape, _Q), dt)
        self.rho = np.zeros(shape, dt)
        self.v = np.zeros((*shape, 3), dt)
        self.force = np.zeros((*shape, 3), dt)
        self.solid = np.zeros(shape, np.int32)
        self.base_force = np.array(config.force, dtype=np.float32).astype(dt)
        self.rho0 = dt.type(np.float32(config.rho0))
        self._initialized = False

    def initialize(self, solid_np=None):
        if solid_np is None:
            solid = np.zeros((self.nx, self.ny, self.nz), np.int32)
        else:
            arr = np.asarray(solid_np)
            if arr.shape != (self.nx, self.ny, self.nz):
                raise ValueError(f"solid_np shape must be {(self.nx, self.ny, self.nz)}, got {arr.shape}.")
            solid = np.ascontiguousarray(np.where(arr > 0, 1, 0).astype(np.int32))
        self.solid[...] = solid
        u0 = np.array(self.config.initial_velocity, dtype=np.float32).astype(self.dtype)
        getattr(lib(), "oracle_lbm_init_" + _suffix(self.dtype))(
            self.nx, self.ny, self.nz, _p(self.f), _p(self.F), _p(self.rho), _p(self.v),
            _p(self.solid), _p(self.w), _real(self.dtype)(self.rho0), _p(u0))
        self.reset_force()
        self._initialized = True

    def step(self):
        if not self._initialized:
            raise RuntimeError("LBMSolver3D.initialize must be called before step().")
        c = self.config
        dt = self.dtype
        real = _real(dt)
        vl = np.array(c.x_left.velocity, np.float32).astype(dt)
        vr = np.array(c.x_right.velocity, np.float32).astype(dt)
        getattr(lib(), "oracle_lbm_step_" + _suffix(dt))(
            self.nx, self.ny, self.nz, _p(self.f), _p(self.F), _p(self.rho), _p(self.v),
            _p(self.force), _p(self.solid), _p(self.M), _p(self.invM), _p(self.S), _p(self.w),
            self.bc_x_left_mode, self.bc_x_right_mode, real(np.float32(c.x_left.rho)),
            real(np.float32(c.x_right.rho)), _p(vl), _p(vr), real(self.rho0), self.nthreads)

    # accessors, fsi/lbm3d.py:435-457
    def density_numpy(self):
        return self.rho.copy()

    def velocity_numpy(self):
        return self.v.copy()

    def solid_numpy(self):
        return self.solid.copy()

    def distribution_numpy(self):
        return self.f.copy()

    def force_numpy(self):
        return self.force.copy()

    def total_mass(self):
        return float(self.rho[self.solid == 0].sum())

    def max_velocity_norm(self):
        return float(np.linalg.norm(self.v, axis=-1).max())

    # force API, fsi/lbm3d.py:459-534
    def clear_force(self):
        self.force[...] = 0

    def reset_force(self):
        self.force[...] = self.base_force
        self.force[self.solid != 0] = 0

    @staticmethod
    def _vec(force, name):
        arr = np.asarray(force, dtype=np.float32)
        if arr.shape != (3,):
            raise ValueError(f"{name} must have 3 components.")
        return arr

    def set_uniform_force(self, force):
        val = self._vec(force, "force").astype(self.dtype)
        self.force[...] = val
        self.force[self.solid != 0] = 0

    def add_uniform_force(self, force):
        val = self._vec(force, "force").astype(self.dtype)
        fluid = self.solid == 0
        self.force[fluid] = self.force[fluid] + val
        self.force[~fluid] = 0

    def set_force_from_numpy(self, force_np):
        arr = np.asarray(force_np, dtype=np.float32)
        if arr.shape != (self.nx, self.ny, self.nz, 3):
            raise ValueError("force_np has the wrong shape.")
        self.force[...] = arr
        self.zero_force_on_solid()

    def total_force(self):
        return self.force[self.solid == 0].sum(axis=0)

    def zero_force_on_solid(self):
        self.force[self.solid != 0] = 0


class MPMSolver3D:
    """Oracle of fsi/mpm3d.py:9-368 over numpy arrays."""

    def __init__(self, config, dtype=np.float32, nthreads: int = 1, deterministic: bool = True,
                 polar: str = "exact", cell_order: bool = False):
        """``cell_order`` sums the P2G scatter (and the coupler's spread) in the cell order of
        the GPU's sorted scatter (oracle/fsi_oracle.cpp, p2g_cell_order); otherwise
        ``deterministic`` selects a serial particle-order loop or threads with atomics."""
        config.validate()
        if polar not in ("exact", "device"):
            raise ValueError("polar must be 'exact' or 'device'")
        self.polar = polar
        self.cell_order = bool(cell_order)
        self.config = config
        self.dtype = np.dtype(dtype)
        self.nthreads = nthreads
        self.deterministic = deterministic
        self.nx, self.ny, self.nz = int(config.nx), int(config.ny), int(config.nz)
        self.max_particles = int(config.max_particles)
        self.dx = float(config.dx)
        self.inv_dx = 1.0 / self.dx
        self.dt_default = float(config.dt)
        self.boundary_width = int(config.boundary_width)
        self.boundary_damping = float(config.boundary_damping)
        self.apic = bool(config.apic)
        self.mu = config.youngs_modulus / (2.0 * (1.0 + config.poisson_ratio))
        self.lam = (config.youngs_modulus * config.poisson_ratio
                    / ((1.0 + config.poisson_ratio) * (1.0 - 2.0 * config.poisson_ratio)))
        P = self.max_particles
        dt = self.dtype
        self.num_particles = 0
        self.x = np.zeros((P, 3), dt)
        self.v = np.zeros((P, 3), dt)
        self.C = np.zeros((P, 3, 3), dt)
        self.F = np.zeros((P, 3, 3), dt)
        self.mass = np.zeros(P, dt)
        self.volume = np.zeros(P, dt)
        self.active = np.zeros(P, np.int32)
        self.particle_force = np.zeros((P, 3), dt)
        self.grid_v = np.zeros((self.nx, self.ny, self.nz, 3), dt)
        self.grid_m = np.zeros((self.nx, self.ny, self.nz), dt)
        self.mu_p = self.lam_p = None
        self._initialized = False

    def initialize_particles_box(self, lower, upper, spacing=None, initial_velocity=(0.0, 0.0, 0.0)):
        lo = np.asarray(lower, dtype=np.float32)
        hi = np.asarray(upper, dtype=np.float32)
        if lo.shape != (3,) or hi.shape != (3,):
            raise ValueError("lower/upper must have 3 components.")
        if np.any(hi <= lo):
            raise ValueError("upper must be greater than lower in every dimension.")
        if spacing is None:
            sp = np.full(3, self.dx / float(self.config.particles_per_cell), np.float32)
        elif np.isscalar(spacing):
            sp = np.full(3, float(spacing), np.float32)
        else:
            sp = np.asarray(spacing, np.float32)
        axes = [np.arange(lo[a], hi[a], sp[a]) for a in range(3)]
        if any(len(ax) == 0 for ax in axes):
            raise ValueError("particle box produced no particles.")
        mesh = np.meshgrid(*axes, indexing="ij")
        pos = np.stack([m.ravel() for m in mesh], axis=1).astype(np.float32)
        vel = np.broadcast_to(np.asarray(initial_velocity, np.float32), pos.shape).astype(np.float32)
        return self.initialize_particles_from_numpy(pos, velocities=vel, particle_volume=float(np.prod(sp)))

    def initialize_particles_from_numpy(self, positions, velocities=None, particle_mass=None,
                                        particle_volume=None, youngs_modulus=None,
                                        poisson_ratio=None):
        pos = np.asarray(positions, dtype=np.float32)
        if pos.ndim != 2 or pos.shape[1] != 3:
            raise ValueError("positions must have shape (n, 3).")
        n = pos.shape[0]
        if n <= 0:
            raise ValueError("positions must contain at least one particle.")
        if n > self.max_particles:
            raise ValueError(f"particle count {n} exceeds max_particles={self.max_particles}.")
        vel = np.zeros((n, 3), np.float32) if velocities is None else np.asarray(velocities, np.float32)
        if vel.shape != (n, 3):
            raise ValueError("velocities have the wrong shape.")
        vol = float(particle_volume) if particle_volume is not None else self.dx ** 3 / float(self.config.particles_per_cell ** 3)
        if vol <= 0:
            raise ValueError("particle_volume must be positive.")
        mass = float(particle_mass) if particle_mass is not None else float(self.config.density) * vol
        if mass <= 0:
            raise ValueError("particle_mass must be positive.")
        for a in (self.x, self.v, self.C, self.F, self.mass, self.volume, self.particle_force):
            a[...] = 0
        self.active[...] = 0
        dt = self.dtype
        self.x[:n] = pos.astype(dt)
        self.v[:n] = vel.astype(dt)
        self.F[:n] = np.eye(3, dtype=dt)
        self.mass[:n] = dt.type(np.float32(mass))
        self.volume[:n] = dt.type(np.float32(vol))
        self.active[:n] = 1
        self.mu_p = self.lam_p = None
        if youngs_modulus is not None or poisson_ratio is not None:
            E = np.broadcast_to(np.asarray(self.config.youngs_modulus if youngs_modulus is None
                                           else youngs_modulus, np.float64), (n,))
            nu = np.broadcast_to(np.asarray(self.config.poisson_ratio if poisson_ratio is None
                                            else poisson_ratio, np.float64), (n,))
            mu = E / (2.0 * (1.0 + nu))
            lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
            self.mu_p = np.zeros(self.max_particles, self.dtype)
            self.lam_p = np.zeros(self.max_particles, self.dtype)
            self.mu_p[:n] = mu.astype(np.float32).astype(self.dtype)
            self.lam_p[:n] = lam.astype(np.float32).astype(self.dtype)
        self.num_particles = n
        self._initialized = True
        return n

    def substep(self, dt=None):
        if not self._initialized:
            raise RuntimeError("MPMSolver3D particle initialization must be called before substep().")
        dt_value = self.dt_default if dt is None else float(dt)
        if dt_value <= 0.0:
            raise ValueError("dt must be positive.")
        d = self.dtype
        real = _real(d)
        cast = (lambda v: real(np.float32(v))) if d == np.float32 else (lambda v: real(v))
        grav = np.array(self.config.gravity, np.float32).astype(d)
        upper = np.array([(self.nx - 1.5) * self.dx, (self.ny - 1.5) * self.dx,
                          (self.nz - 1.5) * self.dx], np.float32).astype(d)
        getattr(lib(), "oracle_mpm_substep_" + _suffix(d))(
            self.nx, self.ny, self.nz, self.num_particles, _p(self.x), _p(self.v), _p(self.C),
            _p(self.F), _p(self.mass), _p(self.volume), _p(self.active), _p(self.particle_force),
            _p(self.grid_v), _p(self.grid_m), cast(dt_value), cast(self.dx), cast(self.inv_dx),
            cast(self.mu), cast(self.lam), _p(grav), self.boundary_width,
            cast(self.boundary_damping), int(self.apic), cast(0.5 * self.dx), _p(upper),
            self.nthreads, 2 if self.cell_order else int(self.deterministic),
            1 if self.polar == "device" else 0,
            _p(self.mu_p) if self.mu_p is not None else None,
            _p(self.lam_p) if self.lam_p is not None else None,
            1 if getattr(self.config, "constitutive_model", "fixed_corotated") == "neo_hookean" else 0)

    def clear_particle_force(self):
        self.particle_force[: self.num_particles] = 0

    def particle_count(self):
        return int(self.num_particles)

    def positions_numpy(self):
        return self.x[: self.num_particles].copy()

    def velocities_numpy(self):
        return self.v[: self.num_particles].copy()

    def particle_forces_numpy(self):
        return self.particle_force[: self.num_particles].copy()

    def deformation_gradients_numpy(self):
        return self.F[: self.num_particles].copy()

    def active_numpy(self):
        return self.active[: self.num_particles].copy()

    def center_of_mass(self):
        n = self.num_particles
        if n == 0:
            return np.zeros(3, np.float32)
        pos = self.positions_numpy()
        m = self.mass[:n]
        tot = m.sum()
        if tot <= 0:
            return np.zeros(3, np.float32)
        return (pos * m[:, None]).sum(axis=0) / tot

    def max_velocity_norm(self):
        vel = self.velocities_numpy()
        if len(vel) == 0:
            return 0.0
        return float(np.linalg.norm(vel, axis=1).max())


class LBMMpmCoupler:
    """Oracle of fsi/coupling.py:11-496."""

    def __init__(self, config, lbm: LBMSolver3D, mpm: MPMSolver3D):
        config.validate()
        self.config = config
        self.lbm, self.mpm = lbm, mpm
        if config.kernel != "quadratic":
            raise ValueError(f"Unsupported coupling kernel: {config.kernel}.")
        if (lbm.nx, lbm.ny, lbm.nz) != (mpm.nx, mpm.ny, mpm.nz):
            raise ValueError("LBM and MPM grids must match.")
        self.enabled = bool(config.enabled)
        self.build_solid_volume_fraction = bool(config.build_solid_volume_fraction)
        self.immersed_boundary_enabled = bool(config.immersed_boundary_enabled)
        self.contact_enabled = bool(config.contact_enabled)
        self.substeps = int(config.mpm_substeps_per_lbm_step)
        self.nx, self.ny, self.nz = lbm.nx, lbm.ny, lbm.nz
        self.inv_dx = 1.0 / float(mpm.dx)
        self.cell_volume = float(mpm.dx) ** 3
        d = lbm.dtype
        self.dtype = d
        shape = (self.nx, self.ny, self.nz)
        self.coupling_force = np.zeros((*shape, 3), d)
        self.solid_volume_fraction = np.zeros(shape, d)
        self.immersed_boundary_force = np.zeros((*shape, 3), d)
        P = mpm.max_particles
        self.particle_valid_weight = np.zeros(P, d)
        self.particle_coupling_mask = np.zeros(P, np.int32)
        self.particle_contact_mask = np.zeros(P, np.int32)
        self.coupled_step = 0
        self.counters = np.zeros(3, np.int32)      # unsupported, partial, clipped
        self.ib_counters = np.zeros(2, np.int32)   # active, clipped
        self.ib_total = np.zeros(3, d)
        self.contact_counters = np.zeros(2, np.int32)  # candidates, damped

    def _validate_initialized(self):
        if not getattr(self.lbm, "_initialized", False):
            raise RuntimeError("LBMSolver3D.initialize must be called before coupling.")
        if not getattr(self.mpm, "_initialized", False):
            raise RuntimeError("MPMSolver3D particle initialization must be called before coupling.")

    def _real(self, v):
        return _real(self.dtype)(np.float32(v) if self.dtype == np.float32 else v)

    def effective_gamma(self):
        g = float(self.config.gamma)
        r = int(self.config.gamma_ramp_steps)
        if r <= 0:
            return g
        return g * min(1.0, float(self.coupled_step + 1) / float(r))

    def _gamma_device(self):
        # _effective_gamma, coupling.py:321-330, in the kernel's float type.
        f = self.dtype.type
        g = f(np.float32(self.config.gamma)) if self.dtype == np.float32 else f(self.config.gamma)
        r = int(self.config.gamma_ramp_steps)
        if r > 0:
            ramp = (f(self.coupled_step) + f(1.0)) / f(r)
            g = g * min(f(1.0), ramp)
        return g

    def clear_coupling_fields(self):
        self.ib_counters[...] = 0
        self.ib_total[...] = 0
        self.coupling_force[...] = 0
        self.solid_volume_fraction[...] = 0
        self.immersed_boundary_force[...] = 0
        self.clear_particle_diagnostics()

    def clear_particle_diagnostics(self):
        self.counters[...] = 0
        self.contact_counters[...] = 0
        self.particle_valid_weight[...] = 0
        self.particle_coupling_mask[...] = 0
        self.particle_contact_mask[...] = 0

    def _coupling_kernel(self, dt_ratio, build_fraction):
        c = self.config
        d = self.dtype
        getattr(lib(), "oracle_coupling_" + _suffix(d))(
            self.nx, self.ny, self.nz, self.mpm.num_particles, _p(self.mpm.x), _p(self.mpm.v),
            _p(self.mpm.mass), _p(self.mpm.volume), _p(self.mpm.active), _p(self.mpm.particle_force),
            _p(self.lbm.v), _p(self.lbm.solid), _p(self.coupling_force),
            _p(self.solid_volume_fraction), _p(self.particle_valid_weight),
            _p(self.particle_coupling_mask), _p(self.counters), self._real(self.inv_dx),
            _real(d)(self._gamma_device()), self._real(dt_ratio), self._real(self.cell_volume),
            int(build_fraction), self._real(c.min_valid_weight),
            int(c.relative_velocity_limit is not None),
            self._real(c.relative_velocity_limit or 0.0), int(c.force_limit is not None),
            self._real(c.force_limit or 0.0), int(getattr(self.mpm, "cell_order", False)),
            self.mpm.nthreads if not self.mpm.deterministic else 1)

    def _clamp_fraction(self):
        np.minimum(self.solid_volume_fraction, self.dtype.type(1.0), out=self.solid_volume_fraction)

    def _apply_coupling(self):
        fluid = self.lbm.solid == 0
        self.lbm.force[fluid] = self.lbm.force[fluid] + self.coupling_force[fluid]
        self.lbm.force[~fluid] = 0

    def _ib_kernel(self):
        c = self.config
        d = self.dtype
        getattr(lib(), "oracle_ib_" + _suffix(d))(
            ctypes.c_long(self.nx * self.ny * self.nz), _p(self.solid_volume_fraction),
            _p(self.lbm.rho), _p(self.lbm.v), _p(self.lbm.solid), _p(self.immersed_boundary_force),
            _p(self.ib_counters), _p(self.ib_total), int(self.immersed_boundary_enabled),
            self._real(c.immersed_boundary_drag), self._real(c.immersed_boundary_fraction_threshold),
            int(c.immersed_boundary_max_force is not None),
            self._real(c.immersed_boundary_max_force or 0.0))

    def _apply_ib(self):
        fluid = self.lbm.solid == 0
        self.lbm.force[fluid] = self.lbm.force[fluid] + self.immersed_boundary_force[fluid]
        self.immersed_boundary_force[~fluid] = 0
        self.lbm.force[~fluid] = 0

    def _contact_kernel(self):
        c = self.config
        d = self.dtype
        getattr(lib(), "oracle_contact_" + _suffix(d))(
            self.nx, self.ny, self.nz, self.mpm.num_particles, _p(self.mpm.x), _p(self.mpm.v),
            _p(self.mpm.active), _p(self.solid_volume_fraction), _p(self.lbm.solid),
            _p(self.particle_contact_mask), _p(self.contact_counters), self._real(self.inv_dx),
            int(self.contact_enabled), self._real(c.contact_fraction_threshold),
            self._real(c.contact_velocity_damping))

    # coupling.py:135-173
    def step(self, lbm_dt):
        lbm_dt = float(lbm_dt)
        if lbm_dt <= 0.0:
            raise ValueError("lbm_dt must be positive.")
        self._validate_initialized()
        self.clear_coupling_fields()
        mpm_dt = lbm_dt / float(self.substeps)
        dt_ratio = mpm_dt / lbm_dt
        for s in range(self.substeps):
            self.mpm.clear_particle_force()
            if self.enabled:
                self.clear_particle_diagnostics()
                self._coupling_kernel(dt_ratio, s == 0 and self.build_solid_volume_fraction)
            self.mpm.substep(dt=mpm_dt)
            if self.contact_enabled:
                self._contact_kernel()
        if self.enabled and self.build_solid_volume_fraction:
            self._clamp_fraction()
        self.lbm.reset_force()
        if self.enabled:
            self._apply_coupling()
        if self.immersed_boundary_enabled:
            self._ib_kernel()
            self._apply_ib()
        self.lbm.step()
        if self.enabled:
            self.coupled_step += 1

    # coupling.py:175-196
    def compute_coupling_forces(self, dt_ratio=1.0):
        dt_ratio = float(dt_ratio)
        if dt_ratio < 0.0:
            raise ValueError("dt_ratio must be non-negative.")
        self._validate_initialized()
        self.clear_coupling_fields()
        self.mpm.clear_particle_force()
        if not self.enabled:
            return
        self._coupling_kernel(dt_ratio, self.build_solid_volume_fraction)
        if self.build_solid_volume_fraction:
            self._clamp_fraction()
        if self.contact_enabled:
            self._contact_kernel()
        if self.immersed_boundary_enabled:
            self._ib_kernel()

    def coupling_force_numpy(self):
        return self.coupling_force.copy()

    def solid_volume_fraction_numpy(self):
        return self.solid_volume_fraction.copy()

    def immersed_boundary_force_numpy(self):
        return self.immersed_boundary_force.copy()

    def particle_valid_weights_numpy(self):
        return self.particle_valid_weight[: self.mpm.num_particles].copy()

    def particle_coupling_mask_numpy(self):
        return self.particle_coupling_mask[: self.mpm.num_particles].copy()

    def particle_contact_mask_numpy(self):
        return self.particle_contact_mask[: self.mpm.num_particles].copy()

    def total_particle_coupling_force(self):
        return self.mpm.particle_forces_numpy().sum(axis=0)

    def total_fluid_coupling_force(self):
        return self.coupling_force[self.lbm.solid == 0].sum(axis=0)

    def immersed_boundary_diagnostics(self):
        t = np.array(self.ib_total, dtype=np.float64)
        return {
            "ib_active_cell_count": int(self.ib_counters[0]),
            "ib_clipped_cell_count": int(self.ib_counters[1]),
            "ib_total_force_x": float(t[0]),
            "ib_total_force_y": float(t[1]),
            "ib_total_force_z": float(t[2]),
            "ib_total_force_norm": float(np.linalg.norm(t)),
            "contact_candidate_count": int(self.contact_counters[0]),
            "contact_damped_particle_count": int(self.contact_counters[1]),
        }

    def coupling_diagnostics(self):
        vw = self.particle_valid_weights_numpy()
        mn = float(vw.min()) if len(vw) else 0.0
        mean = float(vw.mean()) if len(vw) else 0.0
        return {
            "unsupported_particle_count": int(self.counters[0]),
            "partial_support_particle_count": int(self.counters[1]),
            "clipped_particle_count": int(self.counters[2]),
            "min_particle_valid_weight": mn,
            "mean_particle_valid_weight": mean,
            "effective_gamma": self.effective_gamma(),
            **self.immersed_boundary_diagnostics(),
        }


class FSISimulation:
    """Oracle of fsi/simulation.py:12-153 (no snapshot writer)."""

    def __init__(self, config, dtype=np.float32, nthreads: int = 1, polar: str = "exact",
                 deterministic: bool = True, cell_order: bool = False):
        config.validate()
        self.config = config
        self.lbm = LBMSolver3D(config.lbm, dtype=dtype, nthreads=nthreads)
        self.mpm = MPMSolver3D(config.mpm, dtype=dtype, nthreads=nthreads, polar=polar,
                               deterministic=deterministic, cell_order=cell_order)
        self.coupler = LBMMpmCoupler(config.coupling, self.lbm, self.mpm)
        self.step_index = 0
        self.time = 0.0
        self._lbm_initialized = False
        self._mpm_initialized = False

    def initialize_lbm(self, solid_np=None):
        self.lbm.initialize(solid_np=solid_np)
        self._lbm_initialized = True

    def initialize_mpm_box(self, lower, upper, spacing=None, initial_velocity=(0.0, 0.0, 0.0)):
        n = self.mpm.initialize_particles_box(lower, upper, spacing, initial_velocity)
        self._mpm_initialized = True
        return n

    def initialize_mpm_from_numpy(self, positions, velocities=None, particle_mass=None,
                                  particle_volume=None, youngs_modulus=None, poisson_ratio=None):
        n = self.mpm.initialize_particles_from_numpy(positions, velocities, particle_mass,
                                                     particle_volume, youngs_modulus, poisson_ratio)
        self._mpm_initialized = True
        return n

    def initialize(self, solid_np=None, mpm_box_lower=None, mpm_box_upper=None,
                   mpm_box_spacing=None, mpm_initial_velocity=(0.0, 0.0, 0.0)):
        if mpm_box_lower is None or mpm_box_upper is None:
            raise ValueError("mpm_box_lower and mpm_box_upper are required.")
        self.initialize_lbm(solid_np)
        return self.initialize_mpm_box(mpm_box_lower, mpm_box_upper, mpm_box_spacing, mpm_initial_velocity)

    def _validate_initialized(self):
        if not self._lbm_initialized or not self.lbm._initialized:
            raise RuntimeError("FSISimulation.initialize_lbm must be called before stepping.")
        if not self._mpm_initialized or not self.mpm._initialized:
            raise RuntimeError("FSISimulation MPM initialization must be called before stepping.")

    def step(self):
        self._validate_initialized()
        self.coupler.step(self.config.lbm_dt)
        self.step_index += 1
        self.time += self.config.lbm_dt
        return self.diagnostics()

    def run(self, steps=None, write_output=False, write_initial=False):
        self._validate_initialized()
        count = self.config.num_steps if steps is None else int(steps)
        if count <= 0:
            raise ValueError("steps must be positive.")
        return [self.step() for _ in range(count)]

    def diagnostics(self):
        self._validate_initialized()
        cd = self.coupler.coupling_diagnostics()
        return {
            "step": self.step_index,
            "time": self.time,
            "lbm_total_mass": self.lbm.total_mass(),
            "lbm_max_velocity_norm": self.lbm.max_velocity_norm(),
            "mpm_particle_count": self.mpm.particle_count(),
            "mpm_center_of_mass": self.mpm.center_of_mass(),
            "mpm_max_velocity_norm": self.mpm.max_velocity_norm(),
            "total_particle_coupling_force": self.coupler.total_particle_coupling_force(),
            "total_fluid_coupling_force": self.coupler.total_fluid_coupling_force(),
            "coupling_unsupported_particle_count": cd["unsupported_particle_count"],
            "coupling_partial_support_particle_count": cd["partial_support_particle_count"],
            "coupling_clipped_particle_count": cd["clipped_particle_count"],
            "coupling_effective_gamma": cd["effective_gamma"],
            "coupling_ib_active_cell_count": cd["ib_active_cell_count"],
            "coupling_ib_clipped_cell_count": cd["ib_clipped_cell_count"],
            "coupling_ib_total_force_norm": cd["ib_total_force_norm"],
            "coupling_contact_candidate_count": cd["contact_candidate_count"],
            "coupling_contact_damped_particle_count": cd["contact_damped_particle_count"],
        }


def polar_rotation_device_f32(F: np.ndarray) -> np.ndarray:
    """Polar rotation with the device library's float32 operation order."""
    F = np.ascontiguousarray(np.asarray(F, np.float32).reshape(-1, 3, 3))
    R = np.empty_like(F)
    lib().oracle_polar_newton_f32(F.shape[0], _p(F), _p(R))
    return R


def polar_rotation(F: np.ndarray) -> np.ndarray:
    """Polar rotation of a batch of 3x3 matrices via the oracle's Jacobi SVD (float64)."""
    F = np.ascontiguousarray(np.asarray(F, np.float64).reshape(-1, 3, 3))
    R = np.empty_like(F)
    lib().oracle_polar_rotation_f64(F.shape[0], _p(F), _p(R))
    return R
