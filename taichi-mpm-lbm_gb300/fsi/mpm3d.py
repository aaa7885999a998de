"""Dense 3D MLS-MPM/APIC elastic solid on the GPU (drop-in for the reference's fsi/mpm3d.py).

Particles are stored as structure-of-arrays torch CUDA tensors (x, v, force
``[3, capacity]``; C, F ``[9, capacity]``; mass, volume, active ``[capacity]``)
and advanced by the library's sm_103a substep. The default ("atomic" p2g_mode)
scatters through shared-memory tiles with atomics and keeps the float4 grid
all-zero between substeps by clearing only the node blocks that were touched;
"sorted" sorts the particles by cell every substep and sums each grid node's
contributions in one fixed order with plain stores (bit-reproducible). The grid
update is fused into G2P in both.

Public methods, accessors and exceptions follow fsi/mpm3d.py:9-368.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .config import MPMConfig


def mpm_descriptor(config: MPMConfig, dt: float | None = None) -> nat.MpmDesc:
    """The C-ABI descriptor of a solver with this configuration (num_particles 0)."""
    d = nat.MpmDesc()
    d.nx, d.ny, d.nz = int(config.nx), int(config.ny), int(config.nz)
    d.num_particles = 0
    dx = float(config.dx)
    d.dt = float(np.float32(config.dt if dt is None else dt))
    d.dx = float(np.float32(dx))
    d.inv_dx = float(np.float32(1.0 / dx))
    E, nu = config.youngs_modulus, config.poisson_ratio
    d.mu = float(np.float32(E / (2.0 * (1.0 + nu))))  # Lame parameters, mpm3d.py:33-38
    d.lam = float(np.float32(E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))))
    for i in range(3):
        d.gravity[i] = float(np.float32(config.gravity[i]))
    d.boundary_damping = float(np.float32(config.boundary_damping))
    d.boundary_width = int(config.boundary_width)
    d.apic = 1 if config.apic else 0
    # position clamp of mpm3d.py:320-328
    d.clamp_lower = float(np.float32(0.5 * dx))
    for i, n in enumerate((config.nx, config.ny, config.nz)):
        d.clamp_upper[i] = float(np.float32((n - 1.5) * dx))
    d.material = 1 if config.constitutive_model == "neo_hookean" else 0
    return d


def particle_mass_volume(config: MPMConfig, particle_mass=None, particle_volume=None):
    """Per-particle (mass, volume) of mpm3d.py:135-140: volume dx^3 / ppc^3, mass rho V."""
    volume = (float(particle_volume) if particle_volume is not None
              else float(config.dx) ** 3 / float(config.particles_per_cell ** 3))
    if volume <= 0.0:
        raise ValueError("particle_volume must be positive.")
    mass = float(particle_mass) if particle_mass is not None else float(config.density) * volume
    if mass <= 0.0:
        raise ValueError("particle_mass must be positive.")
    return mass, volume


class MPMSolver3D:
    """Standalone dense 3D elastic MLS-MPM solver (GPU)."""

    def __init__(self, config: MPMConfig):
        self.config = config
        self.config.validate()
        self.nx = int(config.nx)
        self.ny = int(config.ny)
        self.nz = int(config.nz)
        self.max_particles = int(config.max_particles)
        self.dx = float(config.dx)
        self.inv_dx = 1.0 / self.dx
        self.dt_default = float(config.dt)
        self.boundary_width = int(config.boundary_width)
        self.boundary_damping = float(config.boundary_damping)
        self.apic = bool(config.apic)
        # Lame parameters (mpm3d.py:33-38)
        self.mu = config.youngs_modulus / (2.0 * (1.0 + config.poisson_ratio))
        self.lam = (config.youngs_modulus * config.poisson_ratio
                    / ((1.0 + config.poisson_ratio) * (1.0 - 2.0 * config.poisson_ratio)))

        self._device = nat.device()
        nat.load()
        cap = self.max_particles
        dev = self._device
        f32 = torch.float32
        self._x = torch.zeros((3, cap), dtype=f32, device=dev)
        self._v = torch.zeros((3, cap), dtype=f32, device=dev)
        self._C = torch.zeros((9, cap), dtype=f32, device=dev)
        self._F = torch.zeros((9, cap), dtype=f32, device=dev)
        self._mass = torch.zeros(cap, dtype=f32, device=dev)
        self._volume = torch.zeros(cap, dtype=f32, device=dev)
        self._active = torch.zeros(cap, dtype=torch.int32, device=dev)
        self._force = torch.zeros((3, cap), dtype=f32, device=dev)
        n_nodes = self.nx * self.ny * self.nz
        self._grid = torch.zeros((n_nodes, 4), dtype=f32, device=dev)
        nblocks = ((self.nx + 3) // 4) * ((self.ny + 3) // 4) * ((self.nz + 3) // 4)
        self._dirty = torch.zeros(nblocks, dtype=torch.uint8, device=dev)
        self.sorted = config.p2g_mode == "sorted"
        self._work = None
        if self.sorted:
            self._work = torch.zeros(self._workspace_bytes(), dtype=torch.uint8, device=dev)
        self._diag = torch.zeros(8, dtype=torch.float64, device=dev)
        self._diag_host = torch.zeros(8, dtype=torch.float64).pin_memory()
        self._num_particles = 0
        self._mu_p = self._lam_p = None
        self._desc = self._make_desc()
        self._parts = self._make_particles()
        self._initialized = False
        self.tuning = None  # launch parameters chosen by fsi.autotune.tune_coupled

    # ----------------------------------------------------------------- setup
    def _make_desc(self) -> nat.MpmDesc:
        return mpm_descriptor(self.config)

    def _workspace_bytes(self) -> int:
        out = nat.ctypes.c_int64(0)
        nat.call("fsi_mpm_workspace_bytes", mpm_descriptor(self.config), self.max_particles,
                 nat.ctypes.byref(out))
        return int(out.value)

    @property
    def workspace(self) -> torch.Tensor | None:
        """The sort workspace of the "sorted" P2G (None in "atomic" mode)."""
        return self._work

    @staticmethod
    def lame_parameters(youngs_modulus, poisson_ratio):
        """(mu, lam) of mpm3d.py:33-38 for scalars or arrays."""
        E = np.asarray(youngs_modulus, dtype=np.float64)
        nu = np.asarray(poisson_ratio, dtype=np.float64)
        mu = E / (2.0 * (1.0 + nu))
        lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
        return mu, lam

    def _set_particle_materials(self, count: int, youngs_modulus, poisson_ratio) -> None:
        if youngs_modulus is None and poisson_ratio is None:
            self._mu_p = self._lam_p = None
            self._parts.mu = self._parts.lam = None
            return
        E = np.broadcast_to(np.asarray(self.config.youngs_modulus if youngs_modulus is None
                                       else youngs_modulus, np.float64), (count,))
        nu = np.broadcast_to(np.asarray(self.config.poisson_ratio if poisson_ratio is None
                                        else poisson_ratio, np.float64), (count,))
        if np.any(E <= 0.0):
            raise ValueError("Young's modulus must be positive.")
        if np.any((nu <= -1.0) | (nu >= 0.5)):
            raise ValueError("Poisson ratio must be in (-1, 0.5).")
        mu, lam = self.lame_parameters(E, nu)
        self._mu_p = torch.zeros(self.max_particles, dtype=torch.float32, device=self._device)
        self._lam_p = torch.zeros(self.max_particles, dtype=torch.float32, device=self._device)
        self._mu_p[:count] = torch.from_numpy(mu.astype(np.float32))
        self._lam_p[:count] = torch.from_numpy(lam.astype(np.float32))
        self._parts.mu = self._mu_p.data_ptr()
        self._parts.lam = self._lam_p.data_ptr()

    def _make_particles(self) -> nat.Particles:
        p = nat.Particles()
        p.x = self._x.data_ptr()
        p.v = self._v.data_ptr()
        p.C = self._C.data_ptr()
        p.F = self._F.data_ptr()
        p.mass = self._mass.data_ptr()
        p.volume = self._volume.data_ptr()
        p.active = self._active.data_ptr()
        p.force = self._force.data_ptr()
        p.capacity = self.max_particles
        return p

    def initialize_particles_box(self, lower, upper, spacing=None,
                                 initial_velocity=(0.0, 0.0, 0.0)) -> int:
        """Regular lattice of particles in [lower, upper) (mpm3d.py:69-96)."""
        lo = self._validate_vec3(lower, "lower")
        hi = self._validate_vec3(upper, "upper")
        if np.any(hi <= lo):
            raise ValueError("upper must be greater than lower in every dimension.")
        sp = self._default_spacing() if spacing is None else self._validate_spacing(spacing)
        axes = [np.arange(lo[a], hi[a], sp[a]) for a in range(3)]
        if any(len(ax) == 0 for ax in axes):
            raise ValueError("particle box produced no particles.")
        grid = np.meshgrid(*axes, indexing="ij")
        positions = np.stack([g.ravel() for g in grid], axis=1).astype(np.float32)
        vel = np.broadcast_to(self._validate_vec3(initial_velocity, "initial_velocity"),
                              positions.shape).astype(np.float32)
        return self.initialize_particles_from_numpy(positions, velocities=vel,
                                                    particle_volume=float(np.prod(sp)))

    def initialize_particles_from_numpy(self, positions, velocities=None, particle_mass=None,
                                        particle_volume=None, youngs_modulus=None,
                                        poisson_ratio=None) -> int:
        """Load particles; F = I, C = 0, active = 1 (mpm3d.py:98-165).

        ``youngs_modulus`` / ``poisson_ratio`` (scalar or one value per particle) are an
        extension: per-particle materials, e.g. bodies of different stiffness in one solver.
        When both are None the configuration's single material applies, as in the reference.
        """
        pos = np.asarray(positions, dtype=np.float32)
        if pos.ndim != 2 or pos.shape[1] != 3:
            raise ValueError("positions must have shape (n, 3).")
        count = int(pos.shape[0])
        if count <= 0:
            raise ValueError("positions must contain at least one particle.")
        if count > self.max_particles:
            raise ValueError(f"particle count {count} exceeds max_particles={self.max_particles}.")
        if velocities is None:
            vel = np.zeros((count, 3), dtype=np.float32)
        else:
            vel = np.asarray(velocities, dtype=np.float32)
            if vel.shape != (count, 3):
                raise ValueError(f"velocities must have shape {(count, 3)}, got {vel.shape}.")
        mass, volume = particle_mass_volume(self.config, particle_mass, particle_volume)

        for t in (self._x, self._v, self._C, self._F, self._mass, self._volume, self._active,
                  self._force):
            t.zero_()
        self._x[:, :count].copy_(torch.from_numpy(np.ascontiguousarray(pos.T)))
        self._v[:, :count].copy_(torch.from_numpy(np.ascontiguousarray(vel.T)))
        self._F[0, :count] = 1.0
        self._F[4, :count] = 1.0
        self._F[8, :count] = 1.0
        self._mass[:count] = float(np.float32(mass))
        self._volume[:count] = float(np.float32(volume))
        self._active[:count] = 1
        self._set_particle_materials(count, youngs_modulus, poisson_ratio)
        self._num_particles = count
        self._desc.num_particles = count
        self._initialized = True
        return count

    def _default_spacing(self) -> np.ndarray:
        return np.full(3, self.dx / float(self.config.particles_per_cell), dtype=np.float32)

    @staticmethod
    def _validate_vec3(values, name: str) -> np.ndarray:
        arr = np.asarray(values, dtype=np.float32)
        if arr.shape != (3,):
            raise ValueError(f"{name} must have 3 components.")
        return arr

    @staticmethod
    def _validate_spacing(spacing) -> np.ndarray:
        arr = (np.full(3, float(spacing), dtype=np.float32) if np.isscalar(spacing)
               else np.asarray(spacing, dtype=np.float32))
        if arr.shape != (3,):
            raise ValueError("spacing must be a scalar or have 3 components.")
        if np.any(arr <= 0.0):
            raise ValueError("spacing must be positive.")
        return arr

    # ----------------------------------------------------------------- step
    def substep(self, dt: float | None = None) -> None:
        if not self._initialized:
            raise RuntimeError(
                "MPMSolver3D.initialize_particles_box or initialize_particles_from_numpy "
                "must be called before substep()."
            )
        dt_value = self.dt_default if dt is None else float(dt)
        if dt_value <= 0.0:
            raise ValueError("dt must be positive.")
        self._desc.dt = float(np.float32(dt_value))
        if self.sorted:
            nat.call("fsi_mpm_substep_sorted", self._desc, self._parts, nat.ptr(self._grid),
                     nat.ptr(self._work), self._work.numel(), nat.stream_ptr())
        else:
            nat.call("fsi_mpm_substep", self._desc, self._parts, nat.ptr(self._grid),
                     nat.ptr(self._dirty), nat.stream_ptr())

    def clear_particle_force(self) -> None:
        self._force[:, : self._num_particles].zero_()

    # ------------------------------------------------------------ accessors
    def particle_count(self) -> int:
        return int(self._num_particles)

    def _rows(self, t: torch.Tensor, width: int) -> np.ndarray:
        n = self._num_particles
        return t[:, :n].t().reshape(n, width).cpu().numpy().copy()

    def positions_numpy(self) -> np.ndarray:
        return self._rows(self._x, 3)

    def velocities_numpy(self) -> np.ndarray:
        return self._rows(self._v, 3)

    def particle_forces_numpy(self) -> np.ndarray:
        return self._rows(self._force, 3)

    def deformation_gradients_numpy(self) -> np.ndarray:
        return self._rows(self._F, 9).reshape(-1, 3, 3)

    def affine_velocities_numpy(self) -> np.ndarray:
        """APIC affine matrices C as (n, 3, 3) (the reference's C field, mpm3d.py:50)."""
        return self._rows(self._C, 9).reshape(-1, 3, 3)

    def active_numpy(self) -> np.ndarray:
        return self._active[: self._num_particles].cpu().numpy().copy()

    def base_cells_numpy(self) -> np.ndarray:
        """Particle-to-cell indices trunc(x / dx - 0.5) as int32 (n, 3) (mpm3d.py:239)."""
        n = self._num_particles
        out = torch.zeros((max(n, 1), 3), dtype=torch.int32, device=self._device)
        nat.call("fsi_mpm_base_cells", self._desc, self._parts, nat.ptr(out), nat.stream_ptr())
        return out[:n].cpu().numpy()

    def _reduce(self) -> np.ndarray:
        nat.call("fsi_mpm_reduce", self._desc, self._parts, nat.ptr(self._diag), None,
                 nat.stream_ptr())
        self._diag_host.copy_(self._diag, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return self._diag_host.numpy().copy()

    def center_of_mass(self) -> np.ndarray:
        """Mass-weighted mean position with the reference's float32 numpy arithmetic
        (mpm3d.py:353-362); the committed goldens depend on its rounding."""
        n = self._num_particles
        if n == 0:
            return np.zeros(3, dtype=np.float32)
        positions = self.positions_numpy()
        masses = self._mass[:n].cpu().numpy()
        total = masses.sum()
        if total <= 0.0:
            return np.zeros(3, dtype=np.float32)
        return (positions * masses[:, None]).sum(axis=0) / total

    def center_of_mass_device(self) -> np.ndarray:
        """Centre of mass from an on-device float64 reduction (no particle copy to the host)."""
        r = self._reduce()
        if self._num_particles == 0 or r[0] <= 0.0:
            return np.zeros(3, dtype=np.float64)
        return r[1:4] / r[0]

    def max_velocity_norm(self) -> float:
        if self._num_particles == 0:
            return 0.0
        return float(self._reduce()[4])

    def total_particle_force(self) -> np.ndarray:
        return self._reduce()[5:8].astype(np.float32)

    # ------------------------------------------------------- checkpointing
    _STATE = ("_x", "_v", "_C", "_F", "_mass", "_volume", "_active", "_force")

    def state_dict(self) -> dict:
        """Complete particle state (device tensors cloned; no reference counterpart)."""
        state = {name: getattr(self, name).clone() for name in self._STATE}
        state.update(kind="MPMSolver3D", capacity=self.max_particles,
                     num_particles=self._num_particles, initialized=self._initialized,
                     mu=None if self._mu_p is None else self._mu_p.clone(),
                     lam=None if self._lam_p is None else self._lam_p.clone())
        return state

    def load_state_dict(self, state: dict) -> None:
        if state.get("kind") != "MPMSolver3D" or int(state["capacity"]) != self.max_particles:
            raise ValueError("checkpoint does not match this particle capacity")
        for name in self._STATE:
            getattr(self, name).copy_(state[name])
        if state.get("mu") is None:
            self._mu_p = self._lam_p = None
            self._parts.mu = self._parts.lam = None
        else:
            self._mu_p, self._lam_p = state["mu"].clone(), state["lam"].clone()
            self._parts.mu, self._parts.lam = self._mu_p.data_ptr(), self._lam_p.data_ptr()
        self._num_particles = int(state["num_particles"])
        self._desc.num_particles = self._num_particles
        self._initialized = bool(state["initialized"])

    # ---------------------------------------------------- device tensors
    @property
    def particles(self) -> nat.Particles:
        return self._parts

    @property
    def desc(self) -> nat.MpmDesc:
        return self._desc
