"""Configuration dataclasses for the coupled LBM-MPM solver.

Field names, defaults and validation errors follow the reference's
``fsi/config.py:20-259`` so that existing configurations and their tests work
unchanged. The ``backend`` literal is accepted for compatibility; this
implementation always runs on the current CUDA device.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from pathlib import Path
from typing import Literal

Backend = Literal["cpu", "gpu", "cuda", "vulkan"]
BoundaryType = Literal["periodic", "pressure", "velocity", "wall"]
CouplingKernel = Literal["quadratic"]
OutputFormat = Literal["npz", "vtk", "both"]

_BACKENDS = frozenset({"cpu", "gpu", "cuda", "vulkan"})
_BOUNDARY_TYPES = frozenset({"periodic", "pressure", "velocity", "wall"})
_COUPLING_KERNELS = frozenset({"quadratic"})
_OUTPUT_FORMATS = frozenset({"npz", "vtk", "both"})
_MATERIALS = frozenset({"elastic"})
_FREE_MRT_MOMENTS = frozenset({1, 2, 4, 6, 8, 10, 12, 16, 17, 18})


def _check_vec3(values, message: str) -> None:
    if len(values) != 3:
        raise ValueError(message)


def _check_grid(kind: str, nx: int, ny: int, nz: int) -> None:
    if min(nx, ny, nz) <= 4:
        raise ValueError(
            f"{kind} grid is too small: {(nx, ny, nz)}. Each dimension should be greater than 4."
        )


@dataclass(frozen=True)
class BoundaryConfig:
    """Boundary condition for one face of the fluid lattice (config.py:20-34)."""

    boundary_type: BoundaryType = "periodic"
    rho: float = 1.0
    velocity: tuple[float, float, float] = (0.0, 0.0, 0.0)

    # Extension (velocity faces): "sequential" is the reference's update, in place in q order
    # (lbm3d.py:375-383), so one member of each opposite pair reads its partner's new value;
    # "simultaneous" reads every population from before the update. On an inflow/outflow
    # channel at tau 0.55 the sequential form grows without bound after a few hundred steps.
    velocity_update: str = "sequential"

    def validate(self) -> None:
        if self.boundary_type not in _BOUNDARY_TYPES:
            raise ValueError(f"Unsupported boundary type: {self.boundary_type}.")
        if self.rho <= 0.0:
            raise ValueError(f"Boundary rho must be positive, got {self.rho}.")
        _check_vec3(self.velocity, "Boundary velocity must have 3 components.")
        if self.velocity_update not in ("sequential", "simultaneous"):
            raise ValueError(f"Unsupported velocity_update: {self.velocity_update}.")


@dataclass(frozen=True)
class LBMConfig:
    """D3Q19 MRT fluid lattice configuration (config.py:37-83)."""

    nx: int = 64
    ny: int = 32
    nz: int = 16

    viscosity: float = 0.1
    rho0: float = 1.0

    force: tuple[float, float, float] = (0.0, 0.0, 0.0)
    initial_velocity: tuple[float, float, float] = (0.0, 0.0, 0.0)

    x_left: BoundaryConfig = field(default_factory=lambda: BoundaryConfig("velocity"))
    x_right: BoundaryConfig = field(default_factory=lambda: BoundaryConfig("pressure"))
    y_left: BoundaryConfig = field(default_factory=BoundaryConfig)
    y_right: BoundaryConfig = field(default_factory=BoundaryConfig)
    z_left: BoundaryConfig = field(default_factory=BoundaryConfig)
    z_right: BoundaryConfig = field(default_factory=BoundaryConfig)

    use_sparse: bool = False

    # Extensions (no reference counterpart; the reference stores and computes float32 in
    # its own operation order, lbm3d.py:117-122, 276-333).
    # population_storage: "f32" populations, or "f16" / "bf16" deviations from the rest
    #   equilibrium f_q - w_q rho0 (half the memory traffic, float32 arithmetic).
    # collision_arithmetic: "exact" (the reference's float32 operations, bit-identical),
    #   "fast" (the same operator, fused and parity-split), or "auto" = "exact" for f32
    #   storage and "fast" otherwise.
    # mrt_rates: {moment index: rate} overriding the default relaxation rates S_k for the
    #   non-conserved moments k in {1, 2, 4, 6, 8, 10, 12, 16, 17, 18}; the shear rates
    #   (9, 11, 13, 14, 15) always follow from the viscosity.
    population_storage: Literal["f32", "f16", "bf16"] = "f32"
    collision_arithmetic: Literal["auto", "exact", "fast"] = "auto"
    mrt_rates: dict | None = None

    def resolved_arithmetic(self) -> str:
        if self.collision_arithmetic != "auto":
            return self.collision_arithmetic
        return "exact" if self.population_storage == "f32" else "fast"

    def validate(self) -> None:
        if self.population_storage not in ("f32", "f16", "bf16"):
            raise ValueError(f"Unsupported population storage: {self.population_storage}.")
        if self.collision_arithmetic not in ("auto", "exact", "fast"):
            raise ValueError(f"Unsupported collision arithmetic: {self.collision_arithmetic}.")
        if self.population_storage != "f32" and self.collision_arithmetic == "exact":
            raise ValueError("f16/bf16 population storage uses the fast collision arithmetic.")
        if self.mrt_rates is not None:
            for k, rate in dict(self.mrt_rates).items():
                if int(k) not in _FREE_MRT_MOMENTS:
                    raise ValueError(f"MRT moment {k} has no free relaxation rate.")
                if not (0.0 < float(rate) < 2.0):
                    raise ValueError(f"MRT rate for moment {k} must be in (0, 2), got {rate}.")
        _check_grid("LBM", self.nx, self.ny, self.nz)
        if self.viscosity <= 0.0:
            raise ValueError(f"LBM viscosity must be positive, got {self.viscosity}.")
        if self.rho0 <= 0.0:
            raise ValueError(f"LBM rho0 must be positive, got {self.rho0}.")
        _check_vec3(self.force, "LBM force must have 3 components.")
        _check_vec3(self.initial_velocity, "LBM initial_velocity must have 3 components.")
        for face in (self.x_left, self.x_right, self.y_left, self.y_right, self.z_left,
                     self.z_right):
            face.validate()


@dataclass(frozen=True)
class MPMConfig:
    """MLS-MPM solid configuration (config.py:86-138)."""

    nx: int = 64
    ny: int = 32
    nz: int = 16

    max_particles: int = 200_000
    particles_per_cell: int = 2

    dx: float = 1.0
    dt: float = 0.25

    density: float = 1.0
    youngs_modulus: float = 1_000.0
    poisson_ratio: float = 0.25

    gravity: tuple[float, float, float] = (0.0, -9.8e-4, 0.0)

    apic: bool = True
    material: Literal["elastic"] = "elastic"
    boundary_width: int = 3
    boundary_damping: float = 0.0

    # Extension (no reference counterpart): the elastic model. The reference's solver is
    # fixed-corotated (mpm3d.py:247-251); "neo_hookean" selects mu (F F^T - I) + lam ln(J) I.
    constitutive_model: Literal["fixed_corotated", "neo_hookean"] = "fixed_corotated"
    # Extension (no reference counterpart): how P2G sums the grid. "atomic" (default, the
    # faster on coupled steps) scatters through shared-memory tiles with atomics, so sums
    # arrive in scheduling order like the reference's parallel loop; "sorted" sorts the
    # particles by cell each substep and adds every node's contributions in one fixed order
    # (atomic-free, bit-reproducible from run to run).
    p2g_mode: Literal["sorted", "atomic"] = "atomic"

    def validate(self) -> None:
        _check_grid("MPM", self.nx, self.ny, self.nz)
        if self.max_particles <= 0:
            raise ValueError("max_particles must be positive.")
        if self.particles_per_cell <= 0:
            raise ValueError("particles_per_cell must be positive.")
        if self.dx <= 0.0:
            raise ValueError("MPM dx must be positive.")
        if self.dt <= 0.0:
            raise ValueError("MPM dt must be positive.")
        if self.density <= 0.0:
            raise ValueError("MPM density must be positive.")
        if self.youngs_modulus <= 0.0:
            raise ValueError("Young's modulus must be positive.")
        if not (-1.0 < self.poisson_ratio < 0.5):
            raise ValueError(f"Poisson ratio must be in (-1, 0.5), got {self.poisson_ratio}.")
        _check_vec3(self.gravity, "MPM gravity must have 3 components.")
        if self.material not in _MATERIALS:
            raise ValueError(f"Unsupported MPM material: {self.material}.")
        if self.boundary_width < 1:
            raise ValueError("boundary_width must be at least 1.")
        if not (0.0 <= self.boundary_damping <= 1.0):
            raise ValueError("boundary_damping must be in [0, 1].")
        if self.constitutive_model not in _CONSTITUTIVE_MODELS:
            raise ValueError(f"Unsupported constitutive model: {self.constitutive_model}.")
        if self.p2g_mode not in ("sorted", "atomic"):
            raise ValueError(f"Unsupported p2g_mode: {self.p2g_mode}.")


_CONSTITUTIVE_MODELS = frozenset({"fixed_corotated", "neo_hookean"})


@dataclass(frozen=True)
class CouplingConfig:
    """Penalty / immersed-boundary / contact coupling options (config.py:141-196).

    The penalty force on a particle is ``F_p = gamma * m_p * (u_fluid - v_p)``.
    """

    enabled: bool = True
    gamma: float = 0.05
    mpm_substeps_per_lbm_step: int = 4
    kernel: CouplingKernel = "quadratic"

    build_solid_volume_fraction: bool = True
    force_limit: float | None = None
    relative_velocity_limit: float | None = None
    gamma_ramp_steps: int = 0
    min_valid_weight: float = 1.0e-6
    immersed_boundary_enabled: bool = False
    immersed_boundary_drag: float = 0.0
    immersed_boundary_fraction_threshold: float = 0.1
    immersed_boundary_max_force: float | None = None
    contact_enabled: bool = False
    contact_velocity_damping: float = 0.0
    contact_fraction_threshold: float = 0.5

    def validate(self) -> None:
        if self.gamma < 0.0:
            raise ValueError(f"Coupling gamma must be non-negative, got {self.gamma}.")
        if self.mpm_substeps_per_lbm_step <= 0:
            raise ValueError("mpm_substeps_per_lbm_step must be positive.")
        if self.kernel not in _COUPLING_KERNELS:
            raise ValueError(f"Unsupported coupling kernel: {self.kernel}.")
        if self.force_limit is not None and self.force_limit <= 0.0:
            raise ValueError("force_limit must be positive when provided.")
        if self.relative_velocity_limit is not None and self.relative_velocity_limit <= 0.0:
            raise ValueError("relative_velocity_limit must be positive when provided.")
        if self.gamma_ramp_steps < 0:
            raise ValueError("gamma_ramp_steps must be non-negative.")
        if self.min_valid_weight <= 0.0:
            raise ValueError("min_valid_weight must be positive.")
        if self.min_valid_weight > 1.0:
            raise ValueError("min_valid_weight must not exceed 1.")
        if self.immersed_boundary_drag < 0.0:
            raise ValueError("immersed_boundary_drag must be non-negative.")
        if not (0.0 <= self.immersed_boundary_fraction_threshold <= 1.0):
            raise ValueError("immersed_boundary_fraction_threshold must be in [0, 1].")
        if self.immersed_boundary_max_force is not None and self.immersed_boundary_max_force <= 0.0:
            raise ValueError("immersed_boundary_max_force must be positive when provided.")
        if not (0.0 <= self.contact_velocity_damping <= 1.0):
            raise ValueError("contact_velocity_damping must be in [0, 1].")
        if not (0.0 <= self.contact_fraction_threshold <= 1.0):
            raise ValueError("contact_fraction_threshold must be in [0, 1].")


@dataclass(frozen=True)
class OutputConfig:
    """Snapshot output options (config.py:199-215)."""

    output_dir: Path = Path("outputs")
    output_interval: int = 100
    output_format: OutputFormat = "npz"

    write_lbm_fields: bool = True
    write_mpm_particles: bool = True
    write_coupling_fields: bool = True

    # Extension: compress and write NPZ snapshots on a background thread (the fields are
    # copied to the host synchronously; FSISimulation.run waits for the writes before it
    # returns). The reference writes synchronously.
    async_write: bool = False

    def validate(self) -> None:
        if self.output_interval <= 0:
            raise ValueError("output_interval must be positive.")
        if self.output_format not in _OUTPUT_FORMATS:
            raise ValueError(f"Unsupported output format: {self.output_format}.")


@dataclass(frozen=True)
class SimulationConfig:
    """Top-level configuration of a coupled run (config.py:218-259)."""

    backend: Backend = "cpu"
    random_seed: int = 0

    num_steps: int = 1000
    lbm_dt: float = 1.0

    lbm: LBMConfig = field(default_factory=LBMConfig)
    mpm: MPMConfig = field(default_factory=MPMConfig)
    coupling: CouplingConfig = field(default_factory=CouplingConfig)
    output: OutputConfig = field(default_factory=OutputConfig)

    def validate(self) -> None:
        if self.backend not in _BACKENDS:
            raise ValueError(f"Unsupported backend: {self.backend}.")
        if self.num_steps <= 0:
            raise ValueError("num_steps must be positive.")
        if self.lbm_dt <= 0.0:
            raise ValueError("lbm_dt must be positive.")
        self.lbm.validate()
        self.mpm.validate()
        self.coupling.validate()
        self.output.validate()
        lbm_shape = (self.lbm.nx, self.lbm.ny, self.lbm.nz)
        mpm_shape = (self.mpm.nx, self.mpm.ny, self.mpm.nz)
        if lbm_shape != mpm_shape:
            raise ValueError(
                "For MVP, LBM and MPM grids must have the same resolution. "
                f"Got LBM={lbm_shape}, MPM={mpm_shape}."
            )

    @property
    def mpm_dt(self) -> float:
        return self.lbm_dt / float(self.coupling.mpm_substeps_per_lbm_step)
