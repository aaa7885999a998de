"""Top-level coupled runner (drop-in for the reference's fsi/simulation.py:12-153)."""
from __future__ import annotations

import numpy as np

from .config import SimulationConfig
from .coupling import LBMMpmCoupler
from .lbm3d import LBMSolver3D
from .mpm3d import MPMSolver3D
from .output import SimulationOutputWriter


class FSISimulation:
    """Explicit LBM-MPM coupled simulation: builds the solvers, steps, reports diagnostics."""

    def __init__(self, config: SimulationConfig):
        self.config = config
        self.config.validate()
        self.lbm = LBMSolver3D(config.lbm)
        self.mpm = MPMSolver3D(config.mpm)
        self.coupler = LBMMpmCoupler(config.coupling, self.lbm, self.mpm)
        self.output_writer = SimulationOutputWriter(config.output)
        self.step_index = 0
        self.time = 0.0
        self._lbm_initialized = False
        self._mpm_initialized = False

    def initialize_lbm(self, solid_np: np.ndarray | None = None) -> None:
        self.lbm.initialize(solid_np=solid_np)
        self._lbm_initialized = True

    def initialize_mpm_box(self, lower, upper, spacing=None,
                           initial_velocity=(0.0, 0.0, 0.0)) -> int:
        count = self.mpm.initialize_particles_box(lower=lower, upper=upper, spacing=spacing,
                                                  initial_velocity=initial_velocity)
        self._mpm_initialized = True
        return count

    def initialize_mpm_from_numpy(self, positions, velocities=None, particle_mass=None,
                                  particle_volume=None, youngs_modulus=None,
                                  poisson_ratio=None) -> int:
        """Load particles (simulation.py:51-59); ``youngs_modulus`` / ``poisson_ratio`` per
        particle are the MPMSolver3D extension for bodies of different stiffness."""
        count = self.mpm.initialize_particles_from_numpy(
            positions=positions, velocities=velocities, particle_mass=particle_mass,
            particle_volume=particle_volume, youngs_modulus=youngs_modulus,
            poisson_ratio=poisson_ratio)
        self._mpm_initialized = True
        return count

    def initialize(self, solid_np=None, mpm_box_lower=None, mpm_box_upper=None,
                   mpm_box_spacing=None, mpm_initial_velocity=(0.0, 0.0, 0.0)) -> int:
        if mpm_box_lower is None or mpm_box_upper is None:
            raise ValueError("mpm_box_lower and mpm_box_upper are required.")
        self.initialize_lbm(solid_np=solid_np)
        return self.initialize_mpm_box(lower=mpm_box_lower, upper=mpm_box_upper,
                                       spacing=mpm_box_spacing,
                                       initial_velocity=mpm_initial_velocity)

    def step(self) -> dict[str, object]:
        self._validate_initialized()
        self.coupler.step(self.config.lbm_dt)
        self.step_index += 1
        self.time += self.config.lbm_dt
        return self.diagnostics()

    def run(self, steps: int | None = None, write_output: bool = False,
            write_initial: bool = False) -> list[dict[str, object]]:
        self._validate_initialized()
        count = self.config.num_steps if steps is None else int(steps)
        if count <= 0:
            raise ValueError("steps must be positive.")
        history = []
        if write_output and write_initial:
            self.write_snapshot()
        for _ in range(count):
            history.append(self.step())
            if write_output and self.output_writer.should_write(self.step_index):
                self.write_snapshot()
        self.output_writer.flush()
        return history

    def advance(self, steps: int, graph: bool = True) -> None:
        """``steps`` coupled steps without per-step diagnostics (no reference counterpart):
        LBMMpmCoupler.step_many, with the step counter and time advanced as by step()."""
        self._validate_initialized()
        count = int(steps)
        if count <= 0:
            raise ValueError("steps must be positive.")
        self.coupler.step_many(self.config.lbm_dt, count, graph=graph)
        for _ in range(count):
            self.step_index += 1
            self.time += self.config.lbm_dt

    def write_snapshot(self):
        self._validate_initialized()
        return self.output_writer.write_snapshot(self)

    def diagnostics(self) -> dict[str, object]:
        """Per-step diagnostics with the reference's keys (simulation.py:117-147)."""
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

    # ------------------------------------------------------- checkpointing
    def state_dict(self) -> dict:
        """Full coupled state for restart (the reference writes snapshots but cannot resume)."""
        return {"kind": "FSISimulation", "step_index": self.step_index, "time": self.time,
                "lbm_initialized": self._lbm_initialized, "mpm_initialized": self._mpm_initialized,
                "lbm": self.lbm.state_dict(), "mpm": self.mpm.state_dict(),
                "coupler": self.coupler.state_dict()}

    def load_state_dict(self, state: dict) -> None:
        if state.get("kind") != "FSISimulation":
            raise ValueError("not a simulation checkpoint")
        self.lbm.load_state_dict(state["lbm"])
        self.mpm.load_state_dict(state["mpm"])
        self.coupler.load_state_dict(state["coupler"])
        self.step_index = int(state["step_index"])
        self.time = float(state["time"])
        self._lbm_initialized = bool(state["lbm_initialized"])
        self._mpm_initialized = bool(state["mpm_initialized"])

    def save_checkpoint(self, path) -> None:
        """Write the full state with torch.save (device tensors are stored as CPU tensors)."""
        import torch

        def to_cpu(v):
            if isinstance(v, torch.Tensor):
                return v.detach().cpu()
            if isinstance(v, dict):
                return {k: to_cpu(x) for k, x in v.items()}
            if isinstance(v, list):
                return [to_cpu(x) for x in v]
            return v

        torch.save(to_cpu(self.state_dict()), path)

    def load_checkpoint(self, path) -> None:
        import torch

        self.load_state_dict(torch.load(path, map_location="cpu", weights_only=False))

    def _validate_initialized(self) -> None:
        if not self._lbm_initialized or not getattr(self.lbm, "_initialized", False):
            raise RuntimeError("FSISimulation.initialize_lbm must be called before stepping.")
        if not self._mpm_initialized or not getattr(self.mpm, "_initialized", False):
            raise RuntimeError("FSISimulation MPM initialization must be called before stepping.")
