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
        self._dbuf = None
        self._diag_fused = False
        self._dhost = None
        # step() replays a captured CUDA graph of (coupled step + diagnostics) once the state
        # repeats with period two (no reference counterpart; set False for eager steps)
        self.graph_steps = True
        self._graphs = {}

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

    def step(self, body_force=None) -> dict[str, object]:
        """One coupled step and its diagnostics (simulation.py:84-89). ``body_force`` is the
        extension of LBMMpmCoupler.step: this step's lattice driving force (3 components).

        With ``graph_steps`` (default), once the solvers' state repeats with period two (the
        lattice's AA parity and force buffers, a settled gamma ramp, rho / u refreshed by the
        last diagnostics), the step and its diagnostics run as the replay of one of two
        captured CUDA graphs, the driving force read from a device buffer filled from pinned
        host memory; the kernels and their arguments are those of the eager step."""
        self._validate_initialized()
        if body_force is not None and np.asarray(body_force).shape != (3,):
            raise ValueError("body_force must have 3 components.")
        if self.graph_steps and self._graph_ready():
            return self._graph_step(body_force)
        self.coupler.step(self.config.lbm_dt, body_force=body_force)
        self.step_index += 1
        self.time += self.config.lbm_dt
        return self.diagnostics()

    # ------------------------------------------------------ graph stepping
    def _graph_ready(self) -> bool:
        lbm, c = self.lbm, self.coupler
        return (lbm._macro_fresh and lbm._fcur == lbm._fprev and lbm._fcur >= 0
                and c._gamma_settled() and self._dbuf is not None)

    def _graph_key(self) -> tuple:
        """What a captured step bakes in: lattice parity and force buffer, particle count and
        arrays (re-initialised particles may live elsewhere), launch tuning, gamma, state
        buffers."""
        lbm, m = self.lbm, self.mpm
        d = m.desc
        c = self.coupler
        parts = m.particles
        arrays = tuple(int(getattr(parts, f) or 0) for f, _ in parts._fields_)
        return (lbm._steps_done % 2, lbm._fcur, m.particle_count(), d.launch_threads,
                d.coupling_fold, lbm._pops.data_ptr(), m._grid.data_ptr(), c._accum.data_ptr(),
                float(c._gamma_for_kernel()), c._ib_written, arrays)

    def _graph_step(self, body_force) -> dict[str, object]:
        import torch

        lbm, c = self.lbm, self.coupler
        if not hasattr(self, "_base_pin"):
            self._base_pin = torch.zeros(3, dtype=torch.float32).pin_memory()
            self._base_dev = torch.zeros(3, dtype=torch.float32, device=self._dbuf.device)
        force = self.lbm.config.force if body_force is None else body_force
        self._base_pin.numpy()[:] = np.asarray(force, dtype=np.float32)
        key = self._graph_key()
        entry = self._graphs.get(key)
        if entry is None:
            if len(self._graphs) >= 4:
                self._graphs.clear()
            g = torch.cuda.CUDAGraph()
            c._device_base = self._base_dev
            steps0, coupled0 = lbm._steps_done, c._coupled_step
            try:
                with torch.cuda.graph(g):
                    # capture records the work without running it; the host-side counters
                    # advance here, and the replay below performs it
                    self._base_dev.copy_(self._base_pin, non_blocking=True)
                    c.step(self.config.lbm_dt)
                    self._diag_enqueue()
            finally:
                c._device_base = None
            entry = (g, lbm._fcur, lbm._fprev, self._diag_fused)
            self._graphs[key] = entry
            lbm._steps_done, c._coupled_step = steps0, coupled0
        g, fcur, fprev, self._diag_fused = entry
        g.replay()
        lbm._steps_done += 1
        lbm._fcur, lbm._fprev = fcur, fprev
        lbm._macro_fresh = True
        lbm._mass_speed_cache = None
        c._coupled_step += 1
        if c.immersed_boundary_enabled:
            c._ib_written = True
        c._reaction_fresh = True
        self.step_index += 1
        self.time += self.config.lbm_dt
        return self._diag_finish(None)

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
        """Per-step diagnostics with the reference's keys (simulation.py:117-147).

        All reductions run on the device (float64 sums of the float32 fields): the lattice's
        fused macro refresh + mass / max |u| pass and one launch for the particles and the
        counters, followed by a single 264-byte copy to pinned host memory and one
        synchronisation. The fluid reaction is summed by the step's force assembly in the same
        pass over the accumulator (after the first step), else by the particle launch. The reference copies every field to the host instead; its
        centre of mass is a float32 numpy sum, here the float64 quotient rounded to float32
        (MPMSolver3D.center_of_mass() keeps the float32 host arithmetic)."""
        self._validate_initialized()
        return self._diag_finish(self._diag_enqueue())

    def _diag_enqueue(self):
        """Enqueue the device reductions and the copy of their record to pinned host memory;
        returns the lattice's cached (mass, max |u|) of this state, or None."""
        import torch

        from . import _native as nat

        c = self.coupler
        if self._dbuf is None:
            dev = self.lbm.macro.device
            # [0:8] lattice, [8:30] particles / reaction / counters, [30:33] the fluid
            # reaction that the coupler's assembly sums from here on
            self._dbuf = torch.zeros(33, dtype=torch.float64, device=dev)
            self._dhost = torch.zeros(33, dtype=torch.float64).pin_memory()
            c._reaction_out = self._dbuf[30:33]
        cached = self.lbm._enqueue_mass_speed(self._dbuf[0:8])
        # the fluid reaction comes from the last assembly when it read the accumulator as it
        # is now; otherwise the diagnostics pass reads the accumulator again
        self._diag_fused = c._reaction_out is not None and c._reaction_fresh
        nat.call("fsi_coupled_diagnostics", self.mpm.desc, self.mpm.particles, self.lbm._desc,
                 nat.ptr(None if self._diag_fused else c._accum), nat.ptr(self.lbm.flags),
                 nat.ptr(c._counters), nat.ptr(self._dbuf[8:30]), nat.stream_ptr())
        self._dhost.copy_(self._dbuf, non_blocking=True)
        return cached

    def _diag_finish(self, cached) -> dict[str, object]:
        """Wait for the enqueued record and build the reference's diagnostics dict."""
        import torch

        c = self.coupler
        torch.cuda.current_stream().synchronize()
        r = self._dhost.numpy().copy()
        if cached is None:
            mass, speed = float(r[0]), float(r[1])
            self.lbm._remember_mass_speed(mass, speed)
        else:
            mass, speed = cached
        d = r[8:30]
        reaction = r[30:33] if self._diag_fused else d[8:11]
        n = self.mpm.particle_count()
        com = (d[1:4] / d[0]).astype(np.float32) if n and d[0] > 0.0 else np.zeros(3, np.float32)
        counts = d[11:19].astype(np.int64)
        ib_total = d[19:22].astype(np.float32).astype(np.float64)
        return {
            "step": self.step_index,
            "time": self.time,
            "lbm_total_mass": mass,
            "lbm_max_velocity_norm": speed,
            "mpm_particle_count": n,
            "mpm_center_of_mass": com,
            "mpm_max_velocity_norm": float(d[4]) if n else 0.0,
            "total_particle_coupling_force": d[5:8].astype(np.float32),
            "total_fluid_coupling_force": reaction.astype(np.float32),
            "coupling_unsupported_particle_count": int(counts[0]),
            "coupling_partial_support_particle_count": int(counts[1]),
            "coupling_clipped_particle_count": int(counts[2]),
            "coupling_effective_gamma": c.effective_gamma(),
            "coupling_ib_active_cell_count": int(counts[5]),
            "coupling_ib_clipped_cell_count": int(counts[6]),
            "coupling_ib_total_force_norm": float(np.linalg.norm(ib_total)),
            "coupling_contact_candidate_count": int(counts[3]),
            "coupling_contact_damped_particle_count": int(counts[4]),
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
        self._graphs.clear()
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
