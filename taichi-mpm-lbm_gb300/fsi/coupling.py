"""Explicit penalty LBM-MPM coupling on the GPU (drop-in for the reference's fsi/coupling.py).

Per coupled step the coupler runs ``substeps`` x [penalty coupling kernel, MPM
substep, optional contact kernel] against the fluid velocity of the last
lattice step, then one assembly kernel that clamps the solid fraction and
rebuilds the lattice force (base + coupling reaction + optional immersed
boundary drag), then one lattice step. The fluid reaction force density and
the solid volume fraction share one float4 accumulator per cell; counters
live in a small device struct.

Public methods, accessors, diagnostics keys and exceptions follow
fsi/coupling.py:11-496.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .config import CouplingConfig
from .lbm3d import LBMSolver3D
from .mpm3d import MPMSolver3D

_SUPPORT_TOLERANCE = 1.0e-5


def coupling_descriptor(config: CouplingConfig, dx: float) -> nat.CouplingDesc:
    """The C-ABI descriptor of the coupling parameters (gamma_eff, dt_ratio and
    build_fraction are set per call)."""
    c, d = config, nat.CouplingDesc()
    f32 = lambda v: float(np.float32(v))  # noqa: E731
    d.cell_volume = f32(float(dx) ** 3)
    d.inv_dx = f32(1.0 / float(dx))
    d.min_valid_weight = f32(c.min_valid_weight)
    d.use_rel_limit = int(c.relative_velocity_limit is not None)
    d.rel_limit = f32(c.relative_velocity_limit or 0.0)
    d.use_force_limit = int(c.force_limit is not None)
    d.force_limit = f32(c.force_limit or 0.0)
    d.ib_enabled = int(c.immersed_boundary_enabled)
    d.ib_drag = f32(c.immersed_boundary_drag)
    d.ib_threshold = f32(c.immersed_boundary_fraction_threshold)
    d.ib_use_max = int(c.immersed_boundary_max_force is not None)
    d.ib_max_force = f32(c.immersed_boundary_max_force or 0.0)
    d.contact_enabled = int(c.contact_enabled)
    d.contact_threshold = f32(c.contact_fraction_threshold)
    d.contact_damping = f32(c.contact_velocity_damping)
    return d


def gamma_for_step(config: CouplingConfig, coupled_step: int) -> float:
    """_effective_gamma of coupling.py:321-330, evaluated in float32."""
    g = np.float32(config.gamma)
    ramp = int(config.gamma_ramp_steps)
    if ramp > 0:
        r = (np.float32(coupled_step) + np.float32(1.0)) / np.float32(ramp)
        g = np.float32(g * min(np.float32(1.0), r))
    return float(g)


class LBMMpmCoupler:
    """Explicit partitioned penalty coupling between the LBM and MPM solvers."""

    def __init__(self, config: CouplingConfig, lbm: LBMSolver3D, mpm: MPMSolver3D):
        self.config = config
        self.config.validate()
        self.lbm = lbm
        self.mpm = mpm
        self._validate_solver_contract()
        self.enabled = bool(config.enabled)
        self.build_solid_volume_fraction = bool(config.build_solid_volume_fraction)
        self.immersed_boundary_enabled = bool(config.immersed_boundary_enabled)
        self.contact_enabled = bool(config.contact_enabled)
        self.substeps = int(config.mpm_substeps_per_lbm_step)
        self.nx, self.ny, self.nz = int(lbm.nx), int(lbm.ny), int(lbm.nz)
        self.inv_dx = 1.0 / float(mpm.dx)
        self.cell_volume = float(mpm.dx) ** 3

        dev = nat.device()
        n = self.nx * self.ny * self.nz
        cap = mpm.max_particles
        self._accum = torch.zeros((n, 4), dtype=torch.float32, device=dev)  # reaction xyz, phi
        self._ib = torch.zeros((3, n), dtype=torch.float32, device=dev)
        self._valid = torch.zeros(cap, dtype=torch.float32, device=dev)
        self._mask = torch.zeros(cap, dtype=torch.int32, device=dev)
        self._contact_mask = torch.zeros(cap, dtype=torch.int32, device=dev)
        self._counters = torch.zeros(12, dtype=torch.int32, device=dev)  # fsi_coupling_counters
        self._diag = torch.zeros(4, dtype=torch.float64, device=dev)
        self._coupled_step = 0
        self._ib_written = False
        self._device_base = None  # device float32[3] driving force, when its owner sets it
        # device float64[3]: when its owner sets it, every assembly also writes the sum of the
        # fluid reaction over fluid cells there, read in the same pass over the accumulator;
        # _reaction_fresh says that the sum belongs to the accumulator as it is now
        self._reaction_out = None
        self._reaction_fresh = False
        self._desc = nat.CouplingDesc()
        self._fill_desc()

    def _validate_solver_contract(self) -> None:
        if self.config.kernel != "quadratic":
            raise ValueError(f"Unsupported coupling kernel: {self.config.kernel}.")
        lbm_shape = (self.lbm.nx, self.lbm.ny, self.lbm.nz)
        mpm_shape = (self.mpm.nx, self.mpm.ny, self.mpm.nz)
        if lbm_shape != mpm_shape:
            raise ValueError(
                "LBM and MPM grids must match for Step 5 coupling. "
                f"Got LBM={lbm_shape}, MPM={mpm_shape}."
            )
        if self.mpm.dx <= 0.0:
            raise ValueError("MPM dx must be positive.")

    def _fill_desc(self) -> None:
        self._desc = coupling_descriptor(self.config, self.mpm.dx)

    # ------------------------------------------------------------ stepping
    def _gamma_for_kernel(self) -> float:
        return gamma_for_step(self.config, self._coupled_step)

    def _coupling_kernel(self, dt_ratio: float, build_fraction: bool) -> None:
        self._desc.gamma_eff = self._gamma_for_kernel()
        self._desc.dt_ratio = float(np.float32(dt_ratio))
        self._desc.build_fraction = int(build_fraction)
        self._reaction_fresh = False
        nat.call("fsi_coupling_forces", self._desc, self.mpm.desc, self.mpm.particles,
                 nat.ptr(self.lbm.macro), nat.ptr(self.lbm.flags), nat.ptr(self._accum),
                 nat.ptr(self._valid), nat.ptr(self._mask), nat.ptr(self._counters),
                 nat.stream_ptr())

    def _coupled_substep(self, mpm_dt: float, dt_ratio: float, build_fraction: bool) -> None:
        """Coupling force + MPM substep with the coupling folded into P2G (the sorted or the
        tiled scatter, after the solver's p2g_mode)."""
        self._desc.gamma_eff = self._gamma_for_kernel()
        self._desc.dt_ratio = float(np.float32(dt_ratio))
        self._desc.build_fraction = int(build_fraction)
        self._reaction_fresh = False
        mpm = self.mpm
        mpm.desc.dt = float(np.float32(mpm_dt))
        common = (self._desc, mpm.desc, mpm.particles, nat.ptr(self.lbm.macro),
                  nat.ptr(self.lbm.flags), nat.ptr(self._accum), nat.ptr(self._valid),
                  nat.ptr(self._mask), nat.ptr(self._counters), nat.ptr(mpm._grid))
        if mpm.sorted:
            nat.call("fsi_coupled_substep", *common, nat.ptr(mpm.workspace),
                     mpm.workspace.numel(), nat.stream_ptr())
        else:
            nat.call("fsi_coupled_substep_tiled", *common, nat.ptr(mpm._dirty), nat.stream_ptr())

    def _contact_kernel(self) -> None:
        nat.call("fsi_contact", self._desc, self.mpm.desc, self.mpm.particles,
                 nat.ptr(self._accum), nat.ptr(self.lbm.flags), nat.ptr(self._contact_mask),
                 nat.ptr(self._counters), nat.stream_ptr())

    def _assemble(self, mode: int, force: torch.Tensor | None, body_force=None) -> None:
        if self._device_base is not None:
            # the step's driving force is read on the device (a captured step's value changes
            # between graph replays); its owner fills the buffer before each step
            mode |= nat.ASSEMBLE_BASE_ON_DEVICE
            base_p = nat.ctypes.cast(self._device_base.data_ptr(),
                                     nat.ctypes.POINTER(nat.ctypes.c_float))
        else:
            base = np.asarray(self.lbm.config.force if body_force is None else body_force,
                              dtype=np.float32)
            if base.shape != (3,):
                raise ValueError("body_force must have 3 components.")
            base_p = base.ctypes.data_as(nat.ctypes.POINTER(nat.ctypes.c_float))
        if mode & nat.ASSEMBLE_IB:
            self._counters[5:7].zero_()
            self._counters[8:12].zero_()
            self._ib_written = True
        macro = self.lbm.macro if mode & nat.ASSEMBLE_IB else None
        args = (self._desc, self.lbm._desc, nat.ptr(self.lbm.flags), base_p, mode,
                nat.ptr(self._accum), nat.ptr(macro), nat.ptr(force), nat.ptr(self._ib),
                nat.ptr(self._counters))
        if self._reaction_out is None:
            nat.call("fsi_coupling_assemble", *args, nat.stream_ptr())
        else:
            nat.call("fsi_coupling_assemble_sum", *args, nat.ptr(self._reaction_out),
                     nat.stream_ptr())
            self._reaction_fresh = True

    def step(self, lbm_dt: float, body_force=None) -> None:
        """One explicit coupled lattice step with the configured MPM substeps (coupling.py:135-173).

        ``body_force`` (extension): the lattice's uniform driving force for this step in
        place of ``LBMConfig.force`` (reset_force's base, lbm3d.py:504-510), e.g. a forcing
        schedule supplied by the host step by step."""
        lbm_dt_value = float(lbm_dt)
        if lbm_dt_value <= 0.0:
            raise ValueError("lbm_dt must be positive.")
        if body_force is not None and np.asarray(body_force).shape != (3,):
            raise ValueError("body_force must have 3 components.")
        self._validate_initialized()
        self.clear_coupling_fields()
        mpm_dt = lbm_dt_value / float(self.substeps)
        dt_ratio = mpm_dt / lbm_dt_value
        for substep in range(self.substeps):
            if self.enabled:
                # Coupling force, spread and MPM substep in one pass. clear_particle_diagnostics
                # of coupling.py:147: the pass zeroes the per-substep counters itself, rewrites
                # the weight and mask of every active particle, and inactive particles keep the
                # zeros written by clear_coupling_fields() above.
                self._coupled_substep(mpm_dt, dt_ratio,
                                      substep == 0 and self.build_solid_volume_fraction)
            else:
                self.mpm.clear_particle_force()
                self.mpm.substep(dt=mpm_dt)
            if self.contact_enabled:
                self._contact_kernel()
        mode = 0
        if self.enabled and self.build_solid_volume_fraction:
            mode |= nat.ASSEMBLE_CLAMP_FRACTION
        if self.enabled:
            mode |= nat.ASSEMBLE_COUPLING
        if self.immersed_boundary_enabled:
            mode |= nat.ASSEMBLE_IB
        self._assemble(mode, self.lbm._writable_force(), body_force)
        self.lbm.step()
        if self.enabled:
            self._coupled_step += 1

    # ------------------------------------------------------- graph stepping
    def _graph_state(self) -> tuple:
        lbm = self.lbm
        return (lbm._steps_done % 2, lbm._fcur, lbm._fprev, lbm._macro_fresh)

    def _gamma_settled(self) -> bool:
        ramp = int(self.config.gamma_ramp_steps)
        return ramp <= 0 or not self.enabled or self._coupled_step + 1 >= ramp

    def step_many(self, lbm_dt: float, steps: int, graph: bool = True) -> None:
        """``steps`` calls of step(lbm_dt) (no reference counterpart).

        With ``graph`` the steady part runs as replays of one captured CUDA graph of two
        coupled steps, which removes the per-launch host cost of the ~40 launches of a step.
        Steps during the gamma ramp (whose gamma differs per step) and a last odd step run
        eagerly. The results are those of the eager loop: the graph replays the same kernels
        with the same arguments, and two steps return the lattice to the same buffers and
        parity."""
        steps = int(steps)
        if steps < 0:
            raise ValueError("steps must be non-negative.")
        self._validate_initialized()
        if not graph or steps < 4:
            for _ in range(steps):
                self.step(lbm_dt)
            return
        # The graph bakes gamma_eff and the lattice's buffer choice: settle both eagerly.
        while steps > 0 and (not self._gamma_settled() or self.lbm._macro_fresh
                             or self.lbm._fcur != self.lbm._fprev):
            self.step(lbm_dt)
            steps -= 1
        if steps < 2:
            for _ in range(steps):
                self.step(lbm_dt)
            return
        before = self._graph_state()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            # Capture records the two steps without running them; the host-side counters
            # advance here, and the first replay below performs the work.
            self.step(lbm_dt)
            self.step(lbm_dt)
        g.replay()
        steps -= 2
        if self._graph_state() != before:
            for _ in range(steps):
                self.step(lbm_dt)
            return
        while steps >= 2:
            g.replay()
            self.lbm._steps_done += 2
            if self.enabled:
                self._coupled_step += 2
            steps -= 2
        if steps:
            self.step(lbm_dt)
        del g

    def compute_coupling_forces(self, dt_ratio: float = 1.0) -> None:
        """Particle force and fluid reaction without stepping (coupling.py:175-196)."""
        dt_ratio_value = float(dt_ratio)
        if dt_ratio_value < 0.0:
            raise ValueError("dt_ratio must be non-negative.")
        self._validate_initialized()
        self.clear_coupling_fields()
        self.mpm.clear_particle_force()
        if not self.enabled:
            return
        self._coupling_kernel(dt_ratio_value, self.build_solid_volume_fraction)
        if self.build_solid_volume_fraction:
            self._assemble(nat.ASSEMBLE_CLAMP_FRACTION, None)
        if self.contact_enabled:
            self._contact_kernel()
        if self.immersed_boundary_enabled:
            self._assemble(nat.ASSEMBLE_IB, None)

    def clear_coupling_fields(self) -> None:
        self._accum.zero_()
        self._reaction_fresh = False
        if self._ib_written:  # the IB force field stays zero while nothing writes it
            self._ib.zero_()
            self._ib_written = self.immersed_boundary_enabled
        self._counters.zero_()
        self.clear_particle_diagnostics()

    def clear_particle_diagnostics(self) -> None:
        self._counters[0:5].zero_()
        self._valid.zero_()
        self._mask.zero_()
        self._contact_mask.zero_()

    # ----------------------------------------------------------- accessors
    def _cells(self, t: torch.Tensor) -> np.ndarray:
        return t.reshape(self.nx, self.ny, self.nz, *t.shape[1:]).cpu().numpy()

    def coupling_force_numpy(self) -> np.ndarray:
        return self._cells(self._accum[:, :3])

    def solid_volume_fraction_numpy(self) -> np.ndarray:
        return self._cells(self._accum[:, 3])

    def immersed_boundary_force_numpy(self) -> np.ndarray:
        return self._cells(self._ib.t())

    def _per_particle(self, t: torch.Tensor) -> np.ndarray:
        return t[: self.mpm.particle_count()].cpu().numpy().copy()

    def particle_valid_weights_numpy(self) -> np.ndarray:
        return self._per_particle(self._valid)

    def particle_coupling_mask_numpy(self) -> np.ndarray:
        return self._per_particle(self._mask)

    def particle_contact_mask_numpy(self) -> np.ndarray:
        return self._per_particle(self._contact_mask)

    def total_particle_coupling_force(self) -> np.ndarray:
        return self.mpm.total_particle_force()

    def total_fluid_coupling_force(self) -> np.ndarray:
        nat.call("fsi_coupling_reduce", self.lbm._desc, nat.ptr(self._accum),
                 nat.ptr(self.lbm.flags), nat.ptr(self._diag), nat.stream_ptr())
        return self._diag[:3].cpu().numpy().astype(np.float32)

    def _counter_values(self) -> tuple[np.ndarray, np.ndarray]:
        raw = self._counters.cpu().numpy()
        return raw[:8].copy(), raw[8:12].view(np.float32).copy()

    def immersed_boundary_diagnostics(self) -> dict[str, int | float]:
        counts, totals = self._counter_values()
        t = totals[:3].astype(np.float64)
        return {
            "ib_active_cell_count": int(counts[5]),
            "ib_clipped_cell_count": int(counts[6]),
            "ib_total_force_x": float(t[0]),
            "ib_total_force_y": float(t[1]),
            "ib_total_force_z": float(t[2]),
            "ib_total_force_norm": float(np.linalg.norm(t)),
            "contact_candidate_count": int(counts[3]),
            "contact_damped_particle_count": int(counts[4]),
        }

    def effective_gamma(self) -> float:
        gamma = float(np.float32(self.config.gamma))
        ramp = int(self.config.gamma_ramp_steps)
        if ramp <= 0:
            return gamma
        return gamma * min(1.0, float(self._coupled_step + 1) / float(ramp))

    @property
    def coupled_step(self) -> int:
        return self._coupled_step

    def coupling_diagnostics(self) -> dict[str, int | float]:
        n = self.mpm.particle_count()
        if n == 0:
            min_w = mean_w = 0.0
        else:
            vw = self._valid[:n]
            min_w = float(vw.min().item())
            mean_w = float(vw.double().mean().item())
        counts, _ = self._counter_values()
        return {
            "unsupported_particle_count": int(counts[0]),
            "partial_support_particle_count": int(counts[1]),
            "clipped_particle_count": int(counts[2]),
            "min_particle_valid_weight": min_w,
            "mean_particle_valid_weight": mean_w,
            "effective_gamma": self.effective_gamma(),
            **self.immersed_boundary_diagnostics(),
        }

    # ------------------------------------------------------- checkpointing
    def state_dict(self) -> dict:
        """Coupler state: accumulated fields, per-particle diagnostics, counters, step count."""
        return {"kind": "LBMMpmCoupler", "accum": self._accum.clone(), "ib": self._ib.clone(),
                "valid": self._valid.clone(), "mask": self._mask.clone(),
                "contact_mask": self._contact_mask.clone(), "counters": self._counters.clone(),
                "coupled_step": self._coupled_step}

    def load_state_dict(self, state: dict) -> None:
        if state.get("kind") != "LBMMpmCoupler":
            raise ValueError("not a coupler checkpoint")
        for name in ("accum", "ib", "valid", "mask", "contact_mask", "counters"):
            getattr(self, "_" + name).copy_(state[name])
        self._ib_written = True
        self._reaction_fresh = False
        self._coupled_step = int(state["coupled_step"])

    def _validate_initialized(self) -> None:
        if not getattr(self.lbm, "_initialized", False):
            raise RuntimeError("LBMSolver3D.initialize must be called before coupling.")
        if not getattr(self.mpm, "_initialized", False):
            raise RuntimeError(
                "MPMSolver3D particle initialization must be called before coupling."
            )
