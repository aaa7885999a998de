"""Dense D3Q19 MRT lattice Boltzmann solver on the GPU (drop-in for the reference's fsi/lbm3d.py).

Storage lives in torch CUDA tensors; every kernel is the library's sm_103a code
reached through the C ABI (``fsi._native``):

* populations ``[19, N]`` in one array updated in place by the fused
  AA-pattern step (collide + stream + bounce-back in one pass): float32, or the
  float16 / bfloat16 deviation forms selected by ``LBMConfig.population_storage``;
* ``macro`` ``float32[N, 4]`` = (ux, uy, uz, rho), materialised on demand: the
  step kernel recomputes rho and u in registers, so the array is refreshed only
  when something reads it (accessors, diagnostics, the coupler);
* two force buffers ``float32[3, N]``: the step's force and the previous
  step's force (needed to recompute the previous macroscopic velocity) are kept
  apart by switching buffers whenever the force is modified after a step.

Public methods, accessors, layouts and exceptions follow fsi/lbm3d.py:57-534.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np
import torch

from . import _native as nat
from .config import BoundaryConfig, LBMConfig

_Q = 19
_SUPPORTED_X_BOUNDARIES = {"periodic", "pressure", "velocity"}


def _boundary_mode(boundary: BoundaryConfig) -> int:
    """Face condition code (lbm3d.py:16-27)."""
    kind = boundary.boundary_type
    if kind == "wall":
        raise NotImplementedError(
            "wall face boundaries are reserved for a later step; use solid masks for now."
        )
    codes = {"periodic": 0, "pressure": 1, "velocity": 2}
    if kind not in codes:
        raise ValueError(f"Unsupported boundary type: {kind}.")
    if kind == "velocity" and getattr(boundary, "velocity_update", "sequential") == "simultaneous":
        return 3
    return codes[kind]


_STORAGE_DTYPE = {"f32": torch.float32, "f16": torch.float16, "bf16": torch.bfloat16}
_STORAGE_CODE = {"f32": nat.STORAGE_F32, "f16": nat.STORAGE_F16, "bf16": nat.STORAGE_BF16}


def relaxation_rates(viscosity: float, overrides: dict | None = None) -> np.ndarray:
    """MRT rates of lbm3d.py:141-168: s_v = 1/tau on the viscous moments, s_o on the others.

    ``overrides`` ({moment: rate}, LBMConfig.mrt_rates) replaces individual non-conserved,
    non-shear rates (an extension; the reference fixes them)."""
    tau_f = 3.0 * viscosity + 0.5
    s_v = 1.0 / tau_f
    s_o = 8.0 * (2.0 - s_v) / (8.0 - s_v)
    v, o = s_v, s_o
    s = np.array([0.0, v, v, 0.0, o, 0.0, o, 0.0, o, v, v, v, v, v, v, v, o, o, o],
                 dtype=np.float32)
    for k, rate in (overrides or {}).items():
        s[int(k)] = np.float32(rate)
    return s


def dhumieres_rates(tau: float) -> dict[int, float]:
    """Relaxation rates of d'Humieres et al. (2002) for LBMConfig.mrt_rates: s_e = 1.19 (k=1),
    s_eps = 1.4 (k=2), s_q = 1.2 (k=4, 6, 8), s_pi = 1/tau (k=10, 12), s_m = 1.98 (k=16-18);
    the shear rates stay 1/tau. The reference instead uses 1/tau and 8(2-s)/(8-s)."""
    s_pi = 1.0 / tau
    return {1: 1.19, 2: 1.4, 4: 1.2, 6: 1.2, 8: 1.2, 10: s_pi, 12: s_pi, 16: 1.98, 17: 1.98,
            18: 1.98}


class LBMSolver3D:
    """Dense single-phase 3D D3Q19/MRT LBM solver (GPU)."""

    def __init__(self, config: LBMConfig):
        self.config = config
        self.config.validate()
        self._validate_supported_config()

        self.nx = int(config.nx)
        self.ny = int(config.ny)
        self.nz = int(config.nz)
        self.q = _Q
        self.n_cells = self.nx * self.ny * self.nz
        self.bc_x_left_mode = _boundary_mode(config.x_left)
        self.bc_x_right_mode = _boundary_mode(config.x_right)

        self._s = relaxation_rates(config.viscosity, config.mrt_rates)
        self._desc = self._make_desc()
        self._device = nat.device()
        nat.load()
        n = self.n_cells
        dev = self._device
        self._pops = torch.zeros((_Q, n), dtype=_STORAGE_DTYPE[config.population_storage],
                                 device=dev)
        self._macro = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        self._force_buf = [torch.zeros((3, n), dtype=torch.float32, device=dev) for _ in range(2)]
        self._flags = torch.zeros(n, dtype=torch.int32, device=dev)
        self._solid_dev = torch.zeros(n, dtype=torch.int32, device=dev)
        self._solid_host = np.zeros((self.nx, self.ny, self.nz), dtype=np.int32)
        self._diag = torch.zeros(8, dtype=torch.float64, device=dev)
        self._diag_host = torch.zeros(8, dtype=torch.float64).pin_memory()
        self._base_force = np.asarray(config.force, dtype=np.float32)
        self._steps_done = 0
        self._macro_fresh = True
        self._fcur = 0
        self._fprev = -1
        self._mass_speed_cache = None
        self._build_flags()
        self._initialized = False

    # ---------------------------------------------------------------- setup
    def _validate_supported_config(self) -> None:
        if self.config.use_sparse:
            raise NotImplementedError("Sparse LBM storage is not implemented in Step 2.")
        for name, face in (("x_left", self.config.x_left), ("x_right", self.config.x_right)):
            if face.boundary_type not in _SUPPORTED_X_BOUNDARIES:
                raise NotImplementedError(f"{name}={face.boundary_type!r} is not implemented in Step 2.")
        for name, face in (("y_left", self.config.y_left), ("y_right", self.config.y_right),
                           ("z_left", self.config.z_left), ("z_right", self.config.z_right)):
            if face.boundary_type != "periodic":
                raise NotImplementedError(
                    f"{name}={face.boundary_type!r} is not implemented in Step 2; "
                    "use periodic Y/Z boundaries and solid masks for now."
                )

    def _make_desc(self) -> nat.LbmDesc:
        c = self.config
        d = nat.LbmDesc()
        d.nx, d.ny, d.nz = self.nx, self.ny, self.nz
        d.bc_mode_left, d.bc_mode_right = self.bc_x_left_mode, self.bc_x_right_mode
        for k in range(_Q):
            d.s[k] = float(self._s[k])
        d.rho0 = float(np.float32(c.rho0))
        d.bc_rho_left = float(np.float32(c.x_left.rho))
        d.bc_rho_right = float(np.float32(c.x_right.rho))
        for i in range(3):
            d.bc_vel_left[i] = float(np.float32(c.x_left.velocity[i]))
            d.bc_vel_right[i] = float(np.float32(c.x_right.velocity[i]))
        d.storage = _STORAGE_CODE[c.population_storage]
        d.arithmetic = nat.ARITH_FAST if c.resolved_arithmetic() == "fast" else nat.ARITH_EXACT
        return d

    def _call(self, name: str, *args) -> None:
        nat.call(name, self._desc, *args)

    def _build_flags(self) -> None:
        self._call("fsi_lbm_build_flags", nat.ptr(self._solid_dev), nat.ptr(self._flags),
                   nat.stream_ptr())

    def initialize(self, solid_np: np.ndarray | None = None) -> None:
        if solid_np is None:
            solid = np.zeros((self.nx, self.ny, self.nz), dtype=np.int32)
        else:
            solid = self._normalize_solid_mask(solid_np)
        self._solid_host = solid
        self._solid_dev.copy_(torch.from_numpy(solid.reshape(-1)))
        self._build_flags()
        u0 = (np.asarray(self.config.initial_velocity, dtype=np.float32)).ctypes.data_as(
            nat.ctypes.POINTER(nat.ctypes.c_float))
        self._call("fsi_lbm_init_fields", nat.ptr(self._flags), u0, nat.ptr(self._pops),
                   nat.ptr(self._macro), nat.stream_ptr())
        self._steps_done = 0
        self._macro_fresh = True
        self._fprev = -1
        self._mass_speed_cache = None
        self.reset_force()
        self._initialized = True

    def _normalize_solid_mask(self, solid_np: np.ndarray) -> np.ndarray:
        arr = np.asarray(solid_np)
        expected = (self.nx, self.ny, self.nz)
        if arr.shape != expected:
            raise ValueError(f"solid_np shape must be {expected}, got {arr.shape}.")
        return np.ascontiguousarray(np.where(arr > 0, 1, 0).astype(np.int32))

    @classmethod
    def load_solid_from_txt(cls, filename: str | Path, nx: int, ny: int, nz: int) -> np.ndarray:
        """Read a whitespace-separated 0/1 mask stored in Fortran order (lbm3d.py:213-217)."""
        data = np.reshape(np.loadtxt(filename), (nx, ny, nz), order="F")
        return np.ascontiguousarray(np.where(data > 0, 1, 0).astype(np.int32))

    # ----------------------------------------------------------------- step
    def step(self) -> None:
        if not self._initialized:
            raise RuntimeError("LBMSolver3D.initialize must be called before step().")
        force = self._force_buf[self._fcur]
        force_prev = None
        if not self._macro_fresh:
            force_prev = self._force_buf[self._fprev]
            if self._fprev == self._fcur:
                force_prev = force
        self._call("fsi_lbm_step", nat.ptr(self._pops), nat.ptr(self._macro), nat.ptr(force),
                   nat.ptr(force_prev), nat.ptr(self._flags), self._steps_done, nat.stream_ptr())
        self._steps_done += 1
        self._fprev = self._fcur
        self._macro_fresh = False

    def _ensure_macro(self) -> None:
        """Materialise rho and u of the current state (update_macro, lbm3d.py:409-425)."""
        if self._macro_fresh:
            return
        self._call("fsi_lbm_update_macro", nat.ptr(self._pops),
                   nat.ptr(self._force_buf[self._fprev]), nat.ptr(self._flags), self._steps_done,
                   nat.ptr(self._macro), nat.stream_ptr())
        self._macro_fresh = True

    @property
    def macro(self) -> torch.Tensor:
        """Current (ux, uy, uz, rho) per cell as a float32[N, 4] device tensor."""
        self._ensure_macro()
        return self._macro

    @property
    def flags(self) -> torch.Tensor:
        return self._flags

    @property
    def steps_done(self) -> int:
        return self._steps_done

    # ------------------------------------------------------------ accessors
    def density_numpy(self) -> np.ndarray:
        return self.macro[:, 3].reshape(self.nx, self.ny, self.nz).cpu().numpy()

    def velocity_numpy(self) -> np.ndarray:
        return self.macro[:, :3].reshape(self.nx, self.ny, self.nz, 3).cpu().numpy()

    def solid_numpy(self) -> np.ndarray:
        return self._solid_host.copy()

    def distribution_numpy(self) -> np.ndarray:
        out = torch.empty((self.n_cells, _Q), dtype=torch.float32, device=self._device)
        self._call("fsi_lbm_distribution", nat.ptr(self._pops), nat.ptr(self._flags),
                   self._steps_done, nat.ptr(out), nat.stream_ptr())
        return out.reshape(self.nx, self.ny, self.nz, _Q).cpu().numpy()

    def force_numpy(self) -> np.ndarray:
        f = self._force_buf[self._fcur]
        return f.t().reshape(self.nx, self.ny, self.nz, 3).cpu().numpy()

    @property
    def force(self) -> torch.Tensor:
        """The current force field as a float32[3, N] device tensor (read-only view)."""
        return self._force_buf[self._fcur]

    def _fetch_diag(self, count: int) -> np.ndarray:
        self._diag_host[:count].copy_(self._diag[:count], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return self._diag_host[:count].numpy().copy()

    def _reduce(self) -> np.ndarray:
        self._ensure_macro()
        self._call("fsi_lbm_reduce", nat.ptr(self._macro), nat.ptr(self._force_buf[self._fcur]),
                   nat.ptr(self._flags), nat.ptr(self._diag), nat.stream_ptr())
        return self._fetch_diag(5)

    def _mass_and_speed(self) -> tuple[float, float]:
        """(total mass, max |u|) of the current state, computed once per state: when rho and u
        are stale the refresh and both reductions run as one fused pass."""
        key = (self._steps_done, self._initialized)
        if self._mass_speed_cache is not None and self._mass_speed_cache[0] == key:
            return self._mass_speed_cache[1]
        if self._macro_fresh:
            r = self._reduce()
            val = (float(r[0]), float(r[1]))
        else:
            self._call("fsi_lbm_macro_diagnostics", nat.ptr(self._pops),
                       nat.ptr(self._force_buf[self._fprev]), nat.ptr(self._flags),
                       self._steps_done, nat.ptr(self._macro), nat.ptr(self._diag),
                       nat.stream_ptr())
            self._macro_fresh = True
            r = self._fetch_diag(2)
            val = (float(r[0]), float(r[1]))
        self._mass_speed_cache = (key, val)
        return val

    def _enqueue_mass_speed(self, out: torch.Tensor) -> tuple | None:
        """Enqueue (total mass, max |u|) of the current state into device double out[0:2]
        (out has at least 8 elements) without synchronising; refreshes rho and u when stale.
        Returns the cached pair when this state's values are already known."""
        key = (self._steps_done, self._initialized)
        if self._mass_speed_cache is not None and self._mass_speed_cache[0] == key:
            return self._mass_speed_cache[1]
        if self._macro_fresh:
            self._call("fsi_lbm_reduce", nat.ptr(self._macro), nat.ptr(self._force_buf[self._fcur]),
                       nat.ptr(self._flags), nat.ptr(out), nat.stream_ptr())
        else:
            self._call("fsi_lbm_macro_diagnostics", nat.ptr(self._pops),
                       nat.ptr(self._force_buf[self._fprev]), nat.ptr(self._flags),
                       self._steps_done, nat.ptr(self._macro), nat.ptr(out), nat.stream_ptr())
            self._macro_fresh = True
        return None

    def _remember_mass_speed(self, mass: float, speed: float) -> None:
        self._mass_speed_cache = ((self._steps_done, self._initialized), (mass, speed))

    def total_mass(self) -> float:
        return self._mass_and_speed()[0]

    def max_velocity_norm(self) -> float:
        return self._mass_and_speed()[1]

    def total_force(self) -> np.ndarray:
        return self._reduce()[2:5].astype(np.float32)

    # ------------------------------------------------------------ force API
    def _target_force_buffer(self) -> tuple[int, int]:
        """(input, output) buffer indices for a force update that must not
        overwrite the force the last step used."""
        src = self._fcur
        if self._fcur == self._fprev:
            self._fcur = 1 - self._fcur
        return src, self._fcur

    def _force_op(self, op: int, value=None) -> None:
        src, dst = self._target_force_buffer()
        val = None
        if value is not None:
            val = np.asarray(value, dtype=np.float32).ctypes.data_as(
                nat.ctypes.POINTER(nat.ctypes.c_float))
        self._call("fsi_lbm_force_op", nat.ptr(self._flags), op, nat.ptr(self._force_buf[src]),
                   val, nat.ptr(self._force_buf[dst]), nat.stream_ptr())

    def clear_force(self) -> None:
        self._force_op(nat.FORCE_CLEAR)

    def reset_force(self) -> None:
        self._force_op(nat.FORCE_SET, self._base_force)

    def set_uniform_force(self, force: tuple[float, float, float]) -> None:
        self._force_op(nat.FORCE_SET, self._validate_force_vector(force, "force"))

    def add_uniform_force(self, force: tuple[float, float, float]) -> None:
        self._force_op(nat.FORCE_ADD, self._validate_force_vector(force, "force"))

    def set_force_from_numpy(self, force_np: np.ndarray) -> None:
        force = self._normalize_force_field(force_np)
        _, dst = self._target_force_buffer()
        host = torch.from_numpy(force.reshape(-1, 3))
        self._force_buf[dst].copy_(host.t())
        self.zero_force_on_solid()

    def total_force_tensor(self) -> torch.Tensor:
        return self._force_buf[self._fcur]

    def zero_force_on_solid(self) -> None:
        self._force_op(nat.FORCE_ZERO_SOLID)

    @staticmethod
    def _validate_force_vector(force, name: str) -> np.ndarray:
        arr = np.asarray(force, dtype=np.float32)
        if arr.shape != (3,):
            raise ValueError(f"{name} must have 3 components.")
        return arr

    def _normalize_force_field(self, force_np: np.ndarray) -> np.ndarray:
        arr = np.asarray(force_np, dtype=np.float32)
        expected = (self.nx, self.ny, self.nz, 3)
        if arr.shape != expected:
            raise ValueError(f"force_np shape must be {expected}, got {arr.shape}.")
        return np.ascontiguousarray(arr)

    def load_populations(self, f: torch.Tensor | np.ndarray) -> None:
        """Replace the populations by ``f`` in the reference layout [nx, ny, nz, 19] (or
        [N, 19]) and restart the step count (no reference counterpart; used to start a
        lattice from a restricted or prolongated state). rho and u are recomputed from ``f``
        and the current force at the next step."""
        if self.config.population_storage != "f32":
            raise NotImplementedError("load_populations needs FP32 population storage.")
        t = torch.as_tensor(f, dtype=torch.float32, device=self._device).reshape(self.n_cells, _Q)
        self._pops.copy_(t.t())
        self._steps_done = 0
        self._fprev = self._fcur
        self._macro_fresh = False
        self._mass_speed_cache = None
        self._initialized = True

    # ------------------------------------------------------- checkpointing
    def state_dict(self) -> dict:
        """Complete lattice state (device tensors are cloned; no reference counterpart)."""
        return {
            "kind": "LBMSolver3D", "shape": (self.nx, self.ny, self.nz),
            "pops": self._pops.clone(), "macro": self._macro.clone(),
            "force": [f.clone() for f in self._force_buf], "solid": self._solid_host.copy(),
            "steps_done": self._steps_done, "macro_fresh": self._macro_fresh,
            "fcur": self._fcur, "fprev": self._fprev, "initialized": self._initialized,
        }

    def load_state_dict(self, state: dict) -> None:
        if state.get("kind") != "LBMSolver3D" or tuple(state["shape"]) != (self.nx, self.ny, self.nz):
            raise ValueError("checkpoint does not match this lattice")
        if state["pops"].dtype != self._pops.dtype:
            raise ValueError(f"checkpoint populations are {state['pops'].dtype}, this lattice "
                             f"stores {self._pops.dtype}")
        self._solid_host = np.ascontiguousarray(state["solid"], dtype=np.int32)
        self._solid_dev.copy_(torch.from_numpy(self._solid_host.reshape(-1)))
        self._build_flags()
        self._pops.copy_(state["pops"])
        self._macro.copy_(state["macro"])
        for dst, src in zip(self._force_buf, state["force"]):
            dst.copy_(src)
        self._steps_done = int(state["steps_done"])
        self._macro_fresh = bool(state["macro_fresh"])
        self._fcur, self._fprev = int(state["fcur"]), int(state["fprev"])
        self._initialized = bool(state["initialized"])
        self._mass_speed_cache = None

    # ------------------------------------------------- coupler entry points
    def _writable_force(self) -> torch.Tensor:
        """Buffer that the coupler may overwrite with the next step's force."""
        _, dst = self._target_force_buffer()
        return self._force_buf[dst]
