"""Batches of independent scenes advanced together (no reference counterpart).

``LatticeBatch`` holds many D3Q19 lattices of different sizes, rates and forces in one set
of concatenated device arrays and advances all of them with one launch per phase
(``fsi_batch_*`` of the C ABI), instead of one LBMSolver3D and one launch per lattice.
Each lattice behaves exactly as an LBMSolver3D with the same configuration: the per-cell
code is shared, so a batch of exact-form lattices is bit-identical to the standalone runs.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as nat
from .config import LBMConfig
from .lbm3d import _STORAGE_CODE, _STORAGE_DTYPE, relaxation_rates

_Q = 19


class LatticeBatch:
    """Many periodic lattices stepped together (all with one storage / arithmetic form)."""

    def __init__(self, configs: list[LBMConfig]):
        if not configs:
            raise ValueError("a batch needs at least one lattice.")
        for c in configs:
            c.validate()
            if c.use_sparse:
                raise NotImplementedError("Sparse LBM storage is not implemented.")
            for face in (c.x_left, c.x_right, c.y_left, c.y_right, c.z_left, c.z_right):
                if face.boundary_type != "periodic":
                    raise NotImplementedError("batched lattices have periodic faces; "
                                              "express walls as solid mask planes.")
        forms = {(c.population_storage, c.resolved_arithmetic()) for c in configs}
        if len(forms) != 1:
            raise ValueError(f"a batch uses one storage / arithmetic form, got {sorted(forms)}.")
        storage, arithmetic = forms.pop()
        self.configs = list(configs)
        self.count = len(configs)
        self.shapes = [(c.nx, c.ny, c.nz) for c in configs]
        self.sizes = [nx * ny * nz for nx, ny, nz in self.shapes]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        self.cells = int(self.offsets[-1])
        table = (nat.BatchLattice * self.count)()
        for s, c in enumerate(configs):
            L = table[s]
            L.nx, L.ny, L.nz = c.nx, c.ny, c.nz
            L.cell_offset = int(self.offsets[s])
            rates = relaxation_rates(c.viscosity, c.mrt_rates)
            for k in range(_Q):
                L.s[k] = float(rates[k])
            L.rho0 = float(np.float32(c.rho0))
            for a in range(3):
                L.base_force[a] = float(np.float32(c.force[a]))
        self._device = nat.device()
        nat.load()
        handle = ctypes.c_void_p()
        nat.call("fsi_batch_create", table, self.count, _STORAGE_CODE[storage],
                 nat.ARITH_FAST if arithmetic == "fast" else nat.ARITH_EXACT, ctypes.byref(handle))
        self._handle = handle
        n, dev = self.cells, self._device
        self._pops = torch.zeros((_Q * n,), dtype=_STORAGE_DTYPE[storage], device=dev)
        self._macro = torch.zeros((n, 4), dtype=torch.float32, device=dev)
        self._force_buf = [torch.zeros((3 * n,), dtype=torch.float32, device=dev) for _ in range(2)]
        self._flags = torch.zeros(n, dtype=torch.int32, device=dev)
        self._solid = torch.zeros(n, dtype=torch.int32, device=dev)
        self._diag = torch.zeros((self.count, 2), dtype=torch.float64, device=dev)
        self._steps_done = 0
        self._macro_fresh = True
        self._fcur = 0
        self._fprev = -1
        self._initialized = False

    def __del__(self):
        handle = getattr(self, "_handle", None)
        if handle is not None and handle.value:
            try:
                nat.call("fsi_batch_destroy", handle)
            except Exception:
                pass
            self._handle = None

    # ---------------------------------------------------------------- setup
    def initialize(self, solids: list[np.ndarray | None] | None = None) -> None:
        host = np.zeros(self.cells, np.int32)
        for s, shape in enumerate(self.shapes):
            mask = None if solids is None else solids[s]
            if mask is None:
                continue
            arr = np.asarray(mask)
            if arr.shape != shape:
                raise ValueError(f"solid mask {s} shape must be {shape}, got {arr.shape}.")
            host[self.offsets[s]:self.offsets[s + 1]] = np.where(arr > 0, 1, 0).reshape(-1)
        self._solid.copy_(torch.from_numpy(host))
        st = nat.stream_ptr()
        nat.call("fsi_batch_lbm_flags", self._handle, nat.ptr(self._solid), nat.ptr(self._flags), st)
        u0 = torch.tensor(np.array([np.float32(c.initial_velocity) for c in self.configs],
                                   np.float32), device=self._device)
        nat.call("fsi_batch_lbm_init", self._handle, nat.ptr(u0), nat.ptr(self._flags),
                 nat.ptr(self._pops), nat.ptr(self._macro), st)
        self._fcur, self._fprev = 0, -1
        nat.call("fsi_batch_lbm_base_force", self._handle, nat.ptr(self._flags),
                 nat.ptr(self._force_buf[0]), st)
        self._steps_done = 0
        self._macro_fresh = True
        self._initialized = True

    # ------------------------------------------------------------------ step
    def step(self) -> None:
        if not self._initialized:
            raise RuntimeError("LatticeBatch.initialize must be called before step().")
        force = self._force_buf[self._fcur]
        force_prev = None
        if not self._macro_fresh:
            force_prev = self._force_buf[self._fprev]
        nat.call("fsi_batch_lbm_step", self._handle, nat.ptr(self._pops), nat.ptr(self._macro),
                 nat.ptr(force), nat.ptr(force_prev), nat.ptr(self._flags), self._steps_done,
                 nat.stream_ptr())
        self._steps_done += 1
        self._fprev = self._fcur
        self._macro_fresh = False

    def writable_force(self) -> torch.Tensor:
        """The force buffer of the next step ([3][N_s] blocks), switched so that the force of
        the last step stays available for recomputing the current velocity."""
        if self._fcur == self._fprev:
            self._fcur = 1 - self._fcur
        return self._force_buf[self._fcur]

    def _ensure_macro(self, diag: bool = False) -> None:
        if self._macro_fresh and not diag:
            return
        force = self._force_buf[self._fprev if self._fprev >= 0 else self._fcur]
        nat.call("fsi_batch_lbm_macro", self._handle, nat.ptr(self._pops), nat.ptr(force),
                 nat.ptr(self._flags), self._steps_done, nat.ptr(self._macro),
                 nat.ptr(self._diag) if diag else None, nat.stream_ptr())
        self._macro_fresh = True

    # ------------------------------------------------------------- accessors
    @property
    def macro(self) -> torch.Tensor:
        self._ensure_macro()
        return self._macro

    @property
    def flags(self) -> torch.Tensor:
        return self._flags

    @property
    def steps_done(self) -> int:
        return self._steps_done

    def _block(self, t: torch.Tensor, s: int, width: int) -> torch.Tensor:
        a, b = int(self.offsets[s]), int(self.offsets[s + 1])
        return t[a * width:b * width] if t.dim() == 1 else t[a:b]

    def density_numpy(self, s: int) -> np.ndarray:
        return self._block(self.macro, s, 1)[:, 3].reshape(self.shapes[s]).cpu().numpy()

    def velocity_numpy(self, s: int) -> np.ndarray:
        return self._block(self.macro, s, 1)[:, :3].reshape(*self.shapes[s], 3).cpu().numpy()

    def distribution_numpy(self, s: int) -> np.ndarray:
        out = torch.empty((self.cells, _Q), dtype=torch.float32, device=self._device)
        nat.call("fsi_batch_lbm_distribution", self._handle, nat.ptr(self._pops),
                 nat.ptr(self._flags), self._steps_done, nat.ptr(out), nat.stream_ptr())
        return self._block(out, s, 1).reshape(*self.shapes[s], _Q).cpu().numpy()

    def mass_and_speed(self) -> np.ndarray:
        """Per lattice (sum of rho over fluid cells, max |u|) as float64[count, 2]."""
        if self._macro_fresh:
            # Current macro (e.g. the initial fields, which are not recomputed from the
            # populations): reduce it as it stands.
            out = np.zeros((self.count, 2))
            for s in range(self.count):
                m = self._block(self._macro, s, 1)
                fluid = self._block(self._flags, s, 1) & 1 == 0
                out[s, 0] = float(m[fluid, 3].double().sum())
                out[s, 1] = float(torch.linalg.vector_norm(m[:, :3], dim=1).max())
            return out
        self._ensure_macro(diag=True)
        return self._diag.cpu().numpy()
