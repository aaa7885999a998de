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
        self.tuning = {"step_tile_cells": 256, "variant": 1}

    # ------------------------------------------------------------ state / tuning
    def snapshot(self) -> dict:
        """Device copies of the lattice state and its host bookkeeping."""
        return {"pops": self._pops.clone(), "macro": self._macro.clone(),
                "force": [f.clone() for f in self._force_buf],
                "host": (self._steps_done, self._macro_fresh, self._fcur, self._fprev)}

    def restore(self, snap: dict) -> None:
        self._pops.copy_(snap["pops"])
        self._macro.copy_(snap["macro"])
        for dst, src in zip(self._force_buf, snap["force"]):
            dst.copy_(src)
        self._steps_done, self._macro_fresh, self._fcur, self._fprev = snap["host"]

    def autotune(self, steps: int = 4, use_cache: bool = True) -> dict:
        """Pick the step kernel's launch parameters for this batch (fsi.autotune)."""
        from .autotune import tune_lattice_batch
        return tune_lattice_batch(self, steps=steps, use_cache=use_cache)

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

    def distribution(self) -> torch.Tensor:
        """Post-stream populations of every lattice in the reference layout, device float32
        [cells][19]; lattice s is rows offsets[s]:offsets[s + 1]."""
        out = torch.empty((self.cells, _Q), dtype=torch.float32, device=self._device)
        nat.call("fsi_batch_lbm_distribution", self._handle, nat.ptr(self._pops),
                 nat.ptr(self._flags), self._steps_done, nat.ptr(out), nat.stream_ptr())
        return out

    def distribution_numpy(self, s: int) -> np.ndarray:
        return self._block(self.distribution(), s, 1).reshape(*self.shapes[s], _Q).cpu().numpy()

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


class SceneBatch:
    """Many independent coupled LBM-MPM scenes stepped together (no reference counterpart).

    Scene s behaves as ``FSISimulation(configs[s])`` stepped with ``coupler.step(lbm_dt)``:
    per coupled step, ``substeps`` times (coupling forces, MPM substep), then force assembly
    and the lattice step -- with each phase one launch over all scenes. All scenes share
    lbm_dt, the number of substeps, the population storage form and periodic faces; contact
    is not batched. ``run(steps)`` replays a captured CUDA graph of two coupled steps once
    every scene's gamma ramp has finished (its gamma is then a constant of the graph).
    """

    def __init__(self, configs):
        from .config import SimulationConfig  # noqa: F401  (type of configs)

        if not configs:
            raise ValueError("a batch needs at least one scene.")
        for c in configs:
            c.validate()
            if c.coupling.contact_enabled:
                raise NotImplementedError("contact is not batched.")
            if not c.coupling.enabled:
                raise NotImplementedError("a scene batch couples every scene.")
        for key in ("build_solid_volume_fraction", "immersed_boundary_enabled"):
            if len({bool(getattr(c.coupling, key)) for c in configs}) != 1:
                raise ValueError(f"scenes of a batch share coupling.{key}.")
        subs = {int(c.coupling.mpm_substeps_per_lbm_step) for c in configs}
        dts = {float(c.lbm_dt) for c in configs}
        if len(subs) != 1 or len(dts) != 1:
            raise ValueError("scenes of a batch share lbm_dt and mpm_substeps_per_lbm_step.")
        self.configs = list(configs)
        self.count = len(configs)
        self.substeps = subs.pop()
        self.lbm_dt = dts.pop()
        self.lattice = LatticeBatch([c.lbm for c in configs])
        self._device = self.lattice._device
        self.step_index = 0
        self._coupled_step = 0
        self._initialized = False

    # ---------------------------------------------------------------- setup
    def initialize(self, solids, positions, youngs_modulus=None, poisson_ratio=None) -> None:
        """solids: per-scene masks (or None); positions: per-scene float32 (n_s, 3) arrays;
        youngs_modulus / poisson_ratio: optional per-scene scalars or per-particle arrays."""
        from .coupling import coupling_descriptor, gamma_for_step
        from .mpm3d import MPMSolver3D, mpm_descriptor, particle_mass_volume

        if len(positions) != self.count:
            raise ValueError("one particle set per scene is required.")
        self.lattice.initialize(solids)
        align = nat.BATCH_PARTICLE_ALIGN
        counts = [int(np.asarray(p).shape[0]) for p in positions]
        offsets, off = [], 0
        for n in counts:
            offsets.append(off)
            off += (n + align - 1) // align * align
        cap = max(off, align)
        self.particle_counts, self.particle_offsets, self.capacity = counts, offsets, cap
        dev, f32 = self._device, torch.float32
        x = np.zeros((3, cap), np.float32)
        F = np.zeros((9, cap), np.float32)
        mass = np.zeros(cap, np.float32)
        vol = np.zeros(cap, np.float32)
        active = np.zeros(cap, np.int32)
        mu = np.zeros(cap, np.float32)
        lam = np.zeros(cap, np.float32)
        table = (nat.BatchSolid * self.count)()
        mpm_dt = self.lbm_dt / float(self.substeps)
        for s, (c, pos, o, n) in enumerate(zip(self.configs, positions, offsets, counts)):
            p = np.asarray(pos, np.float32)
            if p.ndim != 2 or p.shape[1] != 3 or n <= 0:
                raise ValueError(f"positions of scene {s} must have shape (n, 3), n > 0.")
            m, v = particle_mass_volume(c.mpm)
            x[:, o:o + n] = p.T
            F[[0, 4, 8], o:o + n] = 1.0
            mass[o:o + n] = np.float32(m)
            vol[o:o + n] = np.float32(v)
            active[o:o + n] = 1
            E = c.mpm.youngs_modulus if youngs_modulus is None else youngs_modulus[s]
            nu = c.mpm.poisson_ratio if poisson_ratio is None else poisson_ratio[s]
            mu_s, lam_s = MPMSolver3D.lame_parameters(np.broadcast_to(np.asarray(E, np.float64), (n,)),
                                                      np.broadcast_to(np.asarray(nu, np.float64), (n,)))
            mu[o:o + n] = mu_s.astype(np.float32)
            lam[o:o + n] = lam_s.astype(np.float32)
            t = table[s]
            t.mpm = mpm_descriptor(c.mpm, dt=mpm_dt)
            t.mpm.num_particles = n
            t.coupling = coupling_descriptor(c.coupling, c.mpm.dx)
            t.coupling.gamma_eff = gamma_for_step(c.coupling, 0)
            t.particle_offset = o
        self._per_particle_material = youngs_modulus is not None or poisson_ratio is not None
        to = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        self._x, self._F = to(x), to(F)
        self._v = torch.zeros((3, cap), dtype=f32, device=dev)
        self._C = torch.zeros((9, cap), dtype=f32, device=dev)
        self._mass, self._vol, self._active = to(mass), to(vol), to(active)
        self._force = torch.zeros((3, cap), dtype=f32, device=dev)
        self._mu, self._lam = to(mu), to(lam)
        parts = nat.Particles()
        for name, t in (("x", self._x), ("v", self._v), ("C", self._C), ("F", self._F),
                        ("mass", self._mass), ("volume", self._vol), ("active", self._active),
                        ("force", self._force)):
            setattr(parts, name, t.data_ptr())
        parts.capacity = cap
        if self._per_particle_material:
            parts.mu, parts.lam = self._mu.data_ptr(), self._lam.data_ptr()
        self._parts = parts
        dirty = ctypes.c_int64()
        nat.call("fsi_batch_set_solids", self.lattice._handle, table, cap, ctypes.byref(dirty))
        n = self.lattice.cells
        self._grid = torch.zeros((n, 4), dtype=f32, device=dev)
        self._dirty = torch.zeros(max(int(dirty.value), 1), dtype=torch.uint8, device=dev)
        self._accum = torch.zeros((n, 4), dtype=f32, device=dev)
        self._ib = torch.zeros((3 * n,), dtype=f32, device=dev)
        self._valid = torch.zeros(cap, dtype=f32, device=dev)
        self._mask = torch.zeros(cap, dtype=torch.int32, device=dev)
        self._counters = torch.zeros((self.count, 12), dtype=torch.int32, device=dev)
        self._gamma_host = np.array([gamma_for_step(c.coupling, 0) for c in self.configs],
                                    np.float32)
        self._initialized = True

    # ------------------------------------------------------------------ step
    def _set_gamma(self) -> None:
        from .coupling import gamma_for_step

        g = np.array([gamma_for_step(c.coupling, self._coupled_step) for c in self.configs],
                     np.float32)
        if not np.array_equal(g, self._gamma_host):
            nat.call("fsi_batch_set_gamma", self.lattice._handle,
                     g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
            self._gamma_host = g

    def _gamma_settled(self) -> bool:
        return all(int(c.coupling.gamma_ramp_steps) <= 0
                   or self._coupled_step + 1 >= int(c.coupling.gamma_ramp_steps)
                   for c in self.configs)

    def step(self) -> None:
        """One coupled step of every scene (coupling.py:135-173 per scene)."""
        if not self._initialized:
            raise RuntimeError("SceneBatch.initialize must be called before step().")
        self._set_gamma()
        h, st = self.lattice._handle, nat.stream_ptr()
        self._accum.zero_()
        self._ib.zero_()
        self._counters.zero_()
        self._valid.zero_()
        self._mask.zero_()
        dt_ratio = float(np.float32((self.lbm_dt / self.substeps) / self.lbm_dt))
        build = [bool(c.coupling.build_solid_volume_fraction) for c in self.configs]
        for sub in range(self.substeps):
            self._counters[:, 0:5].zero_()
            nat.call("fsi_batch_coupling_forces", h, self._parts, nat.ptr(self.lattice.macro),
                     nat.ptr(self.lattice.flags), nat.ptr(self._accum), nat.ptr(self._valid),
                     nat.ptr(self._mask), nat.ptr(self._counters), dt_ratio,
                     int(sub == 0 and all(build)), st)
            nat.call("fsi_batch_mpm_substep", h, self._parts, nat.ptr(self._grid),
                     nat.ptr(self._dirty), st)
        mode = nat.ASSEMBLE_COUPLING | (nat.ASSEMBLE_CLAMP_FRACTION if all(build) else 0)
        if any(c.coupling.immersed_boundary_enabled for c in self.configs):
            mode |= nat.ASSEMBLE_IB
            self._counters[:, 5:7].zero_()
            self._counters[:, 8:12].zero_()
        force = self.lattice.writable_force()
        nat.call("fsi_batch_coupling_assemble", h, nat.ptr(self.lattice.flags), mode,
                 nat.ptr(self._accum), nat.ptr(self.lattice.macro), nat.ptr(force),
                 nat.ptr(self._ib), nat.ptr(self._counters), st)
        self.lattice.step()
        self._coupled_step += 1
        self.step_index += 1

    def _assemble_mode(self) -> int:
        build = all(bool(c.coupling.build_solid_volume_fraction) for c in self.configs)
        mode = nat.ASSEMBLE_COUPLING | (nat.ASSEMBLE_CLAMP_FRACTION if build else 0)
        if any(c.coupling.immersed_boundary_enabled for c in self.configs):
            mode |= nat.ASSEMBLE_IB
        return mode

    def run_persistent(self, steps: int, max_steps_per_launch: int = 1000,
                       wait_cycles: int = 0) -> None:
        """``steps`` coupled steps of every scene, each launch of up to
        ``max_steps_per_launch`` steps one persistent cooperative kernel (grid-wide barriers
        between the phases of SceneBatch.step, each wait bounded by ``wait_cycles`` SM clock
        cycles, 0 for about a second). Steps inside the gamma ramp and the first step after
        initialisation run eagerly. Raises when a launch reports a barrier wait that gave up
        (the batch's state is then undefined)."""
        steps = int(steps)
        if steps < 0:
            raise ValueError("steps must be non-negative.")
        L = self.lattice
        while steps > 0 and (not self._gamma_settled() or L._fcur != L._fprev):
            self.step()
            steps -= 1
        if steps == 0:
            return
        self._set_gamma()
        if not hasattr(self, "_sync"):
            self._sync = torch.zeros(1, dtype=torch.int32, device=self._device)
            self._error = torch.zeros(1, dtype=torch.int32, device=self._device)
        st = nat.BatchState()
        st.pops, st.macro = L._pops.data_ptr(), L._macro.data_ptr()
        st.force[0], st.force[1] = L._force_buf[0].data_ptr(), L._force_buf[1].data_ptr()
        st.flags, st.accum, st.ib_force = L._flags.data_ptr(), self._accum.data_ptr(), self._ib.data_ptr()
        st.valid_weight, st.coupling_mask = self._valid.data_ptr(), self._mask.data_ptr()
        st.counters, st.grid, st.dirty = (self._counters.data_ptr(), self._grid.data_ptr(),
                                          self._dirty.data_ptr())
        st.sync, st.error = self._sync.data_ptr(), self._error.data_ptr()
        dt_ratio = float(np.float32((self.lbm_dt / self.substeps) / self.lbm_dt))
        build = int(all(bool(c.coupling.build_solid_volume_fraction) for c in self.configs))
        while steps > 0:
            k = min(steps, int(max_steps_per_launch))
            nat.call("fsi_batch_run_persistent", self.lattice._handle, self._parts, st,
                     L._steps_done, k, self.substeps, dt_ratio, build, self._assemble_mode(),
                     L._fprev, int(L._macro_fresh), int(wait_cycles), nat.stream_ptr())
            L._steps_done += k
            L._fprev = L._fcur = L._fprev ^ (k & 1)
            L._macro_fresh = False
            self._coupled_step += k
            self.step_index += k
            steps -= k
        err = int(self._error.item())
        if err:
            self._error.zero_()
            raise nat.NativeError(f"persistent batch launch: a grid barrier wait gave up (code {err})")

    def autotune(self, steps: int = 4, use_cache: bool = True) -> dict:
        """Tune the batched lattice step (fsi.autotune); the simulation state is unchanged."""
        return self.lattice.autotune(steps=steps, use_cache=use_cache)

    def _graph_state(self) -> tuple:
        L = self.lattice
        return (L._steps_done % 2, L._fcur, L._fprev, L._macro_fresh)

    def run(self, steps: int, graph: bool = True) -> None:
        """``steps`` coupled steps of every scene; the steady part as CUDA-graph replays."""
        steps = int(steps)
        if steps < 0:
            raise ValueError("steps must be non-negative.")
        L = self.lattice
        if graph:
            while steps > 0 and (not self._gamma_settled() or L._macro_fresh or L._fcur != L._fprev):
                self.step()
                steps -= 1
        if not graph or steps < 4:
            for _ in range(steps):
                self.step()
            return
        before = self._graph_state()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.step()
            self.step()
        g.replay()
        steps -= 2
        if self._graph_state() != before:
            for _ in range(steps):
                self.step()
            return
        while steps >= 2:
            g.replay()
            L._steps_done += 2
            self._coupled_step += 2
            self.step_index += 2
            steps -= 2
        if steps:
            self.step()

    # ------------------------------------------------------------- accessors
    def _rows(self, t: torch.Tensor, s: int, width: int) -> np.ndarray:
        o, n = self.particle_offsets[s], self.particle_counts[s]
        return t[:, o:o + n].t().reshape(n, width).cpu().numpy().copy()

    def positions_numpy(self, s: int) -> np.ndarray:
        return self._rows(self._x, s, 3)

    def velocities_numpy(self, s: int) -> np.ndarray:
        return self._rows(self._v, s, 3)

    def particle_forces_numpy(self, s: int) -> np.ndarray:
        return self._rows(self._force, s, 3)

    def density_numpy(self, s: int) -> np.ndarray:
        return self.lattice.density_numpy(s)

    def velocity_numpy(self, s: int) -> np.ndarray:
        return self.lattice.velocity_numpy(s)

    def counters_numpy(self) -> np.ndarray:
        """fsi_coupling_counters of every scene as int32[count, 12]."""
        return self._counters.cpu().numpy()
