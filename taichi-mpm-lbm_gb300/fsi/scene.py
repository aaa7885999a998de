"""The coupled step of one scene as a single native call (no reference counterpart).

``NativeScene`` binds an initialised ``LBMMpmCoupler`` (its lattice, solid and coupling
buffers) to a context of the C ABI (``fsi_ctx_create``) and advances it with
``fsi_coupled_step``: the whole of ``LBMMpmCoupler.step`` (fsi/coupling.py:135-173) in one
call, with the launch sequence of the Python coupler issued from C++. It is the path a host
without Python would bind; from Python it removes the per-launch host cost of the ~45
entry-point calls of a coupled step. The solvers' host bookkeeping (lattice parity, force
buffers, macro freshness, the gamma ramp's step count) is handed to the context before each
call and taken back after it, so the Python accessors, ``LBMMpmCoupler.step`` and
``NativeScene.step`` can be mixed freely.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as nat


class NativeScene:
    """One coupled scene advanced through ``fsi_coupled_step``."""

    def __init__(self, coupler):
        coupler._validate_initialized()
        self.coupler = coupler
        lbm, mpm, cfg = coupler.lbm, coupler.mpm, coupler.config
        d = nat.SceneDesc()
        d.lbm = lbm._desc
        d.mpm = mpm.desc
        d.coupling = coupler._desc
        for a in range(3):
            d.base_force[a] = float(np.float32(lbm.config.force[a]))
        d.gamma = float(np.float32(cfg.gamma))
        d.gamma_ramp_steps = int(cfg.gamma_ramp_steps)
        d.coupling_enabled = int(coupler.enabled)
        d.build_solid_fraction = int(coupler.build_solid_volume_fraction)
        d.contact_enabled = int(coupler.contact_enabled)
        d.immersed_boundary_enabled = int(coupler.immersed_boundary_enabled)
        d.p2g_mode = nat.P2G_SORTED if mpm.sorted else nat.P2G_ATOMIC
        b = nat.SceneBuffers()
        b.pops = lbm._pops.data_ptr()
        b.macro = lbm._macro.data_ptr()
        b.force[0] = lbm._force_buf[0].data_ptr()
        b.force[1] = lbm._force_buf[1].data_ptr()
        b.flags = lbm._flags.data_ptr()
        b.particles = mpm.particles
        b.accum = coupler._accum.data_ptr()
        b.ib_force = coupler._ib.data_ptr()
        b.valid_weight = coupler._valid.data_ptr()
        b.coupling_mask = coupler._mask.data_ptr()
        b.contact_mask = coupler._contact_mask.data_ptr()
        b.counters = coupler._counters.data_ptr()
        self._desc, self._buffers = d, b
        handle = ctypes.c_void_p()
        nat.call("fsi_ctx_create", ctypes.byref(d), ctypes.byref(b), ctypes.byref(handle))
        self._handle = handle
        self._particles = mpm.particle_count()

    def close(self) -> None:
        handle = getattr(self, "_handle", None)
        if handle is not None and handle.value:
            nat.call("fsi_ctx_destroy", handle)
        self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ----------------------------------------------------------- bookkeeping
    def _push(self) -> None:
        lbm, c = self.coupler.lbm, self.coupler
        if c.mpm.particle_count() != self._particles:
            raise RuntimeError("the particle count changed after the scene was bound; "
                               "create a new NativeScene.")
        nat.call("fsi_ctx_set_state", self._handle, lbm._steps_done, int(lbm._macro_fresh),
                 lbm._fcur, lbm._fprev, c._coupled_step)

    def _pull(self) -> None:
        lbm, c = self.coupler.lbm, self.coupler
        steps, fresh = ctypes.c_int64(), ctypes.c_int32()
        fnext, flast, coupled = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
        nat.call("fsi_ctx_get_state", self._handle, ctypes.byref(steps), ctypes.byref(fresh),
                 ctypes.byref(fnext), ctypes.byref(flast), ctypes.byref(coupled))
        lbm._steps_done = int(steps.value)
        lbm._macro_fresh = bool(fresh.value)
        lbm._fcur, lbm._fprev = int(fnext.value), int(flast.value)
        c._coupled_step = int(coupled.value)
        c._reaction_fresh = False  # the native step rewrote the accumulator
        if c.immersed_boundary_enabled:
            c._ib_written = True

    # ------------------------------------------------------------------ step
    def step(self, lbm_dt: float, steps: int = 1, body_force=None) -> None:
        """``steps`` coupled steps, each as LBMMpmCoupler.step(lbm_dt, body_force)."""
        lbm_dt = float(lbm_dt)
        if lbm_dt <= 0.0:
            raise ValueError("lbm_dt must be positive.")
        if int(steps) < 0:
            raise ValueError("steps must be non-negative.")
        bf = None
        if body_force is not None:
            arr = np.asarray(body_force, dtype=np.float32)
            if arr.shape != (3,):
                raise ValueError("body_force must have 3 components.")
            bf = (ctypes.c_float * 3)(*[float(v) for v in arr])
        self._push()
        try:
            nat.call("fsi_coupled_step", self._handle, lbm_dt, bf, self.coupler.substeps,
                     int(steps), nat.stream_ptr())
        finally:
            self._pull()
