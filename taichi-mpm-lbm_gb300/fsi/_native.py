"""ctypes binding of the sm_103a library ``_lib/libfsi_gb300.so`` (C ABI: include/fsi_gb300.h).

The library is built in-tree by ``build_native.py``. There is no CPU fallback:
every solver call goes through this module, and a missing library or CUDA
device raises ``RuntimeError``.
"""
from __future__ import annotations

import collections
import ctypes
import os
from pathlib import Path

import torch

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfsi_gb300.so"
_lib = None

FSI_OK = 0
FSI_ERR_INVALID_ARG = 1
FSI_ERR_CUDA = 2
FSI_ERR_GUARD = 3
FSI_ERR_TIMEOUT = 4
FSI_ERR_UNSUPPORTED = 5
ABI_VERSION = 5

STORAGE_F32, STORAGE_F16, STORAGE_BF16 = 0, 1, 2
ARITH_EXACT, ARITH_FAST = 0, 1
FORCE_CLEAR, FORCE_SET, FORCE_ADD, FORCE_ZERO_SOLID = 0, 1, 2, 3
ASSEMBLE_CLAMP_FRACTION, ASSEMBLE_COUPLING, ASSEMBLE_IB, ASSEMBLE_BASE_ON_DEVICE = 1, 2, 4, 8

c_float3 = ctypes.c_float * 3


class LbmDesc(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("bc_mode_left", ctypes.c_int32), ("bc_mode_right", ctypes.c_int32),
        ("s", ctypes.c_float * 19),
        ("rho0", ctypes.c_float),
        ("bc_rho_left", ctypes.c_float), ("bc_rho_right", ctypes.c_float),
        ("bc_vel_left", c_float3), ("bc_vel_right", c_float3),
        ("storage", ctypes.c_int32), ("arithmetic", ctypes.c_int32),
    ]


class MpmDesc(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("num_particles", ctypes.c_int32),
        ("dt", ctypes.c_float), ("dx", ctypes.c_float), ("inv_dx", ctypes.c_float),
        ("mu", ctypes.c_float), ("lam", ctypes.c_float),
        ("gravity", c_float3),
        ("boundary_damping", ctypes.c_float),
        ("boundary_width", ctypes.c_int32),
        ("apic", ctypes.c_int32),
        ("clamp_lower", ctypes.c_float),
        ("clamp_upper", c_float3),
        ("material", ctypes.c_int32),
        ("launch_threads", ctypes.c_int32), ("coupling_fold", ctypes.c_int32),
    ]


class Particles(ctypes.Structure):
    _fields_ = [
        ("x", ctypes.c_void_p), ("v", ctypes.c_void_p), ("C", ctypes.c_void_p),
        ("F", ctypes.c_void_p), ("mass", ctypes.c_void_p), ("volume", ctypes.c_void_p),
        ("active", ctypes.c_void_p), ("force", ctypes.c_void_p),
        ("capacity", ctypes.c_int64),
        ("mu", ctypes.c_void_p), ("lam", ctypes.c_void_p),
    ]


class CouplingDesc(ctypes.Structure):
    _fields_ = [
        ("gamma_eff", ctypes.c_float),
        ("dt_ratio", ctypes.c_float),
        ("cell_volume", ctypes.c_float),
        ("inv_dx", ctypes.c_float),
        ("min_valid_weight", ctypes.c_float),
        ("rel_limit", ctypes.c_float),
        ("force_limit", ctypes.c_float),
        ("build_fraction", ctypes.c_int32),
        ("use_rel_limit", ctypes.c_int32),
        ("use_force_limit", ctypes.c_int32),
        ("ib_enabled", ctypes.c_int32),
        ("ib_drag", ctypes.c_float),
        ("ib_threshold", ctypes.c_float),
        ("ib_use_max", ctypes.c_int32),
        ("ib_max_force", ctypes.c_float),
        ("contact_enabled", ctypes.c_int32),
        ("contact_threshold", ctypes.c_float),
        ("contact_damping", ctypes.c_float),
    ]


P2G_ATOMIC, P2G_SORTED = 0, 1


class SceneDesc(ctypes.Structure):
    _fields_ = [
        ("lbm", LbmDesc), ("mpm", MpmDesc), ("coupling", CouplingDesc),
        ("base_force", c_float3),
        ("gamma", ctypes.c_float), ("gamma_ramp_steps", ctypes.c_int32),
        ("coupling_enabled", ctypes.c_int32), ("build_solid_fraction", ctypes.c_int32),
        ("contact_enabled", ctypes.c_int32), ("immersed_boundary_enabled", ctypes.c_int32),
        ("p2g_mode", ctypes.c_int32),
    ]


class SceneBuffers(ctypes.Structure):
    _fields_ = [
        ("pops", ctypes.c_void_p), ("macro", ctypes.c_void_p),
        ("force", ctypes.c_void_p * 2), ("flags", ctypes.c_void_p),
        ("particles", Particles),
        ("accum", ctypes.c_void_p), ("ib_force", ctypes.c_void_p),
        ("valid_weight", ctypes.c_void_p), ("coupling_mask", ctypes.c_void_p),
        ("contact_mask", ctypes.c_void_p), ("counters", ctypes.c_void_p),
    ]


class BatchLattice(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("cell_offset", ctypes.c_int64),
        ("s", ctypes.c_float * 19),
        ("rho0", ctypes.c_float),
        ("base_force", c_float3),
    ]


class BatchSolid(ctypes.Structure):
    _fields_ = [("mpm", MpmDesc), ("coupling", CouplingDesc), ("particle_offset", ctypes.c_int64)]


class BatchState(ctypes.Structure):
    _fields_ = [
        ("pops", ctypes.c_void_p), ("macro", ctypes.c_void_p), ("force", ctypes.c_void_p * 2),
        ("flags", ctypes.c_void_p), ("accum", ctypes.c_void_p), ("ib_force", ctypes.c_void_p),
        ("valid_weight", ctypes.c_void_p), ("coupling_mask", ctypes.c_void_p),
        ("counters", ctypes.c_void_p), ("grid", ctypes.c_void_p), ("dirty", ctypes.c_void_p),
        ("sync", ctypes.c_void_p), ("error", ctypes.c_void_p),
    ]


class ClosureGemmDesc(ctypes.Structure):
    _fields_ = [
        ("a", ctypes.c_void_p), ("b", ctypes.c_void_p),
        ("lda", ctypes.c_int32), ("ldb", ctypes.c_int32),
        ("m", ctypes.c_int32), ("n", ctypes.c_int32), ("k", ctypes.c_int32),
        ("k_chunk", ctypes.c_int32), ("mode", ctypes.c_int32), ("ldc", ctypes.c_int32),
        ("c", ctypes.c_void_p), ("bias", ctypes.c_void_p),
        ("h", ctypes.c_void_p), ("ht", ctypes.c_void_p),
        ("ldht", ctypes.c_int32), ("reserved", ctypes.c_int32),
        ("zout", ctypes.c_void_p), ("zin", ctypes.c_void_p), ("err", ctypes.c_void_p),
    ]


class ClosureWeights(ctypes.Structure):
    _fields_ = [
        ("w1", ctypes.c_void_p), ("w2", ctypes.c_void_p), ("w3", ctypes.c_void_p),
        ("w4", ctypes.c_void_p), ("bias", ctypes.c_void_p),
        ("pop_scale", ctypes.c_float), ("force_scale", ctypes.c_float),
        ("out_scale", ctypes.c_float), ("reserved", ctypes.c_int32),
    ]


GEMM_STORE, GEMM_ATOMIC, GEMM_GELU_FWD, GEMM_GELU_BWD = 0, 1, 2, 3
BATCH_PARTICLE_ALIGN = 256

_VP = ctypes.c_void_p
_BATCH = ctypes.c_void_p
_SIGNATURES = {
    "fsi_abi_version": ([], ctypes.c_int),
    "fsi_last_error": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_size_t),
    "fsi_lbm_build_flags": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP], ctypes.c_int),
    "fsi_lbm_init_fields": ([ctypes.POINTER(LbmDesc), _VP, ctypes.POINTER(ctypes.c_float), _VP, _VP, _VP], ctypes.c_int),
    "fsi_lbm_step": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP, _VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "fsi_lbm_update_macro": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP, ctypes.c_int64, _VP, _VP], ctypes.c_int),
    "fsi_lbm_distribution": ([ctypes.POINTER(LbmDesc), _VP, _VP, ctypes.c_int64, _VP, _VP], ctypes.c_int),
    "fsi_lbm_force_op": ([ctypes.POINTER(LbmDesc), _VP, ctypes.c_int, _VP, ctypes.POINTER(ctypes.c_float), _VP, _VP], ctypes.c_int),
    "fsi_lbm_reduce": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_lbm_macro_diagnostics": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP, ctypes.c_int64, _VP, _VP, _VP], ctypes.c_int),
    "fsi_mpm_substep": ([ctypes.POINTER(MpmDesc), ctypes.POINTER(Particles), _VP, _VP, _VP], ctypes.c_int),
    "fsi_mpm_substep_noalloc": ([ctypes.POINTER(MpmDesc), ctypes.POINTER(Particles), _VP], ctypes.c_int),
    "fsi_mpm_workspace_bytes": ([ctypes.POINTER(MpmDesc), ctypes.c_int64,
                                 ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "fsi_mpm_substep_sorted": ([ctypes.POINTER(MpmDesc), ctypes.POINTER(Particles), _VP, _VP,
                                ctypes.c_int64, _VP], ctypes.c_int),
    "fsi_coupled_substep": ([ctypes.POINTER(CouplingDesc), ctypes.POINTER(MpmDesc),
                             ctypes.POINTER(Particles), _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                             ctypes.c_int64, _VP], ctypes.c_int),
    "fsi_coupled_substep_tiled": ([ctypes.POINTER(CouplingDesc), ctypes.POINTER(MpmDesc),
                                   ctypes.POINTER(Particles), _VP, _VP, _VP, _VP, _VP, _VP, _VP,
                                   _VP, _VP], ctypes.c_int),
    "fsi_mpm_polar": ([_VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "fsi_mpm_base_cells": ([ctypes.POINTER(MpmDesc), ctypes.POINTER(Particles), _VP, _VP], ctypes.c_int),
    "fsi_mpm_reduce": ([ctypes.POINTER(MpmDesc), ctypes.POINTER(Particles), _VP, _VP, _VP], ctypes.c_int),
    "fsi_coupling_forces": ([ctypes.POINTER(CouplingDesc), ctypes.POINTER(MpmDesc), ctypes.POINTER(Particles), _VP, _VP, _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_coupling_assemble": ([ctypes.POINTER(CouplingDesc), ctypes.POINTER(LbmDesc), _VP, ctypes.POINTER(ctypes.c_float), ctypes.c_int, _VP, _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_coupling_assemble_sum": ([ctypes.POINTER(CouplingDesc), ctypes.POINTER(LbmDesc), _VP, ctypes.POINTER(ctypes.c_float), ctypes.c_int, _VP, _VP, _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_contact": ([ctypes.POINTER(CouplingDesc), ctypes.POINTER(MpmDesc), ctypes.POINTER(Particles), _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_coupling_reduce": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_coupled_diagnostics": ([ctypes.POINTER(MpmDesc), ctypes.POINTER(Particles),
                                 ctypes.POINTER(LbmDesc), _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_ctx_create": ([ctypes.POINTER(SceneDesc), ctypes.POINTER(SceneBuffers),
                        ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "fsi_ctx_destroy": ([_VP], ctypes.c_int),
    "fsi_ctx_get_state": ([_VP, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int32),
                           ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32),
                           ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "fsi_ctx_set_state": ([_VP, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                           ctypes.c_int64], ctypes.c_int),
    "fsi_coupled_step": ([_VP, ctypes.c_double, ctypes.POINTER(ctypes.c_float), ctypes.c_int32,
                          ctypes.c_int32, _VP], ctypes.c_int),
    "fsi_ctx_diagnostics": ([_VP, _VP, _VP], ctypes.c_int),
    "fsi_batch_create": ([ctypes.POINTER(BatchLattice), ctypes.c_int32, ctypes.c_int32,
                          ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "fsi_batch_destroy": ([_BATCH], ctypes.c_int),
    "fsi_batch_cells": ([_BATCH, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "fsi_batch_lbm_flags": ([_BATCH, _VP, _VP, _VP], ctypes.c_int),
    "fsi_batch_lbm_init": ([_BATCH, _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_batch_lbm_step": ([_BATCH, _VP, _VP, _VP, _VP, _VP, ctypes.c_int64, _VP], ctypes.c_int),
    "fsi_batch_lbm_macro": ([_BATCH, _VP, _VP, _VP, ctypes.c_int64, _VP, _VP, _VP], ctypes.c_int),
    "fsi_batch_lbm_distribution": ([_BATCH, _VP, _VP, ctypes.c_int64, _VP, _VP], ctypes.c_int),
    "fsi_batch_lbm_base_force": ([_BATCH, _VP, _VP, _VP], ctypes.c_int),
    "fsi_batch_tune": ([_BATCH, ctypes.c_int32, ctypes.c_int32], ctypes.c_int),
    "fsi_closure_features": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP, _VP, ctypes.c_int64, _VP,
                              ctypes.c_int32, ctypes.c_float, ctypes.c_float, _VP, _VP], ctypes.c_int),
    "fsi_closure_gemm": ([ctypes.POINTER(ClosureGemmDesc), _VP], ctypes.c_int),
    "fsi_closure_rows_bytes": ([ctypes.POINTER(LbmDesc)], ctypes.c_int64),
    "fsi_closure_infer_apply": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP, _VP, ctypes.c_int64,
                                 ctypes.POINTER(ClosureWeights), _VP, _VP, _VP], ctypes.c_int),
    "fsi_closure_infer": ([ctypes.POINTER(LbmDesc), _VP, _VP, _VP, _VP, ctypes.c_int64,
                           ctypes.POINTER(ClosureWeights), _VP, _VP, _VP, _VP], ctypes.c_int),
    "fsi_closure_apply": ([ctypes.POINTER(LbmDesc), _VP, _VP, ctypes.c_int64, _VP, _VP], ctypes.c_int),
    "fsi_selftest_wait_limit": ([_VP, _VP, _VP], ctypes.c_int),
    "fsi_closure_restrict": ([ctypes.POINTER(LbmDesc), _VP, _VP, ctypes.c_int64,
                              ctypes.POINTER(LbmDesc), _VP, _VP], ctypes.c_int),
    "fsi_closure_loss": ([_VP, _VP, _VP, ctypes.c_int32, _VP, _VP, ctypes.c_int32, _VP, _VP],
                         ctypes.c_int),
    "fsi_closure_colsum": ([_VP, ctypes.c_int32, ctypes.c_int32, _VP, _VP], ctypes.c_int),
    "fsi_closure_adam": ([_VP, _VP, _VP, _VP, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                          ctypes.c_float, ctypes.c_float, ctypes.c_int32, _VP], ctypes.c_int),
    "fsi_batch_set_solids": ([_BATCH, ctypes.POINTER(BatchSolid), ctypes.c_int64,
                              ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "fsi_batch_set_gamma": ([_BATCH, ctypes.POINTER(ctypes.c_float)], ctypes.c_int),
    "fsi_batch_mpm_substep": ([_BATCH, ctypes.POINTER(Particles), _VP, _VP, _VP], ctypes.c_int),
    "fsi_batch_coupling_forces": ([_BATCH, ctypes.POINTER(Particles), _VP, _VP, _VP, _VP, _VP, _VP,
                                   ctypes.c_float, ctypes.c_int32, _VP], ctypes.c_int),
    "fsi_batch_coupling_assemble": ([_BATCH, _VP, ctypes.c_int32, _VP, _VP, _VP, _VP, _VP, _VP],
                                    ctypes.c_int),
    "fsi_batch_run_persistent": ([_BATCH, ctypes.POINTER(Particles), ctypes.POINTER(BatchState),
                                  ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                  ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                  ctypes.c_int64, _VP], ctypes.c_int),
}


class NativeError(RuntimeError):
    """A C ABI call returned a non-OK status."""


def library_path() -> Path:
    return Path(os.environ.get("FSI_GB300_LIB", str(_LIB_PATH)))


def load():
    """Load and bind the native library; raises RuntimeError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise RuntimeError(
            f"native library {path} is missing: build it with "
            "`python taichi-mpm-lbm_gb300/build_native.py` (no CPU fallback exists)."
        )
    lib = ctypes.CDLL(str(path))
    for name, (argtypes, restype) in _SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.argtypes = argtypes
        fn.restype = restype
    if lib.fsi_abi_version() != ABI_VERSION:
        raise RuntimeError(f"{path}: ABI version {lib.fsi_abi_version()} != {ABI_VERSION}")
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGNATURES)


def last_error() -> str:
    lib = load()
    buf = ctypes.create_string_buffer(512)
    lib.fsi_last_error(buf, 512)
    return buf.value.decode(errors="replace")


# Number of successful calls per entry point (read by the benchmark to count launches).
CALLS: collections.Counter = collections.Counter()


def call(name: str, *args) -> None:
    """Invoke an entry point and translate its status into a Python exception."""
    lib = load()
    status = getattr(lib, name)(*args)
    CALLS[name] += 1
    if status != FSI_OK:
        msg = f"{name} failed ({status}): {last_error()}"
        if status == FSI_ERR_INVALID_ARG:
            raise ValueError(msg)
        raise NativeError(msg)


def device() -> torch.device:
    """The CUDA device the solvers allocate on; raises if CUDA is unavailable."""
    if not torch.cuda.is_available():
        raise RuntimeError(
            "fsi requires a CUDA device (sm_103a); this build has no CPU fallback."
        )
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


def ptr(t: torch.Tensor | None):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def vec3(values) -> ctypes.Array:
    a = c_float3()
    for i in range(3):
        a[i] = float(values[i])
    return a
