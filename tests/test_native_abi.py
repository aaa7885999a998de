"""The C-ABI library builds, loads without a GPU and exports every declared entry point."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

from fsi import _native

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "fsi_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|size_t)\s+(fsi_\w+)\s*\(", text, flags=re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "fsi_lbm_step" in names and "fsi_mpm_substep" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol():
    lib = _native.load()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(_native.exported_symbols())


def test_abi_version_and_error_channel():
    lib = _native.load()
    assert lib.fsi_abi_version() == _native.ABI_VERSION
    buf = ctypes.create_string_buffer(64)
    lib.fsi_last_error(buf, 64)  # callable without a GPU


def test_invalid_descriptor_is_rejected_without_touching_the_gpu():
    d = _native.LbmDesc()
    d.nx = d.ny = d.nz = 2  # too small
    with pytest.raises(ValueError, match="too small"):
        _native.call("fsi_lbm_step", d, None, None, None, None, None, 0, None)


def test_unknown_face_mode_is_rejected_without_touching_the_gpu():
    d = _native.LbmDesc()
    d.nx = d.ny = d.nz = 8
    d.bc_mode_left = 4
    with pytest.raises(ValueError, match="unknown x boundary mode 4"):
        _native.call("fsi_lbm_step", d, None, None, None, None, None, 0, None)


def test_struct_sizes_match_header_layout():
    assert ctypes.sizeof(_native.LbmDesc) == 4 * (5 + 19 + 3 + 6 + 2)
    assert ctypes.sizeof(_native.BatchLattice) == 4 * 4 + 8 + 4 * (19 + 1 + 3) + 4  # + tail pad
    assert ctypes.sizeof(_native.MpmDesc) == 4 * 22  # + launch_threads, coupling_fold
    assert ctypes.sizeof(_native.Particles) == 8 * 11
    assert ctypes.sizeof(_native.CouplingDesc) == 4 * 18


def test_closure_row_buffer_size():
    """fsi_closure_rows_bytes (host only): 3 chunks x 16 bytes per row of the lattice padded to
    whole inference columns (11 lines in y, 32 cells in z) plus one periodic image per side;
    -1 for lattices the closure rejects."""
    lib = _native.load()
    for nx, ny, nz in [(12, 10, 10), (192, 96, 96), (40, 30, 70), (5, 11, 32)]:
        d = _native.LbmDesc()
        d.nx, d.ny, d.nz = nx, ny, nz
        d.storage = _native.STORAGE_F32
        ny_pad = 11 * -(-ny // 11) + 2
        nz_pad = 32 * -(-nz // 32) + 2
        assert lib.fsi_closure_rows_bytes(ctypes.byref(d)) == 3 * nx * ny_pad * nz_pad * 16
    d = _native.LbmDesc()
    d.nx, d.ny, d.nz = 4, 10, 10  # too small
    assert lib.fsi_closure_rows_bytes(ctypes.byref(d)) == -1
    d.nx, d.ny, d.nz, d.storage = 12, 10, 10, _native.STORAGE_F16  # FP32 populations only
    assert lib.fsi_closure_rows_bytes(ctypes.byref(d)) == -1


def test_scene_context_layout_and_argument_checks():
    """fsi_scene_desc / fsi_scene_buffers layouts, and fsi_ctx_create / fsi_coupled_step
    rejecting bad arguments before any device work."""
    assert ctypes.sizeof(_native.SceneDesc) == 4 * (35 + 22 + 18) + 4 * (3 + 2 + 5)
    assert ctypes.sizeof(_native.SceneBuffers) == 8 * 5 + 8 * 11 + 8 * 6
    d, b = _native.SceneDesc(), _native.SceneBuffers()
    d.lbm.nx = d.lbm.ny = d.lbm.nz = 8
    d.mpm.nx, d.mpm.ny, d.mpm.nz = 8, 8, 4  # grid differs from the lattice
    handle = ctypes.c_void_p()
    with pytest.raises(ValueError, match="coincide"):
        _native.call("fsi_ctx_create", ctypes.byref(d), ctypes.byref(b), ctypes.byref(handle))
    d.mpm.nz = 8
    with pytest.raises(ValueError, match="NULL lattice buffer"):
        _native.call("fsi_ctx_create", ctypes.byref(d), ctypes.byref(b), ctypes.byref(handle))
    assert not handle.value
    with pytest.raises(ValueError, match="NULL context"):
        _native.call("fsi_coupled_step", None, 1.0, None, 10, 1, None)


def _mpm_desc(**kw):
    d = _native.MpmDesc()
    d.nx = d.ny = d.nz = 16
    d.num_particles = 0
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def _particles():
    p = _native.Particles()
    for f in ("x", "v", "C", "F", "mass", "volume", "active", "force"):
        setattr(p, f, 256)  # never dereferenced: validation fails first or no particles
    p.capacity = 0
    return p


@pytest.mark.parametrize("threads,fold,message", [(100, 0, "launch_threads"),
                                                  (256, 5, "coupling_fold")])
def test_launch_tuning_fields_are_validated_without_touching_the_gpu(threads, fold, message):
    d = _mpm_desc(launch_threads=threads, coupling_fold=fold)
    with pytest.raises(ValueError, match=message):
        _native.call("fsi_mpm_substep", d, _particles(), 256, 256, None)


def test_assembly_with_sum_requires_its_output():
    c, l = _native.CouplingDesc(), _native.LbmDesc()
    base = (ctypes.c_float * 3)()
    with pytest.raises(ValueError, match="NULL reaction"):
        _native.call("fsi_coupling_assemble_sum", c, l, None, base, 0, None, None, None, None,
                     None, None, None)


def test_persistent_batch_call_rejects_a_missing_batch():
    st = _native.BatchState()
    with pytest.raises(ValueError, match="invalid batch handle"):
        _native.call("fsi_batch_run_persistent", None, _particles(), st, 0, 1, 10, 0.1, 1, 2, 0,
                     0, 0, None)
    assert ctypes.sizeof(_native.BatchState) == 8 * 14
