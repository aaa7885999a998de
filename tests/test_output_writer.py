"""Snapshot writer (fsi/output.py): NPZ keys of the reference's writer (output.py:39-116), and
background writing giving the same files as synchronous writing. Runs on CPU with a stub
simulation exposing the accessors the writer reads."""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np

from fsi.config import OutputConfig
from fsi.output import SimulationOutputWriter


def stub_sim(step: int, seed: int = 0):
    rng = np.random.default_rng(seed)
    shape = (6, 5, 4)
    f3 = lambda: rng.standard_normal((*shape, 3)).astype(np.float32)  # noqa: E731
    lbm = SimpleNamespace(nx=6, ny=5, nz=4,
                          density_numpy=lambda: np.ones(shape, np.float32),
                          velocity_numpy=f3, force_numpy=f3,
                          solid_numpy=lambda: np.zeros(shape, np.int32))
    p = 7
    mpm = SimpleNamespace(dx=1.0, particle_count=lambda: p,
                          positions_numpy=lambda: rng.random((p, 3)).astype(np.float32),
                          velocities_numpy=lambda: np.zeros((p, 3), np.float32),
                          particle_forces_numpy=lambda: np.zeros((p, 3), np.float32),
                          deformation_gradients_numpy=lambda: np.tile(np.eye(3, dtype=np.float32), (p, 1, 1)),
                          active_numpy=lambda: np.ones(p, np.int32))
    diag = {"ib_total_force_x": 0.0, "ib_total_force_y": 0.0, "ib_total_force_z": 0.0,
            "ib_active_cell_count": 1, "ib_clipped_cell_count": 0, "contact_candidate_count": 2,
            "contact_damped_particle_count": 0, "unsupported_particle_count": 0,
            "partial_support_particle_count": 3, "clipped_particle_count": 0}
    cp = SimpleNamespace(coupling_diagnostics=lambda: diag, coupling_force_numpy=f3,
                         solid_volume_fraction_numpy=lambda: np.zeros(shape, np.float32),
                         immersed_boundary_force_numpy=f3,
                         total_particle_coupling_force=lambda: np.zeros(3, np.float32),
                         total_fluid_coupling_force=lambda: np.zeros(3, np.float32),
                         particle_valid_weights_numpy=lambda: np.ones(p, np.float32),
                         particle_coupling_mask_numpy=lambda: np.ones(p, np.int32),
                         particle_contact_mask_numpy=lambda: np.zeros(p, np.int32))
    return SimpleNamespace(step_index=step, time=float(step), lbm=lbm, mpm=mpm, coupler=cp)


def test_background_writes_match_synchronous(tmp_path):
    sync = SimulationOutputWriter(OutputConfig(output_dir=tmp_path / "sync"))
    back = SimulationOutputWriter(OutputConfig(output_dir=tmp_path / "async", async_write=True))
    paths = []
    for step in (100, 200, 300):
        a = sync.write_snapshot(stub_sim(step, seed=step))
        b = back.write_snapshot(stub_sim(step, seed=step))
        paths.append((a[0], b[0]))
    back.flush()
    for a, b in paths:
        assert a.name == b.name
        with np.load(a) as za, np.load(b) as zb:
            assert sorted(za.files) == sorted(zb.files)
            for key in za.files:
                np.testing.assert_array_equal(za[key], zb[key])
    with np.load(paths[0][0]) as z:
        for key in ("step", "time", "lbm_density", "lbm_velocity", "mpm_positions",
                    "coupling_force", "coupling_partial_support_particle_count"):
            assert key in z.files
        assert int(z["coupling_partial_support_particle_count"]) == 3
