"""NPZ / VTK snapshots of a coupled run (API of the reference's fsi/output.py:15-198).

Snapshots are host-side files built from the solvers' accessors. pyevtk is
imported only when a VTK snapshot is written, so the package works without it.
"""
from __future__ import annotations

from pathlib import Path
from typing import TYPE_CHECKING

import numpy as np

from .config import OutputConfig

if TYPE_CHECKING:
    from .simulation import FSISimulation


def _components(vectors: np.ndarray):
    return tuple(np.ascontiguousarray(vectors[..., a]) for a in range(3))


class SimulationOutputWriter:
    """Writes snapshot_*.npz and fluid_*.vti / particles_*.vtu files."""

    def __init__(self, config: OutputConfig):
        self.config = config
        self.config.validate()
        self.output_dir = Path(config.output_dir)
        self._pool = None
        self._pending: list = []

    def _save(self, path: Path, arrays: dict) -> None:
        if not getattr(self.config, "async_write", False):
            np.savez_compressed(path, **arrays)
            return
        if self._pool is None:
            from concurrent.futures import ThreadPoolExecutor
            self._pool = ThreadPoolExecutor(max_workers=1, thread_name_prefix="fsi-snapshot")
        self._pending.append(self._pool.submit(np.savez_compressed, path, **arrays))

    def flush(self) -> None:
        """Wait for snapshots still being written in the background; re-raises their errors."""
        pending, self._pending = self._pending, []
        for fut in pending:
            fut.result()

    def ensure_output_dir(self) -> None:
        self.output_dir.mkdir(parents=True, exist_ok=True)

    def should_write(self, step: int) -> bool:
        return int(step) % self.config.output_interval == 0

    def write_snapshot(self, sim: "FSISimulation") -> list[Path]:
        fmt = self.config.output_format
        if fmt == "npz":
            return [self.write_npz_snapshot(sim)]
        if fmt == "vtk":
            return self.write_vtk_snapshot(sim)
        if fmt == "both":
            return [self.write_npz_snapshot(sim), *self.write_vtk_snapshot(sim)]
        raise ValueError(f"Unsupported output format: {fmt}.")

    def write_npz_snapshot(self, sim: "FSISimulation") -> Path:
        self.ensure_output_dir()
        path = self.output_dir / f"snapshot_{sim.step_index:06d}.npz"
        arrays: dict[str, np.ndarray] = {
            "step": np.array(sim.step_index, dtype=np.int64),
            "time": np.array(sim.time, dtype=np.float64),
            "lbm_shape": np.array([sim.lbm.nx, sim.lbm.ny, sim.lbm.nz], dtype=np.int32),
            "mpm_particle_count": np.array(sim.mpm.particle_count(), dtype=np.int32),
        }
        if self.config.write_lbm_fields:
            arrays["lbm_density"] = sim.lbm.density_numpy()
            arrays["lbm_velocity"] = sim.lbm.velocity_numpy()
            arrays["lbm_force"] = sim.lbm.force_numpy()
            arrays["lbm_solid"] = sim.lbm.solid_numpy()
        if self.config.write_mpm_particles:
            arrays["mpm_positions"] = sim.mpm.positions_numpy()
            arrays["mpm_velocities"] = sim.mpm.velocities_numpy()
            arrays["mpm_particle_forces"] = sim.mpm.particle_forces_numpy()
            arrays["mpm_deformation_gradients"] = sim.mpm.deformation_gradients_numpy()
            arrays["mpm_active"] = sim.mpm.active_numpy()
        if self.config.write_coupling_fields:
            cp = sim.coupler
            d = cp.coupling_diagnostics()
            arrays.update({
                "coupling_force": cp.coupling_force_numpy(),
                "solid_volume_fraction": cp.solid_volume_fraction_numpy(),
                "immersed_boundary_force": cp.immersed_boundary_force_numpy(),
                "total_particle_coupling_force": cp.total_particle_coupling_force(),
                "total_fluid_coupling_force": cp.total_fluid_coupling_force(),
                "coupling_particle_valid_weight": cp.particle_valid_weights_numpy(),
                "coupling_particle_mask": cp.particle_coupling_mask_numpy(),
                "particle_contact_mask": cp.particle_contact_mask_numpy(),
                "ib_total_force": np.array([d["ib_total_force_x"], d["ib_total_force_y"],
                                            d["ib_total_force_z"]], dtype=np.float32),
            })
            for key, src in (("ib_active_cell_count", "ib_active_cell_count"),
                             ("ib_clipped_cell_count", "ib_clipped_cell_count"),
                             ("contact_candidate_count", "contact_candidate_count"),
                             ("contact_damped_particle_count", "contact_damped_particle_count"),
                             ("coupling_unsupported_particle_count", "unsupported_particle_count"),
                             ("coupling_partial_support_particle_count",
                              "partial_support_particle_count"),
                             ("coupling_clipped_particle_count", "clipped_particle_count")):
                arrays[key] = np.array(d[src], dtype=np.int32)
        self._save(path, arrays)
        return path

    def write_vtk_snapshot(self, sim: "FSISimulation") -> list[Path]:
        paths = []
        if self.config.write_lbm_fields or self.config.write_coupling_fields:
            paths.append(self._write_fluid_vtk(sim, sim.step_index))
        if self.config.write_mpm_particles:
            paths.append(self._write_particles_vtk(sim, sim.step_index))
        return paths

    def _write_fluid_vtk(self, sim: "FSISimulation", step: int) -> Path:
        from pyevtk.hl import imageToVTK

        self.ensure_output_dir()
        cells = {}
        if self.config.write_lbm_fields:
            cells["rho"] = np.ascontiguousarray(sim.lbm.density_numpy())
            cells["velocity"] = _components(sim.lbm.velocity_numpy())
            cells["force"] = _components(sim.lbm.force_numpy())
            cells["solid"] = np.ascontiguousarray(sim.lbm.solid_numpy())
        if self.config.write_coupling_fields:
            cells["coupling_force"] = _components(sim.coupler.coupling_force_numpy())
            cells["solid_volume_fraction"] = np.ascontiguousarray(
                sim.coupler.solid_volume_fraction_numpy())
            cells["immersed_boundary_force"] = _components(
                sim.coupler.immersed_boundary_force_numpy())
        name = imageToVTK(str(self.output_dir / f"fluid_{step:06d}"), origin=(0.0, 0.0, 0.0),
                          spacing=(sim.mpm.dx,) * 3, cellData=cells)
        return Path(name)

    def _write_particles_vtk(self, sim: "FSISimulation", step: int) -> Path:
        from pyevtk.hl import pointsToVTK

        self.ensure_output_dir()
        pos = np.ascontiguousarray(sim.mpm.positions_numpy())
        if len(pos) == 0:
            x = y = z = np.zeros(0, dtype=np.float32)
        else:
            x, y, z = (np.ascontiguousarray(pos[:, a]) for a in range(3))
        data = {"velocity": _components(sim.mpm.velocities_numpy()),
                "particle_force": _components(sim.mpm.particle_forces_numpy())}
        if self.config.write_coupling_fields:
            data["contact_mask"] = np.ascontiguousarray(sim.coupler.particle_contact_mask_numpy())
        name = pointsToVTK(str(self.output_dir / f"particles_{step:06d}"), x, y, z, data=data)
        return Path(name)
