"""Offline analysis of NPZ snapshots and validation summaries.

Same public functions as the reference's fsi/postprocess.py (snapshot listing,
time-series extraction, CSV/JSON export, validation tables, optional
matplotlib plots). Host-side numpy only; not part of the timestep.
"""
from __future__ import annotations

import csv
import json
from dataclasses import dataclass
from pathlib import Path
from typing import Any

import numpy as np

_PREFERRED = (
    "step", "time", "mpm_particle_count", "lbm_mean_density", "lbm_total_mass_estimate",
    "lbm_max_velocity_norm", "mpm_center_of_mass_x", "mpm_center_of_mass_y",
    "mpm_center_of_mass_z", "mpm_max_velocity_norm", "coupling_force_norm",
    "total_particle_coupling_force_norm", "total_fluid_coupling_force_norm",
    "coupling_unsupported_particle_count", "coupling_partial_support_particle_count",
    "coupling_clipped_particle_count", "ib_force_norm", "ib_total_force_norm",
    "ib_active_cell_count", "ib_clipped_cell_count", "contact_candidate_count",
    "contact_damped_particle_count",
)
_COUNT_KEYS = (
    "coupling_unsupported_particle_count", "coupling_partial_support_particle_count",
    "coupling_clipped_particle_count", "ib_active_cell_count", "ib_clipped_cell_count",
    "contact_candidate_count", "contact_damped_particle_count",
)
_VALIDATION_FIELDS = ["case_name", "case_passed", "metric_name", "value", "lower", "upper",
                      "metric_passed", "units", "description"]


@dataclass(frozen=True)
class SnapshotInfo:
    """Metadata of one NPZ snapshot."""

    path: Path
    step: int
    time: float
    particle_count: int
    lbm_shape: tuple[int, int, int]

    def to_dict(self) -> dict[str, Any]:
        return {"path": str(self.path), "step": self.step, "time": self.time,
                "particle_count": self.particle_count, "lbm_shape": self.lbm_shape}


def _scalar(value) -> Any:
    return np.asarray(value).reshape(()).item()


def _sort_key(path: Path):
    stem = path.stem
    tail = stem[len("snapshot_"):] if stem.startswith("snapshot_") else ""
    return (0, int(tail)) if tail.isdigit() else (1, path.name)


def list_npz_snapshots(output_dir: str | Path) -> list[Path]:
    """snapshot_*.npz files of a directory, ordered by step number."""
    d = Path(output_dir)
    return sorted(d.glob("snapshot_*.npz"), key=_sort_key) if d.exists() else []


def load_npz_snapshot(path: str | Path) -> dict[str, np.ndarray]:
    with np.load(Path(path), allow_pickle=False) as data:
        return {k: np.array(data[k]) for k in data.files}


def snapshot_info(path: str | Path) -> SnapshotInfo:
    data = load_npz_snapshot(path)
    shape = tuple(int(v) for v in np.asarray(data["lbm_shape"]).reshape(-1))
    if len(shape) != 3:
        raise ValueError(f"lbm_shape must have 3 entries, got {shape}.")
    return SnapshotInfo(path=Path(path), step=int(_scalar(data["step"])),
                        time=float(_scalar(data["time"])),
                        particle_count=int(_scalar(data["mpm_particle_count"])), lbm_shape=shape)


def summarize_snapshots(output_dir: str | Path) -> list[SnapshotInfo]:
    return [snapshot_info(p) for p in list_npz_snapshots(output_dir)]


def _max_norm(value) -> float:
    a = np.asarray(value, dtype=np.float64)
    if a.size == 0:
        return 0.0
    return float(np.linalg.norm(a.reshape(-1, a.shape[-1]), axis=1).max())


def _row(path: Path) -> dict[str, float | int]:
    d = load_npz_snapshot(path)
    row: dict[str, float | int] = {"step": int(_scalar(d["step"])), "time": float(_scalar(d["time"])),
                                   "mpm_particle_count": int(_scalar(d["mpm_particle_count"]))}
    if "lbm_density" in d:
        rho = np.asarray(d["lbm_density"])
        row["lbm_mean_density"] = float(np.mean(rho))
        row["lbm_total_mass_estimate"] = float(np.sum(rho))
    if "lbm_velocity" in d:
        row["lbm_max_velocity_norm"] = _max_norm(d["lbm_velocity"])
    if "mpm_positions" in d and np.asarray(d["mpm_positions"]).size:
        com = np.mean(np.asarray(d["mpm_positions"], dtype=np.float64), axis=0)
        row["mpm_center_of_mass_x"], row["mpm_center_of_mass_y"], row["mpm_center_of_mass_z"] = (
            float(com[0]), float(com[1]), float(com[2]))
    if "mpm_velocities" in d:
        row["mpm_max_velocity_norm"] = _max_norm(d["mpm_velocities"])
    for key, name in (("coupling_force", "coupling_force_norm"),
                      ("immersed_boundary_force", "ib_force_norm"),
                      ("total_particle_coupling_force", "total_particle_coupling_force_norm"),
                      ("total_fluid_coupling_force", "total_fluid_coupling_force_norm"),
                      ("ib_total_force", "ib_total_force_norm")):
        if key in d:
            row[name] = float(np.linalg.norm(np.asarray(d[key])))
    for key in _COUNT_KEYS:
        if key in d:
            row[key] = int(_scalar(d[key]))
    return row


def _ordered(keys) -> list[str]:
    keys = set(keys)
    out = [k for k in _PREFERRED if k in keys]
    return out + sorted(keys.difference(out))


def extract_snapshot_timeseries(output_dir: str | Path) -> dict[str, np.ndarray]:
    """One array per quantity present in every snapshot, ordered by step."""
    rows = [_row(p) for p in list_npz_snapshots(output_dir)]
    if not rows:
        return {"step": np.array([], dtype=np.int64), "time": np.array([], dtype=np.float64),
                "mpm_particle_count": np.array([], dtype=np.int64)}
    common = set(rows[0]).intersection(*[set(r) for r in rows[1:]])
    return {k: np.array([r[k] for r in rows]) for k in _ordered(common)}


def summarize_coupling_diagnostics(output_dir: str | Path) -> dict[str, np.ndarray]:
    ts = extract_snapshot_timeseries(output_dir)
    wanted = ["step", "time", "coupling_force_norm", "total_particle_coupling_force_norm",
              "total_fluid_coupling_force_norm", *(_COUNT_KEYS[:3]), "ib_force_norm",
              "ib_total_force_norm", *(_COUNT_KEYS[3:])]
    return {k: ts[k] for k in wanted if k in ts}


def _plain(value: Any) -> Any:
    if isinstance(value, dict):
        return {k: _plain(v) for k, v in value.items()}
    if isinstance(value, (list, tuple)):
        return [_plain(v) for v in value]
    if isinstance(value, np.ndarray):
        return value.tolist()
    if isinstance(value, np.generic):
        return value.item()
    return value


def _check_series(ts: dict[str, np.ndarray]) -> list[str]:
    if not ts:
        raise ValueError("time series must not be empty.")
    keys = _ordered(ts)
    if len({len(np.asarray(ts[k])) for k in keys}) != 1:
        raise ValueError("all time series arrays must have the same length.")
    return keys


def write_timeseries_csv(timeseries: dict[str, np.ndarray], path: str | Path) -> Path:
    keys = _check_series(timeseries)
    out = Path(path)
    out.parent.mkdir(parents=True, exist_ok=True)
    n = len(np.asarray(timeseries[keys[0]]))
    with out.open("w", newline="", encoding="utf-8") as fh:
        w = csv.DictWriter(fh, fieldnames=keys)
        w.writeheader()
        for i in range(n):
            w.writerow({k: _plain(np.asarray(timeseries[k])[i]) for k in keys})
    return out


def write_timeseries_json(timeseries: dict[str, np.ndarray], path: str | Path) -> Path:
    _check_series(timeseries)
    out = Path(path)
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text(json.dumps(_plain(timeseries), indent=2), encoding="utf-8")
    return out


def load_validation_summary(path: str | Path) -> list[dict[str, Any]]:
    data = json.loads(Path(path).read_text(encoding="utf-8"))
    if not isinstance(data, list):
        raise ValueError("validation summary JSON must contain a list of reports.")
    return data


def validation_summary_table(reports: list[dict[str, Any]]) -> list[dict[str, Any]]:
    """One row per metric of each validation report dict."""
    rows = []
    for rep in reports:
        for m in rep.get("metrics", []):
            rows.append({
                "case_name": rep.get("case_name", ""),
                "case_passed": bool(rep.get("passed", False)),
                "metric_name": m.get("name", ""),
                "value": m.get("value"),
                "lower": m.get("lower"),
                "upper": m.get("upper"),
                "metric_passed": bool(m.get("passed", False)),
                "units": m.get("units", ""),
                "description": m.get("description", ""),
            })
    return rows


def write_validation_summary_csv(rows: list[dict[str, Any]], path: str | Path) -> Path:
    out = Path(path)
    out.parent.mkdir(parents=True, exist_ok=True)
    with out.open("w", newline="", encoding="utf-8") as fh:
        w = csv.DictWriter(fh, fieldnames=_VALIDATION_FIELDS)
        w.writeheader()
        for r in rows:
            w.writerow({k: _plain(r.get(k)) for k in _VALIDATION_FIELDS})
    return out


def plot_timeseries(timeseries: dict[str, np.ndarray], y_key: str, output_path: str | Path, *,
                    x_key: str = "step") -> Path:
    """PNG line plot of one series (needs matplotlib)."""
    for k, what in ((x_key, "x_key"), (y_key, "y_key")):
        if k not in timeseries:
            raise KeyError(f"Missing {what} in time series: {k}.")
    import matplotlib.pyplot as plt

    out = Path(output_path)
    out.parent.mkdir(parents=True, exist_ok=True)
    fig, ax = plt.subplots()
    ax.plot(np.asarray(timeseries[x_key]), np.asarray(timeseries[y_key]), marker="o")
    ax.set_xlabel(x_key)
    ax.set_ylabel(y_key)
    ax.grid(True)
    fig.tight_layout()
    fig.savefig(out)
    plt.close(fig)
    return out
