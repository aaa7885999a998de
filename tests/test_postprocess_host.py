"""Snapshot output and offline analysis on the host (fsi/output.py, fsi/postprocess.py): the
writer's interval and field groups, and the analysis functions of the reference's
fsi/postprocess.py (listing, metadata, time series, coupling counts, CSV / JSON export,
validation tables) on snapshots written by the writer from a stub simulation."""
from __future__ import annotations

import csv
import json

import numpy as np
import pytest

from fsi import postprocess as pp
from fsi.config import OutputConfig
from fsi.output import SimulationOutputWriter
from test_output_writer import stub_sim


def write_run(tmp_path, steps=(0, 5, 10), **flags):
    w = SimulationOutputWriter(OutputConfig(output_dir=tmp_path, output_interval=5, **flags))
    return [w.write_snapshot(stub_sim(s, seed=s))[0] for s in steps]


def test_writer_interval_and_format_checks(tmp_path):
    w = SimulationOutputWriter(OutputConfig(output_dir=tmp_path, output_interval=5))
    assert [s for s in range(12) if w.should_write(s)] == [0, 5, 10]
    with pytest.raises(ValueError, match="output_interval"):
        OutputConfig(output_interval=0).validate()
    with pytest.raises(ValueError, match="Unsupported output format"):
        OutputConfig(output_format="hdf5").validate()


def test_writer_field_groups(tmp_path):
    (path,) = write_run(tmp_path, steps=(3,), write_lbm_fields=False, write_coupling_fields=False)
    with np.load(path) as z:
        keys = set(z.files)
    assert {"step", "time", "lbm_shape", "mpm_particle_count", "mpm_positions"} <= keys
    assert not any(k.startswith("lbm_") and k != "lbm_shape" for k in keys)
    assert "coupling_force" not in keys and "ib_total_force" not in keys
    assert path.name == "snapshot_000003.npz"


def test_listing_orders_by_step_number(tmp_path):
    for name in ("snapshot_10.npz", "snapshot_9.npz", "snapshot_100.npz", "notes.npz"):
        np.savez(tmp_path / name, step=np.array(0))
    assert [p.name for p in pp.list_npz_snapshots(tmp_path)] == \
        ["snapshot_9.npz", "snapshot_10.npz", "snapshot_100.npz"]
    assert pp.list_npz_snapshots(tmp_path / "missing") == []


def test_snapshot_metadata(tmp_path):
    paths = write_run(tmp_path)
    infos = pp.summarize_snapshots(tmp_path)
    assert [i.step for i in infos] == [0, 5, 10]
    assert infos[1].time == 5.0 and infos[1].particle_count == 7
    assert infos[0].lbm_shape == (6, 5, 4) and infos[0].path == paths[0]
    assert pp.snapshot_info(paths[2]).to_dict()["step"] == 10
    data = pp.load_npz_snapshot(paths[0])
    assert data["lbm_density"].shape == (6, 5, 4)


def test_timeseries_from_full_snapshots(tmp_path):
    paths = write_run(tmp_path)
    ts = pp.extract_snapshot_timeseries(tmp_path)
    assert list(ts["step"]) == [0, 5, 10]
    assert list(ts)[:3] == ["step", "time", "mpm_particle_count"]
    snap = pp.load_npz_snapshot(paths[1])
    assert ts["lbm_mean_density"][1] == pytest.approx(1.0)
    assert ts["lbm_total_mass_estimate"][1] == pytest.approx(6 * 5 * 4)
    com = snap["mpm_positions"].astype(np.float64).mean(axis=0)
    assert ts["mpm_center_of_mass_y"][1] == pytest.approx(com[1])
    vmax = np.linalg.norm(snap["lbm_velocity"].reshape(-1, 3).astype(np.float64), axis=1).max()
    assert ts["lbm_max_velocity_norm"][1] == pytest.approx(vmax)
    assert list(ts["coupling_partial_support_particle_count"]) == [3, 3, 3]
    assert ts["coupling_force_norm"][1] == pytest.approx(np.linalg.norm(snap["coupling_force"]))
    counts = pp.summarize_coupling_diagnostics(tmp_path)
    assert list(counts)[:2] == ["step", "time"]
    assert list(counts["contact_candidate_count"]) == [2, 2, 2]
    assert "lbm_mean_density" not in counts


def test_timeseries_keeps_only_quantities_of_every_snapshot(tmp_path):
    write_run(tmp_path, steps=(0, 5))
    write_run(tmp_path, steps=(10,), write_coupling_fields=False)
    ts = pp.extract_snapshot_timeseries(tmp_path)
    assert list(ts["step"]) == [0, 5, 10]
    assert "lbm_mean_density" in ts and "coupling_force_norm" not in ts
    empty = pp.extract_snapshot_timeseries(tmp_path / "none")
    assert set(empty) == {"step", "time", "mpm_particle_count"} and empty["step"].size == 0


def test_timeseries_csv_and_json(tmp_path):
    write_run(tmp_path / "run")
    ts = pp.extract_snapshot_timeseries(tmp_path / "run")
    c = pp.write_timeseries_csv(ts, tmp_path / "out" / "ts.csv")
    with c.open() as fh:
        rows = list(csv.DictReader(fh))
    assert [int(r["step"]) for r in rows] == [0, 5, 10]
    assert float(rows[1]["lbm_mean_density"]) == pytest.approx(1.0)
    j = pp.write_timeseries_json(ts, tmp_path / "out" / "ts.json")
    back = json.loads(j.read_text())
    assert back["step"] == [0, 5, 10] and set(back) == set(ts)
    with pytest.raises(ValueError, match="same length"):
        pp.write_timeseries_csv({"step": np.arange(3), "time": np.arange(2.0)}, tmp_path / "x.csv")
    with pytest.raises(ValueError, match="empty"):
        pp.write_timeseries_json({}, tmp_path / "x.json")


def test_validation_summary_table_and_csv(tmp_path):
    reports = [
        {"case_name": "lbm_mass", "passed": True,
         "metrics": [{"name": "relative_mass_error", "value": 1e-7, "lower": None, "upper": 1e-5,
                      "passed": True, "units": "", "description": "mass drift"}]},
        {"case_name": "mpm_gravity", "passed": False,
         "metrics": [{"name": "dy", "value": 0.1, "lower": -1.0, "upper": 0.0, "passed": False},
                     {"name": "finite", "value": 1.0, "passed": True}]},
    ]
    src = tmp_path / "summary.json"
    src.write_text(json.dumps(reports))
    rows = pp.validation_summary_table(pp.load_validation_summary(src))
    assert [(r["case_name"], r["metric_name"], r["metric_passed"]) for r in rows] == [
        ("lbm_mass", "relative_mass_error", True), ("mpm_gravity", "dy", False),
        ("mpm_gravity", "finite", True)]
    assert rows[1]["case_passed"] is False and rows[2]["units"] == ""
    out = pp.write_validation_summary_csv(rows, tmp_path / "t" / "summary.csv")
    with out.open() as fh:
        back = list(csv.DictReader(fh))
    assert list(back[0]) == ["case_name", "case_passed", "metric_name", "value", "lower",
                             "upper", "metric_passed", "units", "description"]
    assert back[0]["upper"] == "1e-05" and back[2]["value"] == "1.0"
    bad = tmp_path / "bad.json"
    bad.write_text(json.dumps({"case_name": "x"}))
    with pytest.raises(ValueError, match="list"):
        pp.load_validation_summary(bad)


def test_plot_checks_its_keys_before_plotting(tmp_path):
    ts = {"step": np.arange(3), "lbm_mean_density": np.ones(3)}
    with pytest.raises(KeyError, match="y_key"):
        pp.plot_timeseries(ts, "missing", tmp_path / "p.png")
    with pytest.raises(KeyError, match="x_key"):
        pp.plot_timeseries(ts, "lbm_mean_density", tmp_path / "p.png", x_key="time")
    pytest.importorskip("matplotlib")
    out = pp.plot_timeseries(ts, "lbm_mean_density", tmp_path / "plots" / "p.png")
    assert out.exists() and out.stat().st_size > 0
