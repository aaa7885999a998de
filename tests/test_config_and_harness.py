"""Configuration validation, reference-dataset harness and validation metrics (CPU only).

Mirrors the reference's tests/test_config.py, tests/test_reference_validation.py
(dataset I/O and comparison parts) and tests/test_validation_benchmarks.py
(metric helpers).
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import pytest

from fsi.config import (BoundaryConfig, CouplingConfig, LBMConfig, MPMConfig, OutputConfig,
                        SimulationConfig)
from fsi.postprocess import validation_summary_table
from fsi.reference import (ReferenceDataset, ReferenceMetricTolerance, compare_metrics,
                           load_reference_dataset, reference_report_to_validation_report,
                           save_reference_dataset)
from fsi.reference_cases import default_reference_data_dir
from fsi.validation import ValidationReport, bounded_metric, finite_metric, relative_error

PKG = Path(__file__).resolve().parents[1] / "taichi-mpm-lbm_gb300" / "fsi"


def test_defaults_validate_and_mpm_dt():
    SimulationConfig().validate()
    cfg = SimulationConfig(lbm_dt=1.0, coupling=CouplingConfig(mpm_substeps_per_lbm_step=4))
    assert cfg.mpm_dt == pytest.approx(0.25)
    assert SimulationConfig().num_steps == 1000


@pytest.mark.parametrize("bad", [
    LBMConfig(viscosity=0.0), LBMConfig(initial_velocity=(0.0, 1.0)), LBMConfig(nx=4),
    MPMConfig(poisson_ratio=0.5), MPMConfig(boundary_width=0), MPMConfig(boundary_damping=1.5),
    CouplingConfig(gamma=-1.0), CouplingConfig(force_limit=0.0),
    CouplingConfig(relative_velocity_limit=0.0), CouplingConfig(gamma_ramp_steps=-1),
    CouplingConfig(min_valid_weight=0.0), CouplingConfig(min_valid_weight=1.1),
    CouplingConfig(immersed_boundary_drag=-1.0),
    CouplingConfig(immersed_boundary_fraction_threshold=-0.1),
    CouplingConfig(immersed_boundary_fraction_threshold=1.1),
    CouplingConfig(immersed_boundary_max_force=0.0), CouplingConfig(contact_velocity_damping=-0.1),
    CouplingConfig(contact_velocity_damping=1.1), CouplingConfig(contact_fraction_threshold=-0.1),
    CouplingConfig(contact_fraction_threshold=1.1), OutputConfig(output_interval=0),
    OutputConfig(output_format="bad"), BoundaryConfig(velocity=(0.0, 1.0)),
    BoundaryConfig("velocity", velocity_update="in_order"),
    MPMConfig(constitutive_model="plastic"),
    LBMConfig(population_storage="f8"), LBMConfig(collision_arithmetic="approx"),
    LBMConfig(population_storage="f16", collision_arithmetic="exact"),
    LBMConfig(mrt_rates={9: 1.5}), LBMConfig(mrt_rates={4: 2.5}),
    SimulationConfig(lbm=LBMConfig(nx=64, ny=32, nz=16), mpm=MPMConfig(nx=32, ny=32, nz=16)),
])
def test_invalid_configs_raise_value_error(bad):
    with pytest.raises(ValueError):
        bad.validate()


def test_library_never_initialises_a_runtime():
    for path in PKG.glob("*.py"):
        src = path.read_text()
        assert "ti.init(" not in src and "taichi.init(" not in src


def _sample() -> ReferenceDataset:
    return ReferenceDataset(1, "sample_reference", "Sample reference dataset.",
                            {"x": 10.0, "zero": 0.0},
                            {"x": ReferenceMetricTolerance(0.1, 0.01),
                             "zero": ReferenceMetricTolerance(1.0e-6, 0.0)},
                            {"steps": 1}, "test")


def test_dataset_round_trip_and_rejections(tmp_path):
    loaded = load_reference_dataset(save_reference_dataset(_sample(), tmp_path / "s.json"))
    assert loaded.case_name == "sample_reference" and loaded.metadata == {"steps": 1}
    assert loaded.tolerances["x"].rel == pytest.approx(0.01)
    bad = _sample().to_dict()
    bad["schema_version"] = 2
    (tmp_path / "b.json").write_text(json.dumps(bad))
    with pytest.raises(ValueError):
        load_reference_dataset(tmp_path / "b.json")
    miss = _sample().to_dict()
    del miss["tolerances"]["x"]
    (tmp_path / "m.json").write_text(json.dumps(miss))
    with pytest.raises(ValueError):
        load_reference_dataset(tmp_path / "m.json")


def test_compare_metrics_and_bridge():
    ok = compare_metrics("sample_reference", {"x": 10.05, "zero": 5.0e-7}, _sample())
    bad = compare_metrics("sample_reference", {"x": 11.0, "zero": 2.0e-6}, _sample())
    assert ok.passed and not bad.passed
    assert bad.comparisons[0].abs_error == pytest.approx(1.0)
    assert bad.comparisons[0].rel_error == pytest.approx(0.1)
    with pytest.raises(KeyError):
        compare_metrics("sample_reference", {"x": 10.0}, _sample())
    vr = reference_report_to_validation_report(ok)
    rows = validation_summary_table([vr.to_dict()])
    assert vr.case_name == "reference_sample_reference" and vr.passed
    assert rows[0]["metric_name"].endswith("_abs_error")
    rel = ReferenceDataset(1, "r", "r", {"x": 100.0}, {"x": ReferenceMetricTolerance(0.1, 0.01)})
    v = reference_report_to_validation_report(compare_metrics("r", {"x": 100.5}, rel))
    assert v.metrics[0].upper == pytest.approx(1.0) and v.metrics[0].passed


def test_committed_goldens_load():
    paths = sorted(default_reference_data_dir().glob("*.json"))
    assert len(paths) == 6
    for p in paths:
        ds = load_reference_dataset(p)
        assert set(ds.metrics) == set(ds.tolerances)


def test_metric_helpers():
    assert bounded_metric("x", 0.5, lower=0.0, upper=1.0).passed
    assert not bounded_metric("x", 2.0, lower=0.0, upper=1.0).passed
    assert not bounded_metric("x", math.nan).passed
    assert not finite_metric("x", 2.0, upper=1.0).passed
    assert relative_error(11.0, 10.0) == pytest.approx(0.1)
    assert relative_error(0.0, 0.0) == 0.0
    rep = ValidationReport("sample", (bounded_metric("x", 0.5, lower=0.0, upper=1.0),), {"steps": 1})
    assert rep.to_dict()["passed"] is True


def test_package_exports():
    import fsi
    for name in ("SimulationConfig", "LBMConfig", "MPMConfig", "CouplingConfig", "LBMSolver3D",
                 "MPMSolver3D", "LBMMpmCoupler", "FSISimulation", "SimulationOutputWriter",
                 "ValidationMetric", "ValidationReport", "run_validation_suite"):
        assert hasattr(fsi, name)
    for name in ("SnapshotInfo", "list_npz_snapshots", "extract_snapshot_timeseries",
                 "load_validation_summary", "validation_summary_table", "ReferenceDataset",
                 "ReferenceReport", "load_reference_dataset", "run_reference_validation_suite"):
        assert name in fsi.__all__


def test_storage_forms_resolve_their_arithmetic():
    assert LBMConfig().resolved_arithmetic() == "exact"
    assert LBMConfig(population_storage="bf16").resolved_arithmetic() == "fast"
    assert LBMConfig(collision_arithmetic="fast").resolved_arithmetic() == "fast"


def test_mrt_rate_overrides_touch_only_the_named_moments():
    import numpy as np
    from fsi.lbm3d import dhumieres_rates, relaxation_rates
    base = relaxation_rates(1 / 30)
    rates = relaxation_rates(1 / 30, dhumieres_rates(0.6))
    changed = {k for k in range(19) if rates[k] != base[k]}
    assert changed == {1, 2, 4, 6, 8, 16, 17, 18}  # s_pi = 1/tau equals the default at k=10, 12
    assert rates[4] == np.float32(1.2) and rates[16] == np.float32(1.98)
    LBMConfig(mrt_rates=dhumieres_rates(0.6)).validate()
