"""Committed golden datasets and their regeneration (reference fsi/reference_cases.py:1-235)."""
from __future__ import annotations

from pathlib import Path

from . import validation_cases as _cases
from .reference import (
    ReferenceDataset,
    ReferenceMetricTolerance as Tol,
    ReferenceReport,
    compare_metrics,
    load_reference_dataset,
    save_reference_dataset,
)
from .validation import ValidationReport

STEP11_CREATED_BY = "fsi-lbm-mpm Step 11 reference generator"
STEP12_CREATED_BY = "fsi-lbm-mpm Step 12 reference generator"


def default_reference_data_dir() -> Path:
    """Directory of the committed golden datasets (``data/reference`` beside the package)."""
    return Path(__file__).resolve().parents[1] / "data" / "reference"


def _pick(report: ValidationReport, names: tuple[str, ...]) -> dict[str, float]:
    values = {m.name: float(m.value) for m in report.metrics}
    return {n: values[n] for n in names}


def compute_lbm_periodic_mass_reference_metrics() -> dict[str, float]:
    return _pick(_cases.run_lbm_mass_conservation_case(),
                 ("relative_mass_error", "max_velocity_norm"))


def compute_lbm_force_response_reference_metrics() -> dict[str, float]:
    return _pick(_cases.run_lbm_force_response_case(), ("mean_ux_growth", "max_velocity_norm"))


def compute_mpm_gravity_reference_metrics() -> dict[str, float]:
    return _pick(_cases.run_mpm_gravity_response_case(),
                 ("center_of_mass_y_delta", "positions_finite", "velocities_finite"))


def compute_coupled_drift_reference_metrics() -> dict[str, float]:
    return _pick(_cases.run_coupled_drift_case(),
                 ("enabled_dx", "disabled_dx_abs", "enabled_minus_disabled_dx"))


def compute_coupling_stability_reference_metrics() -> dict[str, float]:
    out = _pick(_cases.run_coupling_force_limit_case(),
                ("particle_force_norm", "force_balance_norm"))
    out.update(_pick(_cases.run_coupling_boundary_support_case(),
                     ("partial_support_particle_count", "min_particle_valid_weight")))
    return out


def compute_immersed_boundary_contact_reference_metrics() -> dict[str, float]:
    out = _pick(_cases.run_immersed_boundary_drag_case(),
                ("ib_active_cell_count", "ib_total_force_x", "ib_total_force_norm"))
    out.update(_pick(_cases.run_contact_diagnostics_case(),
                     ("contact_candidate_count", "contact_damped_particle_count")))
    return out


def build_reference_datasets() -> list[ReferenceDataset]:
    """Recompute every golden dataset from the current implementation (tolerances as committed)."""
    return [
        ReferenceDataset(1, "lbm_periodic_mass_reference",
                         "Small periodic LBM mass conservation reference.",
                         compute_lbm_periodic_mass_reference_metrics(),
                         {"relative_mass_error": Tol(1.0e-5, 0.0),
                          "max_velocity_norm": Tol(1.0e-4, 0.0)},
                         {"source_case": "lbm_periodic_mass_conservation", "steps": 20},
                         STEP11_CREATED_BY),
        ReferenceDataset(1, "lbm_force_response_reference",
                         "Small forced periodic LBM velocity-growth reference.",
                         compute_lbm_force_response_reference_metrics(),
                         {"mean_ux_growth": Tol(1.0e-8, 1.0e-2),
                          "max_velocity_norm": Tol(1.0e-8, 1.0e-2)},
                         {"source_case": "lbm_force_response", "steps": 20}, STEP11_CREATED_BY),
        ReferenceDataset(1, "mpm_gravity_reference", "Weak-gravity MPM response reference.",
                         compute_mpm_gravity_reference_metrics(),
                         {"center_of_mass_y_delta": Tol(1.0e-6, 1.0e-2),
                          "positions_finite": Tol(0.0, 0.0),
                          "velocities_finite": Tol(0.0, 0.0)},
                         {"source_case": "mpm_gravity_response", "steps": 10}, STEP11_CREATED_BY),
        ReferenceDataset(1, "coupled_drift_reference",
                         "Enabled-vs-disabled coupling drift reference.",
                         compute_coupled_drift_reference_metrics(),
                         {"enabled_dx": Tol(1.0e-6, 5.0e-2), "disabled_dx_abs": Tol(1.0e-6, 0.0),
                          "enabled_minus_disabled_dx": Tol(1.0e-6, 5.0e-2)},
                         {"source_case": "coupled_enabled_vs_disabled_drift", "steps": 2},
                         STEP11_CREATED_BY),
        ReferenceDataset(1, "coupling_stability_reference",
                         "Step 9 force-limit and boundary-support reference.",
                         compute_coupling_stability_reference_metrics(),
                         {"particle_force_norm": Tol(1.0e-7, 1.0e-3),
                          "force_balance_norm": Tol(1.0e-6, 0.0),
                          "partial_support_particle_count": Tol(0.0, 0.0),
                          "min_particle_valid_weight": Tol(1.0e-6, 1.0e-3)},
                         {"source_cases": ["coupling_force_limit", "coupling_boundary_support"]},
                         STEP11_CREATED_BY),
        ReferenceDataset(1, "immersed_boundary_contact_reference",
                         "Small Step 12 immersed-boundary/contact MVP reference.",
                         compute_immersed_boundary_contact_reference_metrics(),
                         {"ib_active_cell_count": Tol(0.0, 0.0),
                          "ib_total_force_x": Tol(1.0e-9, 1.0e-3),
                          "ib_total_force_norm": Tol(1.0e-9, 1.0e-3),
                          "contact_candidate_count": Tol(0.0, 0.0),
                          "contact_damped_particle_count": Tol(0.0, 0.0)},
                         {"source_cases": ["immersed_boundary_drag", "contact_diagnostics"]},
                         STEP12_CREATED_BY),
    ]


def generate_reference_datasets(output_dir: str | Path) -> list[Path]:
    """Write freshly computed datasets into ``output_dir`` (never over the committed ones)."""
    directory = Path(output_dir)
    return [save_reference_dataset(ds, directory / f"{ds.case_name}.json")
            for ds in build_reference_datasets()]


def _current_metrics_by_case() -> dict[str, dict[str, float]]:
    return {
        "lbm_periodic_mass_reference": compute_lbm_periodic_mass_reference_metrics(),
        "lbm_force_response_reference": compute_lbm_force_response_reference_metrics(),
        "mpm_gravity_reference": compute_mpm_gravity_reference_metrics(),
        "coupled_drift_reference": compute_coupled_drift_reference_metrics(),
        "coupling_stability_reference": compute_coupling_stability_reference_metrics(),
        "immersed_boundary_contact_reference": compute_immersed_boundary_contact_reference_metrics(),
    }


def run_reference_validation_suite(reference_dir: str | Path | None = None) -> list[ReferenceReport]:
    """Compare the current small-case metrics against the committed golden datasets."""
    directory = default_reference_data_dir() if reference_dir is None else Path(reference_dir)
    current = _current_metrics_by_case()
    datasets = [load_reference_dataset(p) for p in sorted(directory.glob("*.json"))]
    return [compare_metrics(ds.case_name, current[ds.case_name], ds) for ds in datasets]
