"""Schema-v1 JSON reference datasets (API of the reference's fsi/reference.py:1-249).

A dataset holds scalar metrics with per-metric absolute/relative tolerances; a
current value passes when either its absolute or its relative error is within
tolerance.
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any

from .validation import ValidationMetric, ValidationReport

SCHEMA_VERSION = 1


@dataclass(frozen=True)
class ReferenceMetricTolerance:
    abs: float = 0.0
    rel: float = 0.0

    def to_dict(self) -> dict[str, float]:
        return {"abs": float(self.abs), "rel": float(self.rel)}


@dataclass(frozen=True)
class ReferenceDataset:
    schema_version: int
    case_name: str
    description: str
    metrics: dict[str, float]
    tolerances: dict[str, ReferenceMetricTolerance]
    metadata: dict[str, Any] = field(default_factory=dict)
    created_by: str = ""

    def to_dict(self) -> dict[str, Any]:
        out: dict[str, Any] = {
            "schema_version": int(self.schema_version),
            "case_name": self.case_name,
            "description": self.description,
            "metrics": {k: float(self.metrics[k]) for k in sorted(self.metrics)},
            "tolerances": {k: self.tolerances[k].to_dict() for k in sorted(self.tolerances)},
        }
        if self.created_by:
            out["created_by"] = self.created_by
        if self.metadata:
            out["metadata"] = self.metadata
        return out


@dataclass(frozen=True)
class ReferenceComparison:
    case_name: str
    metric_name: str
    value: float
    reference: float
    abs_error: float
    rel_error: float
    abs_tolerance: float
    rel_tolerance: float
    passed: bool

    def to_dict(self) -> dict[str, Any]:
        return {
            "case_name": self.case_name,
            "metric_name": self.metric_name,
            "value": self.value,
            "reference": self.reference,
            "abs_error": self.abs_error,
            "rel_error": self.rel_error,
            "abs_tolerance": self.abs_tolerance,
            "rel_tolerance": self.rel_tolerance,
            "passed": self.passed,
        }


@dataclass(frozen=True)
class ReferenceReport:
    case_name: str
    comparisons: tuple[ReferenceComparison, ...]
    metadata: dict[str, Any] = field(default_factory=dict)

    @property
    def passed(self) -> bool:
        return all(c.passed for c in self.comparisons)

    def to_dict(self) -> dict[str, Any]:
        return {
            "case_name": self.case_name,
            "passed": self.passed,
            "comparisons": [c.to_dict() for c in self.comparisons],
            "metadata": self.metadata,
        }


def _need(data: dict[str, Any], key: str) -> Any:
    if key not in data:
        raise ValueError(f"Missing required reference field: {key}.")
    return data[key]


def _as_float(value: Any, what: str) -> float:
    try:
        return float(value)
    except (TypeError, ValueError) as exc:
        raise ValueError(f"{what} must be numeric.") from exc


def _tolerance(name: str, raw: Any) -> ReferenceMetricTolerance:
    if not isinstance(raw, dict):
        raise ValueError(f"Tolerance for {name} must be an object.")
    return ReferenceMetricTolerance(
        abs=_as_float(raw.get("abs", 0.0), f"tolerances.{name}.abs"),
        rel=_as_float(raw.get("rel", 0.0), f"tolerances.{name}.rel"),
    )


def load_reference_dataset(path: str | Path) -> ReferenceDataset:
    raw = json.loads(Path(path).read_text(encoding="utf-8"))
    if not isinstance(raw, dict):
        raise ValueError("reference dataset JSON must contain an object.")
    version = int(_need(raw, "schema_version"))
    if version != SCHEMA_VERSION:
        raise ValueError(f"Unsupported reference schema_version: {version}.")
    metrics_raw = _need(raw, "metrics")
    tol_raw = _need(raw, "tolerances")
    if not isinstance(metrics_raw, dict) or not metrics_raw:
        raise ValueError("reference metrics must be a non-empty object.")
    if not isinstance(tol_raw, dict):
        raise ValueError("reference tolerances must be an object.")
    metrics = {str(k): _as_float(v, f"metrics.{k}") for k, v in metrics_raw.items()}
    tolerances = {}
    for name in metrics:
        if name not in tol_raw:
            raise ValueError(f"Missing tolerance for reference metric: {name}.")
        tolerances[name] = _tolerance(name, tol_raw[name])
    metadata = raw.get("metadata", {})
    if not isinstance(metadata, dict):
        raise ValueError("reference metadata must be an object when provided.")
    return ReferenceDataset(
        schema_version=version,
        case_name=str(_need(raw, "case_name")),
        description=str(_need(raw, "description")),
        metrics=metrics,
        tolerances=tolerances,
        metadata=metadata,
        created_by=str(raw.get("created_by", "")),
    )


def save_reference_dataset(dataset: ReferenceDataset, path: str | Path) -> Path:
    out = Path(path)
    out.parent.mkdir(parents=True, exist_ok=True)
    out.write_text(json.dumps(dataset.to_dict(), indent=2, sort_keys=True) + "\n", encoding="utf-8")
    return out


def compare_metrics(case_name: str, current: dict[str, float],
                    reference: ReferenceDataset) -> ReferenceReport:
    comparisons = []
    for name, ref_value in reference.metrics.items():
        if name not in current:
            raise KeyError(f"Missing current metric for reference comparison: {name}.")
        value, ref = float(current[name]), float(ref_value)
        abs_err = abs(value - ref)
        rel_err = abs_err if ref == 0.0 else abs_err / abs(ref)
        tol = reference.tolerances[name]
        comparisons.append(ReferenceComparison(
            case_name=case_name, metric_name=name, value=value, reference=ref,
            abs_error=abs_err, rel_error=rel_err, abs_tolerance=float(tol.abs),
            rel_tolerance=float(tol.rel),
            passed=bool(abs_err <= float(tol.abs) or rel_err <= float(tol.rel)),
        ))
    return ReferenceReport(
        case_name=case_name,
        comparisons=tuple(comparisons),
        metadata={"reference_case_name": reference.case_name,
                  "reference_description": reference.description, **reference.metadata},
    )


def _effective_abs_tolerance(c: ReferenceComparison) -> float:
    if c.reference == 0.0:
        return max(c.abs_tolerance, c.rel_tolerance)
    return max(c.abs_tolerance, abs(c.reference) * c.rel_tolerance)


def reference_report_to_validation_report(report: ReferenceReport) -> ValidationReport:
    metrics = tuple(
        ValidationMetric(
            name=f"{c.metric_name}_abs_error",
            value=c.abs_error,
            upper=_effective_abs_tolerance(c),
            passed=c.passed,
            description=f"Reference comparison for {c.metric_name}.",
        )
        for c in report.comparisons
    )
    return ValidationReport(case_name=f"reference_{report.case_name}", metrics=metrics,
                            metadata=report.metadata)
