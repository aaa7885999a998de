"""Scalar validation metrics and reports (API of the reference's fsi/validation.py:8-101)."""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Any


@dataclass(frozen=True)
class ValidationMetric:
    """One named scalar with optional inclusive bounds and its pass/fail verdict."""

    name: str
    value: float
    lower: float | None = None
    upper: float | None = None
    passed: bool = True
    units: str = ""
    description: str = ""

    def to_dict(self) -> dict[str, Any]:
        return {
            "name": self.name,
            "value": self.value,
            "lower": self.lower,
            "upper": self.upper,
            "passed": self.passed,
            "units": self.units,
            "description": self.description,
        }


@dataclass(frozen=True)
class ValidationReport:
    """The metrics of one validation case; it passes when every metric passes."""

    case_name: str
    metrics: tuple[ValidationMetric, ...]
    metadata: dict[str, Any] = field(default_factory=dict)

    @property
    def passed(self) -> bool:
        return all(m.passed for m in self.metrics)

    def to_dict(self) -> dict[str, Any]:
        return {
            "case_name": self.case_name,
            "passed": self.passed,
            "metrics": [m.to_dict() for m in self.metrics],
            "metadata": self.metadata,
        }


def bounded_metric(name: str, value: float, *, lower: float | None = None,
                   upper: float | None = None, units: str = "",
                   description: str = "") -> ValidationMetric:
    """A metric that passes when finite and within ``[lower, upper]`` (either bound optional)."""
    v = float(value)
    ok = math.isfinite(v)
    if ok and lower is not None and v < float(lower):
        ok = False
    if ok and upper is not None and v > float(upper):
        ok = False
    return ValidationMetric(name=name, value=v, lower=lower, upper=upper, passed=bool(ok),
                            units=units, description=description)


def finite_metric(name: str, value: float, *, upper: float | None = None, units: str = "",
                  description: str = "") -> ValidationMetric:
    """A metric that passes when finite and not above ``upper``."""
    return bounded_metric(name, value, upper=upper, units=units, description=description)


def relative_error(value: float, reference: float) -> float:
    """|value - reference| / |reference|, or the absolute difference when reference is 0."""
    v, r = float(value), float(reference)
    if r == 0.0:
        return abs(v - r)
    return abs((v - r) / r)
