"""fsi -- coupled LBM-MPM fluid-solid timestep on NVIDIA GB300 (sm_103a).

Drop-in for the Python API of lizhuoh9/taichi-mpm-lbm: the same configuration
dataclasses, solver classes and runner, with storage in torch CUDA tensors and
every kernel implemented as hand-written CUDA behind a C ABI
(include/fsi_gb300.h). Solver classes are imported lazily so that the
configuration and validation helpers work without a GPU.
"""
from importlib import import_module
from typing import TYPE_CHECKING

from .config import (
    BoundaryConfig,
    CouplingConfig,
    LBMConfig,
    MPMConfig,
    OutputConfig,
    SimulationConfig,
)

if TYPE_CHECKING:
    from .coupling import LBMMpmCoupler
    from .lbm3d import LBMSolver3D
    from .mpm3d import MPMSolver3D
    from .output import SimulationOutputWriter
    from .postprocess import (SnapshotInfo, extract_snapshot_timeseries, list_npz_snapshots,
                              load_validation_summary, validation_summary_table)
    from .reference import ReferenceDataset, ReferenceReport, load_reference_dataset
    from .reference_cases import run_reference_validation_suite
    from .simulation import FSISimulation
    from .validation import ValidationMetric, ValidationReport
    from .validation_cases import run_validation_suite

__all__ = [
    "BoundaryConfig",
    "CouplingConfig",
    "FSISimulation",
    "LBMConfig",
    "LBMMpmCoupler",
    "LBMSolver3D",
    "MPMConfig",
    "MPMSolver3D",
    "OutputConfig",
    "ReferenceDataset",
    "ReferenceReport",
    "SimulationConfig",
    "SimulationOutputWriter",
    "SnapshotInfo",
    "ValidationMetric",
    "ValidationReport",
    "extract_snapshot_timeseries",
    "list_npz_snapshots",
    "load_reference_dataset",
    "load_validation_summary",
    "run_reference_validation_suite",
    "run_validation_suite",
    "validation_summary_table",
]

_LAZY = {
    "LBMSolver3D": "lbm3d",
    "MPMSolver3D": "mpm3d",
    "LBMMpmCoupler": "coupling",
    "FSISimulation": "simulation",
    "SimulationOutputWriter": "output",
    "SnapshotInfo": "postprocess",
    "list_npz_snapshots": "postprocess",
    "extract_snapshot_timeseries": "postprocess",
    "load_validation_summary": "postprocess",
    "validation_summary_table": "postprocess",
    "ReferenceDataset": "reference",
    "ReferenceReport": "reference",
    "load_reference_dataset": "reference",
    "ValidationMetric": "validation",
    "ValidationReport": "validation",
    "run_validation_suite": "validation_cases",
    "run_reference_validation_suite": "reference_cases",
}


def __getattr__(name: str):
    module = _LAZY.get(name)
    if module is None:
        raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
    value = getattr(import_module(f".{module}", __name__), name)
    globals()[name] = value
    return value
