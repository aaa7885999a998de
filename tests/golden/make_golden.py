"""Regenerate the committed golden fixtures.

1. The reference's own golden datasets (``data/reference/*.json`` of
   lizhuoh9/taichi-mpm-lbm, schema v1 with per-metric tolerances) are copied
   byte-for-byte into ``taichi-mpm-lbm_gb300/data/reference/``, where
   ``fsi.reference_cases.default_reference_data_dir()`` finds them. They are
   data (metric values and tolerances produced by the reference's Taichi
   path), not source.
2. ``oracle_fields_*.npz``: field-level vectors of the CPU oracle on small
   seeded cases, used by tests that must run without the oracle library.

Run from the repository root with the reference checkout available:
    python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import shutil
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
DEST = ROOT / "taichi-mpm-lbm_gb300" / "data" / "reference"


def copy_reference_goldens(reference_root: Path) -> list[Path]:
    src = reference_root / "data" / "reference"
    DEST.mkdir(parents=True, exist_ok=True)
    out = []
    for path in sorted(src.glob("*.json")):
        target = DEST / path.name
        shutil.copyfile(path, target)
        out.append(target)
    return out


if __name__ == "__main__":
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference")
    for p in copy_reference_goldens(ref):
        print("wrote", p.relative_to(ROOT))
