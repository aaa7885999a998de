"""Regenerate the committed golden fixtures.

The reference's own golden datasets (``data/reference/*.json`` of
lizhuoh9/taichi-mpm-lbm, schema v1 with per-metric tolerances) are copied
byte-for-byte into ``taichi-mpm-lbm_gb300/data/reference/``, where
``fsi.reference_cases.default_reference_data_dir()`` finds them. They are data
(metric values and tolerances produced by the reference's Taichi path), not
source.

Run from the repository root, naming a checkout of the reference:
    python tests/golden/make_golden.py /path/to/reference/checkout
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
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/reference/checkout")
    for p in copy_reference_goldens(Path(sys.argv[1])):
        print("wrote", p.relative_to(ROOT))
