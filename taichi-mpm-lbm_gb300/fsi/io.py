"""Filesystem helpers (reference fsi/io.py)."""
from __future__ import annotations

from pathlib import Path


def ensure_output_dir(path: Path) -> None:
    Path(path).mkdir(parents=True, exist_ok=True)
