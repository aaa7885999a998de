"""Lattice-unit conversion placeholder (reference fsi/units.py): the solvers run in lattice units."""
from __future__ import annotations


class LatticeUnits:
    """Placeholder for physical-to-lattice unit conversion."""
