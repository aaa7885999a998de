"""fsi.units.LatticeUnits: the reference's placeholder name with real scale factors (host only)."""
from __future__ import annotations

import pytest

from fsi.units import LatticeUnits


def test_default_is_the_identity_of_lattice_units():
    u = LatticeUnits()
    assert u.velocity(0.05) == 0.05 and u.stress(0.1) == 0.1 and u.length(3.0) == 3.0
    assert u.tau(1.0 / 30.0) == pytest.approx(0.6)


def test_water_in_a_millimetre_lattice():
    u = LatticeUnits(dx=1e-3, dt=1e-4, rho=1000.0)
    assert u.viscosity(1e-6) == pytest.approx(1e-4)
    assert u.tau(1e-6) == pytest.approx(0.5003)
    assert u.viscosity_si(u.tau(1e-6)) == pytest.approx(1e-6)
    assert u.velocity(0.5) == pytest.approx(0.05)
    assert u.velocity_si(0.05) == pytest.approx(0.5)
    assert u.acceleration(9.81) == pytest.approx(9.81e-5)
    assert u.stress_si(u.stress(1e5)) == pytest.approx(1e5)
    assert u.stress(1e5) == pytest.approx(1e5 * 1e-8 / (1000.0 * 1e-6))
    assert u.force_density(1000.0 * 9.81) == pytest.approx(u.acceleration(9.81))
    assert u.density(1200.0) == pytest.approx(1.2)
    assert u.mach(0.05) == pytest.approx(0.05 * 3 ** 0.5)


@pytest.mark.parametrize("field", ["dx", "dt", "rho"])
def test_scales_must_be_positive(field):
    with pytest.raises(ValueError, match=field):
        LatticeUnits(**{field: 0.0})
