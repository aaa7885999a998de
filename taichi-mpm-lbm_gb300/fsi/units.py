"""Physical <-> lattice unit conversion for setting up scenes.

The reference's ``fsi/units.py`` declares an empty ``LatticeUnits`` placeholder: its solvers,
like these, run in lattice units (dx = dt = 1, the fluid's rest density rho0 = 1). This
class keeps that name and its no-argument construction (the identity conversion) and adds
the scale factors a physical set-up needs: a lattice cell of ``dx`` metres, a lattice step
of ``dt`` seconds and a reference density of ``rho`` kg/m^3. A D3Q19 BGK/MRT lattice has
c_s^2 = 1/3, so the shear viscosity of relaxation time tau is (tau - 1/2) / 3.
"""
from __future__ import annotations

from dataclasses import dataclass

CS2 = 1.0 / 3.0  # lattice speed of sound squared


@dataclass(frozen=True)
class LatticeUnits:
    dx: float = 1.0   # metres per lattice cell
    dt: float = 1.0   # seconds per lattice step
    rho: float = 1.0  # kg/m^3 that lattice density 1 stands for

    def __post_init__(self):
        for name in ("dx", "dt", "rho"):
            if not getattr(self, name) > 0.0:
                raise ValueError(f"{name} must be positive.")

    # kinematics
    def length(self, metres: float) -> float:
        return metres / self.dx

    def steps(self, seconds: float) -> float:
        return seconds / self.dt

    def velocity(self, metres_per_second: float) -> float:
        return metres_per_second * self.dt / self.dx

    def velocity_si(self, lattice_velocity: float) -> float:
        return lattice_velocity * self.dx / self.dt

    def acceleration(self, metres_per_second2: float) -> float:
        """Body acceleration, e.g. gravity for MPMConfig.gravity."""
        return metres_per_second2 * self.dt * self.dt / self.dx

    # fluid
    def viscosity(self, m2_per_second: float) -> float:
        return m2_per_second * self.dt / (self.dx * self.dx)

    def tau(self, m2_per_second: float) -> float:
        """LBMConfig.tau that gives kinematic viscosity ``m2_per_second``."""
        return self.viscosity(m2_per_second) / CS2 + 0.5

    def viscosity_si(self, tau: float) -> float:
        return (tau - 0.5) * CS2 * self.dx * self.dx / self.dt

    def force_density(self, newtons_per_m3: float) -> float:
        """Force per unit volume, e.g. a pressure gradient for LBMConfig.force."""
        return newtons_per_m3 * self.dt * self.dt / (self.rho * self.dx)

    # solid
    def density(self, kg_per_m3: float) -> float:
        """MPM particle density relative to the fluid's reference density."""
        return kg_per_m3 / self.rho

    def stress(self, pascals: float) -> float:
        """Stress or modulus, e.g. MPMConfig.youngs_modulus."""
        return pascals * self.dt * self.dt / (self.rho * self.dx * self.dx)

    def stress_si(self, lattice_stress: float) -> float:
        return lattice_stress * self.rho * self.dx * self.dx / (self.dt * self.dt)

    def mach(self, lattice_velocity: float) -> float:
        """Lattice Mach number u / c_s (keep well under 0.3 for the weakly compressible
        lattice)."""
        return abs(lattice_velocity) / CS2 ** 0.5
