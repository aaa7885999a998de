"""The ten small deterministic physics cases of the reference's fsi/validation_cases.py.

Each case builds the same configuration as the reference (validation_cases.py:88-581),
runs it through the solver classes named at module level, and reports the same
metric names and bounds. The committed golden datasets are built from these
cases (reference_cases.py).
"""
from __future__ import annotations

import numpy as np

from .config import BoundaryConfig, CouplingConfig, LBMConfig, MPMConfig, SimulationConfig
from .lbm3d import LBMSolver3D
from .mpm3d import MPMSolver3D
from .simulation import FSISimulation
from .validation import ValidationReport, bounded_metric, finite_metric, relative_error

_PERIODIC_FACES = {name: BoundaryConfig("periodic")
                   for name in ("x_left", "x_right", "y_left", "y_right", "z_left", "z_right")}


def _periodic_lbm_config(**overrides) -> LBMConfig:
    params = dict(nx=8, ny=8, nz=8, viscosity=0.1, rho0=1.0, force=(0.0, 0.0, 0.0),
                  initial_velocity=(0.0, 0.0, 0.0), **_PERIODIC_FACES)
    params.update(overrides)
    return LBMConfig(**params)


def _mpm_config(**overrides) -> MPMConfig:
    params = dict(nx=16, ny=16, nz=16, max_particles=10_000, dx=1.0, dt=1.0e-3, density=1.0,
                  youngs_modulus=1_000.0, poisson_ratio=0.25, gravity=(0.0, 0.0, 0.0),
                  boundary_width=2)
    params.update(overrides)
    return MPMConfig(**params)


def _small_mpm_config() -> MPMConfig:
    return MPMConfig(nx=8, ny=8, nz=8, max_particles=128, dx=1.0, dt=1.0e-3, density=1.0,
                     youngs_modulus=100.0, poisson_ratio=0.25, gravity=(0.0, 0.0, 0.0),
                     boundary_width=1)


def _coupled_config(*, enabled: bool = True) -> SimulationConfig:
    return SimulationConfig(
        num_steps=2,
        lbm_dt=0.1,
        lbm=_periodic_lbm_config(initial_velocity=(1.0e-3, 0.0, 0.0)),
        mpm=_small_mpm_config(),
        coupling=CouplingConfig(enabled=enabled, gamma=5.0, mpm_substeps_per_lbm_step=1),
    )


def _one_particle(sim, position=(4.0, 4.0, 4.0), velocity=(0.0, 0.0, 0.0), volume=1.0):
    sim.initialize_mpm_from_numpy(
        positions=np.array([position], dtype=np.float32),
        velocities=np.array([velocity], dtype=np.float32),
        particle_mass=1.0,
        particle_volume=volume,
    )


def _initialized_one_particle_simulation(config: SimulationConfig):
    sim = FSISimulation(config)
    _one_particle(sim)
    sim.initialize_lbm()
    return sim


def _force_balance_norm(coupler) -> float:
    integrated = coupler.total_fluid_coupling_force() * coupler.cell_volume
    return float(np.linalg.norm(coupler.total_particle_coupling_force() + integrated))


def run_lbm_mass_conservation_case() -> ValidationReport:
    steps = 20
    solver = LBMSolver3D(_periodic_lbm_config())
    solver.initialize()
    mass0 = solver.total_mass()
    for _ in range(steps):
        solver.step()
    mass1 = solver.total_mass()
    return ValidationReport(
        case_name="lbm_periodic_mass_conservation",
        metrics=(
            bounded_metric("relative_mass_error", relative_error(mass1, mass0), upper=1.0e-5,
                           description="Periodic lattice: change of total mass relative to the start."),
            finite_metric("max_velocity_norm", solver.max_velocity_norm(), upper=1.0e-4,
                          description="Largest fluid speed stays finite and close to zero."),
        ),
        metadata={"steps": steps, "grid": [solver.nx, solver.ny, solver.nz]},
    )


def run_lbm_force_response_case() -> ValidationReport:
    steps = 20
    solver = LBMSolver3D(_periodic_lbm_config(force=(1.0e-6, 0.0, 0.0)))
    solver.initialize()
    ux0 = float(solver.velocity_numpy()[..., 0].mean())
    for _ in range(steps):
        solver.step()
    ux1 = float(solver.velocity_numpy()[..., 0].mean())
    return ValidationReport(
        case_name="lbm_force_response",
        metrics=(
            bounded_metric("mean_ux_growth", ux1 - ux0, lower=1.0e-12,
                           description="A positive x body force raises the mean x velocity."),
            finite_metric("max_velocity_norm", solver.max_velocity_norm(), upper=1.0e-2,
                          description="The forced flow speed stays bounded."),
        ),
        metadata={"steps": steps, "grid": [solver.nx, solver.ny, solver.nz]},
    )


def run_mpm_zero_gravity_com_case() -> ValidationReport:
    steps = 10
    solver = MPMSolver3D(_mpm_config(gravity=(0.0, 0.0, 0.0), dt=1.0e-3))
    solver.initialize_particles_box((6.0, 6.0, 6.0), (10.0, 10.0, 10.0), spacing=1.0)
    com0 = solver.center_of_mass()
    for _ in range(steps):
        solver.substep()
    com1 = solver.center_of_mass()
    return ValidationReport(
        case_name="mpm_zero_gravity_com_stability",
        metrics=(
            bounded_metric("center_of_mass_drift_norm", float(np.linalg.norm(com1 - com0)),
                           upper=1.0e-3, units="grid",
                           description="Centre of mass barely moves with no gravity and no initial velocity."),
            finite_metric("max_velocity_norm", solver.max_velocity_norm(), upper=1.0e-3,
                          description="Particle speeds stay bounded with gravity off."),
        ),
        metadata={"steps": steps, "particle_count": solver.particle_count()},
    )


def run_mpm_gravity_response_case() -> ValidationReport:
    steps = 10
    solver = MPMSolver3D(_mpm_config(gravity=(0.0, -1.0e-3, 0.0), dt=1.0e-2))
    solver.initialize_particles_box((6.0, 8.0, 6.0), (10.0, 12.0, 10.0), spacing=1.0)
    com0 = solver.center_of_mass()
    for _ in range(steps):
        solver.substep()
    com1 = solver.center_of_mass()
    positions = solver.positions_numpy()
    velocities = solver.velocities_numpy()
    return ValidationReport(
        case_name="mpm_gravity_response",
        metrics=(
            bounded_metric("center_of_mass_y_delta", float(com1[1] - com0[1]), upper=-1.0e-12,
                           units="grid",
                           description="A weak -y gravity lowers the centre of mass."),
            bounded_metric("positions_finite", 1.0 if np.isfinite(positions).all() else 0.0,
                           lower=1.0, upper=1.0,
                           description="No particle position becomes NaN or infinite."),
            bounded_metric("velocities_finite", 1.0 if np.isfinite(velocities).all() else 0.0,
                           lower=1.0, upper=1.0,
                           description="No particle velocity becomes NaN or infinite."),
        ),
        metadata={"steps": steps, "particle_count": solver.particle_count()},
    )


def run_coupled_drift_case() -> ValidationReport:
    enabled = _initialized_one_particle_simulation(_coupled_config(enabled=True))
    disabled = _initialized_one_particle_simulation(_coupled_config(enabled=False))
    x_on0 = float(enabled.mpm.center_of_mass()[0])
    x_off0 = float(disabled.mpm.center_of_mass()[0])
    enabled.run(steps=2)
    disabled.run(steps=2)
    enabled_dx = float(enabled.mpm.center_of_mass()[0] - x_on0)
    disabled_dx = float(disabled.mpm.center_of_mass()[0] - x_off0)
    return ValidationReport(
        case_name="coupled_enabled_vs_disabled_drift",
        metrics=(
            bounded_metric("enabled_dx", enabled_dx, lower=1.0e-7, units="grid",
                           description="With coupling on, the +x flow carries the particle in +x."),
            bounded_metric("disabled_dx_abs", abs(disabled_dx), upper=1.0e-6, units="grid",
                           description="With coupling off, the particle stays put."),
            bounded_metric("enabled_minus_disabled_dx", enabled_dx - disabled_dx, lower=1.0e-7,
                           units="grid",
                           description="Coupling on moves the particle farther than coupling off."),
        ),
        metadata={"steps": 2, "gamma": 5.0, "initial_lbm_ux": 1.0e-3},
    )


def run_coupling_force_balance_case() -> ValidationReport:
    sim = _initialized_one_particle_simulation(_coupled_config(enabled=True))
    sim.coupler.compute_coupling_forces(dt_ratio=1.0)
    particle_force = sim.coupler.total_particle_coupling_force()
    fluid_force = sim.coupler.total_fluid_coupling_force() * sim.coupler.cell_volume
    return ValidationReport(
        case_name="coupling_force_balance",
        metrics=(
            bounded_metric("particle_force_x", float(particle_force[0]), lower=1.0e-12,
                           description="A uniform +x flow pushes the particle in +x."),
            bounded_metric("fluid_force_x", float(fluid_force[0]), upper=-1.0e-12,
                           description="The fluid takes the equal and opposite x reaction."),
            bounded_metric("force_balance_norm", _force_balance_norm(sim.coupler), upper=1.0e-6,
                           description="Particle force and summed fluid reaction cancel."),
        ),
        metadata={"dt_ratio": 1.0, "cell_volume": sim.coupler.cell_volume},
    )


def _unit_flow_config(coupling: CouplingConfig) -> SimulationConfig:
    return SimulationConfig(num_steps=1, lbm_dt=0.1,
                            lbm=_periodic_lbm_config(initial_velocity=(1.0, 0.0, 0.0)),
                            mpm=_small_mpm_config(), coupling=coupling)


def run_coupling_force_limit_case() -> ValidationReport:
    config = _unit_flow_config(CouplingConfig(gamma=100.0, force_limit=0.05,
                                              mpm_substeps_per_lbm_step=1))
    sim = _initialized_one_particle_simulation(config)
    sim.coupler.compute_coupling_forces(dt_ratio=1.0)
    particle_force = sim.coupler.total_particle_coupling_force()
    diagnostics = sim.coupler.coupling_diagnostics()
    return ValidationReport(
        case_name="coupling_force_limit",
        metrics=(
            bounded_metric("particle_force_norm", float(np.linalg.norm(particle_force)),
                           upper=0.05 + 1.0e-7,
                           description="A large penalty gamma triggers the force clip."),
            bounded_metric("clipped_particle_count", float(diagnostics["clipped_particle_count"]),
                           lower=1.0,
                           description="The clip counter records at least one particle."),
            bounded_metric("force_balance_norm", _force_balance_norm(sim.coupler), upper=1.0e-6,
                           description="After clipping, particle force and fluid reaction still cancel."),
        ),
        metadata={"gamma": 100.0, "force_limit": 0.05},
    )


def run_coupling_boundary_support_case() -> ValidationReport:
    config = _unit_flow_config(CouplingConfig(gamma=1.0, min_valid_weight=1.0e-6,
                                              mpm_substeps_per_lbm_step=1))
    sim = FSISimulation(config)
    _one_particle(sim, position=(-0.75, 4.0, 4.0))
    sim.initialize_lbm()
    sim.coupler.compute_coupling_forces(dt_ratio=1.0)
    particle_force = sim.coupler.total_particle_coupling_force()
    diagnostics = sim.coupler.coupling_diagnostics()
    return ValidationReport(
        case_name="coupling_boundary_support",
        metrics=(
            bounded_metric("partial_support_particle_count",
                           float(diagnostics["partial_support_particle_count"]), lower=1.0,
                           description="A particle by the grid edge is counted as partially supported."),
            bounded_metric("min_particle_valid_weight",
                           float(diagnostics["min_particle_valid_weight"]), lower=1.0e-6,
                           upper=1.0 - 1.0e-5,
                           description="Its valid weight is positive and below one."),
            bounded_metric("force_balance_norm", _force_balance_norm(sim.coupler), upper=1.0e-6,
                           description="With partial support, particle force and fluid reaction still cancel."),
            bounded_metric("particle_force_finite",
                           1.0 if np.isfinite(particle_force).all() else 0.0, lower=1.0,
                           upper=1.0, description="The edge particle's force stays finite."),
        ),
        metadata={"particle_position": [-0.75, 4.0, 4.0], "min_valid_weight": 1.0e-6},
    )


def _short_config(lbm_velocity, coupling: CouplingConfig) -> SimulationConfig:
    return SimulationConfig(num_steps=1, lbm_dt=1.0e-3,
                            lbm=_periodic_lbm_config(initial_velocity=lbm_velocity),
                            mpm=_small_mpm_config(), coupling=coupling)


def run_immersed_boundary_drag_case() -> ValidationReport:
    config = _short_config((1.0e-3, 0.0, 0.0), CouplingConfig(
        gamma=0.0, mpm_substeps_per_lbm_step=1, immersed_boundary_enabled=True,
        immersed_boundary_drag=0.1, immersed_boundary_fraction_threshold=0.01,
        immersed_boundary_max_force=1.0e-3))
    sim = FSISimulation(config)
    sim.initialize_lbm()
    _one_particle(sim, volume=4.0)
    initial_speed = sim.lbm.max_velocity_norm()
    sim.step()
    diagnostics = sim.coupler.coupling_diagnostics()
    velocity = sim.lbm.velocity_numpy()
    return ValidationReport(
        case_name="immersed_boundary_drag",
        metrics=(
            bounded_metric("ib_active_cell_count", float(diagnostics["ib_active_cell_count"]),
                           lower=1.0,
                           description="Some fluid cell covered by the body gets immersed-boundary drag."),
            bounded_metric("ib_total_force_x", float(diagnostics["ib_total_force_x"]),
                           upper=-1.0e-12,
                           description="The immersed-boundary drag points against the +x flow."),
            bounded_metric("ib_total_force_norm", float(diagnostics["ib_total_force_norm"]),
                           lower=1.0e-12, description="The summed immersed-boundary drag is not zero."),
            bounded_metric("max_velocity_not_increased",
                           float(sim.lbm.max_velocity_norm() - initial_speed), upper=1.0e-8,
                           description="Immersed-boundary drag does not speed up the fluid."),
            bounded_metric("velocity_finite", 1.0 if np.isfinite(velocity).all() else 0.0,
                           lower=1.0, upper=1.0,
                           description="Fluid velocity stays finite with immersed-boundary drag on."),
        ),
        metadata={"drag": 0.1, "particle_volume": 4.0},
    )


def run_contact_diagnostics_case() -> ValidationReport:
    config = _short_config((0.0, 0.0, 0.0), CouplingConfig(
        gamma=0.0, mpm_substeps_per_lbm_step=1, contact_enabled=True,
        contact_velocity_damping=0.25, contact_fraction_threshold=0.01))
    solid = np.zeros((8, 8, 8), dtype=np.int32)
    solid[3:6, 3:6, 3:6] = 1
    sim = FSISimulation(config)
    sim.initialize_lbm(solid_np=solid)
    _one_particle(sim, velocity=(0.1, 0.0, 0.0))
    initial_speed = sim.mpm.max_velocity_norm()
    sim.step()
    final_speed = sim.mpm.max_velocity_norm()
    diagnostics = sim.coupler.coupling_diagnostics()
    contact_mask_sum = float(sim.coupler.particle_contact_mask_numpy().sum())
    return ValidationReport(
        case_name="contact_diagnostics",
        metrics=(
            bounded_metric("contact_candidate_count",
                           float(diagnostics["contact_candidate_count"]), lower=1.0,
                           description="Support from static solid flags at least one contact candidate."),
            bounded_metric("contact_damped_particle_count",
                           float(diagnostics["contact_damped_particle_count"]), lower=1.0,
                           description="At least one particle is damped on contact."),
            bounded_metric("particle_contact_mask_sum", contact_mask_sum, lower=1.0,
                           description="The contact mask of the particle is set."),
            bounded_metric("particle_speed_delta", float(final_speed - initial_speed),
                           upper=-1.0e-6, description="Contact damping slows the particle."),
        ),
        metadata={"damping": 0.25, "initial_speed": initial_speed},
    )


def run_validation_suite() -> list[ValidationReport]:
    return [
        run_lbm_mass_conservation_case(),
        run_lbm_force_response_case(),
        run_mpm_zero_gravity_com_case(),
        run_mpm_gravity_response_case(),
        run_coupled_drift_case(),
        run_coupling_force_balance_case(),
        run_coupling_force_limit_case(),
        run_coupling_boundary_support_case(),
        run_immersed_boundary_drag_case(),
        run_contact_diagnostics_case(),
    ]
