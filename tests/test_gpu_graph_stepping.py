"""Coupled stepping through a captured CUDA graph (LBMMpmCoupler.step_many, FSISimulation.advance)
against the eager step() loop on the same inputs.

The coupled step scatters with float atomics, so two eager runs already differ in the last
bits; the graph run is held to the same bounds as the coupled parity test (rho and x 1e-5,
u 2.5e-4 relative L2) and to identical host-side state."""
from __future__ import annotations

import numpy as np
import pytest

from fsi.config import CouplingConfig
from fsi.simulation import FSISimulation
from helpers import coupled_smoke_config, rel_l2

pytestmark = pytest.mark.gpu


def make(cfg, solid, pos, graph_steps=False):
    sim = FSISimulation(cfg)
    sim.graph_steps = graph_steps
    sim.initialize_lbm(solid)
    sim.initialize_mpm_from_numpy(pos)
    return sim


@pytest.mark.parametrize("ramp,steps", [(0, 9), (5, 12)])
def test_graph_steps_match_eager(ramp, steps):
    cfg, solid, pos = coupled_smoke_config(steps=steps)
    if ramp:
        import dataclasses
        cfg = dataclasses.replace(cfg, coupling=dataclasses.replace(cfg.coupling,
                                                                    gamma_ramp_steps=ramp))
    eager, graph = make(cfg, solid, pos), make(cfg, solid, pos)
    for _ in range(steps):
        eager.step()
    graph.advance(steps, graph=True)
    assert graph.step_index == eager.step_index == steps
    assert graph.time == eager.time
    assert graph.lbm.steps_done == eager.lbm.steps_done
    assert graph.coupler.coupled_step == eager.coupler.coupled_step
    assert graph.coupler.effective_gamma() == eager.coupler.effective_gamma()
    assert rel_l2(graph.lbm.density_numpy(), eager.lbm.density_numpy()) < 1e-5
    assert rel_l2(graph.lbm.velocity_numpy(), eager.lbm.velocity_numpy()) < 2.5e-4
    assert rel_l2(graph.mpm.positions_numpy(), eager.mpm.positions_numpy()) < 1e-5
    d_e, d_g = eager.diagnostics(), graph.diagnostics()
    for key in ("coupling_unsupported_particle_count", "coupling_partial_support_particle_count",
                "mpm_particle_count"):
        assert d_e[key] == d_g[key], key
    # The graph path leaves the solvers usable by the eager API.
    graph.step()
    eager.step()
    assert rel_l2(graph.lbm.velocity_numpy(), eager.lbm.velocity_numpy()) < 2.5e-4


def test_lattice_alone_graph_is_bit_exact():
    """Without particles in the fluid the coupled step has no atomics that matter: the
    lattice of the graph run is bit-identical to the eager run."""
    cfg, solid, pos = coupled_smoke_config(steps=8)
    import dataclasses
    cfg = dataclasses.replace(cfg, coupling=CouplingConfig(enabled=False,
                                                           mpm_substeps_per_lbm_step=2))
    eager, graph = make(cfg, solid, pos), make(cfg, solid, pos)
    for _ in range(8):
        eager.step()
    graph.advance(8)
    np.testing.assert_array_equal(graph.lbm.distribution_numpy(), eager.lbm.distribution_numpy())


def test_runner_graph_steps_are_the_eager_steps():
    """FSISimulation.step with graph_steps (the coupled step and its diagnostics replayed from
    two captured CUDA graphs, the driving force read from a device buffer) against eager
    steps, on the sorted (deterministic) scatter and a driving force that changes every step:
    every diagnostics value and the final state are bit-identical."""
    import dataclasses
    cfg, solid, pos = coupled_smoke_config(steps=8)
    cfg = dataclasses.replace(cfg, mpm=dataclasses.replace(cfg.mpm, p2g_mode="sorted"))
    eager, graph = make(cfg, solid, pos), make(cfg, solid, pos, graph_steps=True)
    for k in range(8):
        g = (1e-5 * (1 + 0.1 * k), 2e-7 * k, 0.0)
        de, dg = eager.step(body_force=g), graph.step(body_force=g)
        assert de.keys() == dg.keys()
        for key in de:
            np.testing.assert_array_equal(np.asarray(dg[key]), np.asarray(de[key]), err_msg=key)
    assert len(graph._graphs) == 2  # one graph per lattice parity, replayed from step 2 on
    np.testing.assert_array_equal(graph.lbm.distribution_numpy(), eager.lbm.distribution_numpy())
    np.testing.assert_array_equal(graph.mpm.positions_numpy(), eager.mpm.positions_numpy())
    assert (graph.lbm.steps_done, graph.coupler.coupled_step, graph.step_index) == \
        (eager.lbm.steps_done, eager.coupler.coupled_step, eager.step_index)
    # eager and graph steps interleave
    graph.graph_steps = False
    graph.step()
    graph.graph_steps = True
    eager.step(), eager.step()
    graph.step()
    np.testing.assert_array_equal(graph.mpm.positions_numpy(), eager.mpm.positions_numpy())


def test_runner_graph_steps_with_immersed_boundary_and_contact():
    """The captured runner step with the immersed-boundary drag (assembly in IB mode) and the
    contact kernel (after every substep): the same diagnostics and state as eager steps; the
    IB force total adds with float atomics, so its norm is held to float32 rounding."""
    import dataclasses
    cfg, solid, pos = coupled_smoke_config(steps=6)
    coupling = dataclasses.replace(cfg.coupling, immersed_boundary_enabled=True,
                                   immersed_boundary_drag=0.05, contact_enabled=True,
                                   contact_velocity_damping=0.2)
    cfg = dataclasses.replace(cfg, coupling=coupling,
                              mpm=dataclasses.replace(cfg.mpm, p2g_mode="sorted"))
    eager, graph = make(cfg, solid, pos), make(cfg, solid, pos, graph_steps=True)
    for _ in range(6):
        de, dg = eager.step(), graph.step()
        for key in de:
            if key == "coupling_ib_total_force_norm":
                assert dg[key] == pytest.approx(de[key], rel=1e-5, abs=1e-12)
            else:
                np.testing.assert_array_equal(np.asarray(dg[key]), np.asarray(de[key]),
                                              err_msg=key)
    assert len(graph._graphs) == 2
    assert rel_l2(graph.mpm.positions_numpy(), eager.mpm.positions_numpy()) < 1e-6
