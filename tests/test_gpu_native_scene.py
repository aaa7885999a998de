"""The one-call coupled step (fsi_ctx_create / fsi_coupled_step through fsi.scene.NativeScene)
against the Python coupler (LBMMpmCoupler.step, fsi/coupling.py:135-173) and the oracle.

With the sorted scatter both paths are deterministic, so every field must match bit for bit;
with the atomic scatter the grid sums arrive in scheduling order and the comparison holds to
that order's float32 noise."""
from __future__ import annotations

import dataclasses

import numpy as np
import pytest
import torch

from fsi.scene import NativeScene
from fsi.simulation import FSISimulation
from helpers import coupled_smoke_config, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _sim(steps=10, p2g_mode="sorted", **coupling):
    cfg, solid, pos = coupled_smoke_config(steps=steps)
    cfg = dataclasses.replace(cfg, mpm=dataclasses.replace(cfg.mpm, p2g_mode=p2g_mode),
                              coupling=dataclasses.replace(cfg.coupling, **coupling))
    sim = FSISimulation(cfg)
    sim.initialize_lbm(solid)
    sim.initialize_mpm_from_numpy(pos)
    return cfg, sim


def _fields(sim) -> dict:
    c = sim.coupler
    return {
        "pops": sim.lbm.distribution_numpy(), "rho": sim.lbm.density_numpy(),
        "u": sim.lbm.velocity_numpy(), "x": sim.mpm.positions_numpy(),
        "v": sim.mpm.velocities_numpy(), "F": sim.mpm.deformation_gradients_numpy(),
        "fp": sim.mpm.particle_forces_numpy(), "accum": c.coupling_force_numpy(),
        "phi": c.solid_volume_fraction_numpy(), "valid": c.particle_valid_weights_numpy(),
        "mask": c.particle_coupling_mask_numpy(), "counters": c._counters.cpu().numpy(),
        "ib": c.immersed_boundary_force_numpy(), "contact": c.particle_contact_mask_numpy(),
    }


def _assert_same(a: dict, b: dict) -> None:
    for k in a:
        if k == "counters":
            # the eight integer counters exactly; the IB force totals (float atomics summed in
            # arrival order) to float32 rounding
            np.testing.assert_array_equal(a[k][:8], b[k][:8], err_msg=k)
            np.testing.assert_allclose(a[k][8:11].view(np.float32), b[k][8:11].view(np.float32),
                                       rtol=1e-5, atol=0, err_msg=k)
        else:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_native_step_bit_identical_to_python_coupler():
    cfg, py = _sim()
    _, nat = _sim()
    scene = NativeScene(nat.coupler)
    for _ in range(6):
        py.coupler.step(cfg.lbm_dt)
    scene.step(cfg.lbm_dt, steps=6)
    _assert_same(_fields(py), _fields(nat))
    assert nat.lbm.steps_done == py.lbm.steps_done == 6
    assert nat.coupler.coupled_step == py.coupler.coupled_step == 6
    scene.close()


def test_native_step_matches_oracle_bit_for_bit():
    """Ten native steps of the 48x32x32 smoke workload against the oracle in the cell order."""
    cfg, solid, pos = coupled_smoke_config(steps=10)
    cfg = dataclasses.replace(cfg, mpm=dataclasses.replace(cfg.mpm, p2g_mode="sorted"))
    sim = FSISimulation(cfg)
    sim.initialize_lbm(solid)
    sim.initialize_mpm_from_numpy(pos)
    ref = O.FSISimulation(cfg, nthreads=4, polar="device", cell_order=True)
    ref.initialize_lbm(solid)
    ref.initialize_mpm_from_numpy(pos)
    scene = NativeScene(sim.coupler)
    scene.step(cfg.lbm_dt, steps=10)
    for _ in range(10):
        ref.coupler.step(cfg.lbm_dt)
    np.testing.assert_array_equal(sim.lbm.distribution_numpy(), ref.lbm.distribution_numpy())
    np.testing.assert_array_equal(sim.lbm.velocity_numpy(), ref.lbm.v)
    np.testing.assert_array_equal(sim.mpm.positions_numpy(), ref.mpm.positions_numpy())
    np.testing.assert_array_equal(sim.mpm.velocities_numpy(), ref.mpm.velocities_numpy())
    np.testing.assert_array_equal(sim.coupler.coupling_force_numpy(),
                                  ref.coupler.coupling_force_numpy())


def test_native_and_python_steps_mix():
    """3 Python + 3 native + 2 Python steps equal 8 Python steps (the host bookkeeping moves
    between the two paths)."""
    cfg, a = _sim()
    _, b = _sim()
    for _ in range(8):
        a.coupler.step(cfg.lbm_dt)
    scene = NativeScene(b.coupler)
    for _ in range(3):
        b.coupler.step(cfg.lbm_dt)
    b.lbm.velocity_numpy()  # a Python accessor between the paths (macro made current)
    scene.step(cfg.lbm_dt, steps=3)
    for _ in range(2):
        b.coupler.step(cfg.lbm_dt)
    _assert_same(_fields(a), _fields(b))


def test_native_step_ib_contact_ramp_and_body_force():
    """Immersed boundary, contact damping, the gamma ramp and a per-step body force."""
    kw = dict(immersed_boundary_enabled=True, immersed_boundary_drag=0.05,
              immersed_boundary_max_force=1e-4, contact_enabled=True,
              contact_velocity_damping=0.25, gamma_ramp_steps=4)
    cfg, py = _sim(**kw)
    _, nat = _sim(**kw)
    scene = NativeScene(nat.coupler)
    g = np.array([2e-5, 0.0, 1e-6], np.float32)
    for _ in range(5):
        py.coupler.step(cfg.lbm_dt, body_force=g)
    scene.step(cfg.lbm_dt, steps=5, body_force=g)
    _assert_same(_fields(py), _fields(nat))
    assert nat.coupler.effective_gamma() == py.coupler.effective_gamma()
    assert np.abs(_fields(nat)["ib"]).max() > 0.0


def test_native_step_uncoupled():
    cfg, py = _sim(enabled=False)
    _, nat = _sim(enabled=False)
    scene = NativeScene(nat.coupler)
    for _ in range(4):
        py.coupler.step(cfg.lbm_dt)
    scene.step(cfg.lbm_dt, steps=4)
    _assert_same(_fields(py), _fields(nat))


def test_native_step_atomic_scatter_close_to_python():
    cfg, py = _sim(p2g_mode="atomic")
    _, nat = _sim(p2g_mode="atomic")
    scene = NativeScene(nat.coupler)
    for _ in range(6):
        py.coupler.step(cfg.lbm_dt)
    scene.step(cfg.lbm_dt, steps=6)
    a, b = _fields(py), _fields(nat)
    for k in ("rho", "x", "F"):
        assert rel_l2(b[k], a[k]) <= 1e-6, k
    assert rel_l2(b["u"], a["u"]) <= 1e-4
    np.testing.assert_array_equal(a["mask"], b["mask"])


def test_native_step_in_a_cuda_graph():
    """Two native steps captured in a graph and replayed equal the eager native steps."""
    cfg, eager = _sim()
    _, graphed = _sim()
    se, sg = NativeScene(eager.coupler), NativeScene(graphed.coupler)
    se.step(cfg.lbm_dt, steps=2)  # settle the buffer choice and parity before capture
    sg.step(cfg.lbm_dt, steps=2)
    before = (graphed.lbm.steps_done, graphed.lbm._fcur, graphed.lbm._fprev)
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        with torch.cuda.graph(graph, stream=stream):
            sg.step(cfg.lbm_dt, steps=2)  # recorded, not run; the host state advances by 2
    torch.cuda.current_stream().wait_stream(stream)
    assert graphed.lbm.steps_done == before[0] + 2
    for _ in range(3):
        graph.replay()
    torch.cuda.synchronize()
    graphed.lbm._steps_done = before[0] + 6
    graphed.coupler._coupled_step = before[0] + 6
    se.step(cfg.lbm_dt, steps=6)
    _assert_same(_fields(eager), _fields(graphed))


def test_native_scene_errors():
    cfg, sim = _sim()
    scene = NativeScene(sim.coupler)
    with pytest.raises(ValueError):
        scene.step(0.0)
    with pytest.raises(ValueError):
        scene.step(cfg.lbm_dt, body_force=[1.0, 2.0])
    with pytest.raises(ValueError):
        sim.lbm._fprev = -1
        sim.lbm._macro_fresh = False  # stale rho/u without the last step's force
        scene.step(cfg.lbm_dt)
