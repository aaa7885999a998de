"""GPU MLS-MPM vs the CPU oracle and analytic checks.

Bit-exact: particle-to-cell indices (trunc(x/dx - 0.5), negative positions
included), a full substep while no rotation is involved, and every substep of the
sorted scatter (p2g_mode="sorted") against the oracle summing in the same cell order with the
device's float32 polar rotation. Tolerance: the polar rotation (float32 Newton
iteration vs a float64 SVD) and the atomic scatter, whose grid sums arrive in a
different order on the GPU.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from fsi import _native as nat
from fsi.config import MPMConfig
from fsi.mpm3d import MPMSolver3D
from helpers import rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def mpm_cfg(**kw) -> MPMConfig:
    p = dict(nx=16, ny=16, nz=16, max_particles=10_000, dt=1.0e-3, gravity=(0.0, 0.0, 0.0),
             boundary_width=2)
    p.update(kw)
    return MPMConfig(**p)


def svd_rotation(f: np.ndarray) -> np.ndarray:
    u, _, vt = np.linalg.svd(f)
    if np.linalg.det(u @ vt) < 0:
        u[:, -1] = -u[:, -1]
    return u @ vt


def test_polar_rotation_against_svd():
    rng = np.random.default_rng(11)
    F = np.eye(3)[None] + rng.normal(0, 0.25, (4000, 3, 3))
    F[:200] = np.eye(3) + rng.normal(0, 1e-4, (200, 3, 3))       # near identity
    F[200:300] = F[200:300] * np.array([1.0, -1.0, 1.0])          # inverted
    F = F.astype(np.float32)
    Fd = torch.from_numpy(F.reshape(-1, 9)).cuda()
    Rd = torch.empty_like(Fd)
    nat.call("fsi_mpm_polar", nat.ptr(Fd), nat.ptr(Rd), F.shape[0], nat.stream_ptr())
    R = Rd.cpu().numpy().reshape(-1, 3, 3).astype(np.float64)
    ref = O.polar_rotation(F.astype(np.float64))
    err = np.abs(R - ref).max(axis=(1, 2))
    assert err.max() < 2e-5, err.max()
    for f, r in zip(F[:50].astype(np.float64), R[:50]):
        np.testing.assert_allclose(r, svd_rotation(f), atol=2e-5)
    dets = np.linalg.det(R)
    np.testing.assert_allclose(dets, 1.0, atol=1e-5)


def test_particle_cell_indices_bit_exact():
    rng = np.random.default_rng(2)
    pos = rng.uniform(-2.0, 18.0, (5000, 3)).astype(np.float32)
    pos[:10] = [[-0.75, 4, 4], [0.4999, 0.5, 0.5001], [-0.5, -0.49, 0], [15.5, 15.49, 0.0],
                [3.0, 3.5, 4.5], [1e-8, -1e-8, 7.25], [2.5, 2.4999998, 2.5000002],
                [-1.5, -1.0, -0.25], [8.0, 8.0, 8.0], [0.0, 0.0, 0.0]]
    for dx in (1.0, 0.5, 0.3):
        s = MPMSolver3D(mpm_cfg(dx=dx))
        s.initialize_particles_from_numpy(pos)
        inv = np.float32(1.0 / dx)
        expect = ((pos * inv) - np.float32(0.5)).astype(np.int32)  # C cast truncates toward 0
        np.testing.assert_array_equal(s.base_cells_numpy(), expect)


def test_first_substep_bit_exact_single_particle():
    """With F = I and C = 0 the first substep needs no rotation: results are bit-exact."""
    cfg = mpm_cfg(gravity=(0.0, -1.0e-3, 0.0), dt=1e-2)
    for pos, vel in (((4.3, 5.7, 6.1), (0.1, -0.2, 0.05)), ((0.7, 8.0, 14.9), (0.0, 0.0, -1.0))):
        g, o = MPMSolver3D(cfg), O.MPMSolver3D(cfg)
        for s in (g, o):
            s.initialize_particles_from_numpy(np.array([pos], np.float32),
                                              np.array([vel], np.float32), 1.3, 0.7)
            s.substep()
        np.testing.assert_array_equal(g.positions_numpy(), o.positions_numpy())
        np.testing.assert_array_equal(g.velocities_numpy(), o.velocities_numpy())
        np.testing.assert_array_equal(g.deformation_gradients_numpy(), o.deformation_gradients_numpy())
        np.testing.assert_array_equal(g.affine_velocities_numpy(), o.C[:1])


@pytest.mark.parametrize("gravity,dt,steps", [((0.0, -1.0e-3, 0.0), 1.0e-2, 10),
                                               ((0.0, 0.0, 0.0), 1.0e-3, 10),
                                               ((1e-3, -2e-3, 5e-4), 1.0e-2, 40)])
def test_box_against_oracle(gravity, dt, steps):
    """The default (atomic) scatter against the oracle with the device's float32 polar
    rotation (so only the order of the grid sums differs) and against the float64 rotation.
    The stiff box (E = 1000, CFL ~0.3 per substep) amplifies float32 order differences:
    velocities agree to 1e-3 relative, positions and F far closer."""
    cfg = mpm_cfg(gravity=gravity, dt=dt, youngs_modulus=1000.0)
    g = MPMSolver3D(cfg)
    refs = [O.MPMSolver3D(cfg, polar="device"), O.MPMSolver3D(cfg)]
    rng = np.random.default_rng(4)
    for s in (g, *refs):
        s.initialize_particles_box((6.0, 8.0, 6.0), (10.0, 12.0, 10.0), spacing=0.5)
    vel = rng.normal(0, 1e-2, (g.particle_count(), 3)).astype(np.float32)
    pos = g.positions_numpy()
    for s in (g, *refs):
        s.initialize_particles_from_numpy(pos, vel, particle_volume=0.125)
    for _ in range(steps):
        for s in (g, *refs):
            s.substep()
    for o in refs:
        assert rel_l2(g.positions_numpy(), o.positions_numpy()) < 1e-6
        assert rel_l2(g.velocities_numpy(), o.velocities_numpy()) < 1e-3
        assert rel_l2(g.deformation_gradients_numpy(), o.deformation_gradients_numpy()) < 1e-5
        np.testing.assert_allclose(g.center_of_mass(), o.center_of_mass(), rtol=0, atol=2e-5)
    assert np.isfinite(g.velocities_numpy()).all()


def test_reference_mpm_behaviour():
    """The reference's tests/test_mpm3d.py assertions on the GPU solver."""
    s = MPMSolver3D(mpm_cfg())
    with pytest.raises(RuntimeError):
        s.substep()
    n = s.initialize_particles_box((6.0, 6.0, 6.0), (10.0, 10.0, 10.0), spacing=1.0)
    assert n == 64 and s.particle_count() == n and np.all(s.active_numpy() == 1)
    p = s.positions_numpy()
    assert p.shape == (n, 3) and p.min() >= 6.0 and p.max() < 10.0
    with pytest.raises(ValueError):
        s.substep(0.0)
    with pytest.raises(ValueError):
        MPMSolver3D(mpm_cfg(max_particles=10)).initialize_particles_box((2.0,) * 3, (10.0,) * 3, 0.5)
    com0 = s.center_of_mass()
    for _ in range(5):
        s.substep()
    assert np.linalg.norm(s.center_of_mass() - com0) < 1e-3
    gcfg = mpm_cfg(gravity=(0.0, -1.0e-3, 0.0), dt=1.0e-2)
    g = MPMSolver3D(gcfg)
    g.initialize_particles_box((6.0, 8.0, 6.0), (10.0, 12.0, 10.0), spacing=1.0)
    c0 = g.center_of_mass()
    for _ in range(10):
        g.substep()
    assert g.center_of_mass()[1] < c0[1]
    d = MPMSolver3D(mpm_cfg(gravity=(0.0, -1.0e-3, 0.0)))
    d.initialize_particles_box((2.0, 2.0, 2.0), (5.0, 5.0, 5.0), spacing=1.0)
    for _ in range(20):
        d.substep()
    pos = d.positions_numpy()
    assert np.isfinite(pos).all() and np.isfinite(d.deformation_gradients_numpy()).all()
    assert (pos >= 0.0).all() and (pos <= 16 - 1e-4).all()


def test_grid_is_left_clean_between_substeps():
    """The atomic scatter's invariant: the grid is all zero between substeps."""
    cfg = mpm_cfg(gravity=(0.0, -1e-3, 0.0), dt=1e-2, p2g_mode="atomic")
    s = MPMSolver3D(cfg)
    s.initialize_particles_box((3.0, 3.0, 3.0), (12.0, 6.0, 5.0), spacing=0.5)
    for _ in range(3):
        s.substep()
        assert float(s._grid.abs().max()) == 0.0
        assert int(s._dirty.max()) == 0


@pytest.mark.parametrize("model", ["fixed_corotated", "neo_hookean"])
def test_material_models_and_per_particle_moduli(model):
    """Extensions with no reference counterpart, checked against the oracle restatement:
    the Neo-Hookean model and per-particle Young's moduli (two bodies of different stiffness)."""
    cfg = mpm_cfg(gravity=(0.0, -1.0e-3, 0.0), dt=1.0e-2, youngs_modulus=500.0,
                  constitutive_model=model)
    g, o = MPMSolver3D(cfg), O.MPMSolver3D(cfg)
    rng = np.random.default_rng(8)
    a = np.stack(np.meshgrid(*[np.arange(4.0, 6.0, 0.5)] * 3, indexing="ij"), -1).reshape(-1, 3)
    b = a + np.array([5.0, 1.0, 3.0])
    pos = np.concatenate([a, b]).astype(np.float32)
    vel = rng.normal(0, 1e-2, pos.shape).astype(np.float32)
    E = np.concatenate([np.full(len(a), 200.0), np.full(len(b), 800.0)])
    for s in (g, o):
        s.initialize_particles_from_numpy(pos, vel, particle_volume=0.125, youngs_modulus=E)
    for _ in range(20):
        g.substep()
        o.substep()
    assert rel_l2(g.positions_numpy(), o.positions_numpy()) < 1e-6
    assert rel_l2(g.velocities_numpy(), o.velocities_numpy()) < 1e-3
    assert rel_l2(g.deformation_gradients_numpy(), o.deformation_gradients_numpy()) < 1e-5
    # the stiffer body deforms less
    Fg = g.deformation_gradients_numpy()
    dev = np.linalg.norm(Fg - np.eye(3), axis=(1, 2))
    assert dev[len(a):].mean() < dev[: len(a)].mean()


def _assert_state_equal(g, o, what=""):
    np.testing.assert_array_equal(g.positions_numpy(), o.positions_numpy(), err_msg=what)
    np.testing.assert_array_equal(g.velocities_numpy(), o.velocities_numpy(), err_msg=what)
    np.testing.assert_array_equal(g.deformation_gradients_numpy(),
                                  o.deformation_gradients_numpy(), err_msg=what)
    np.testing.assert_array_equal(g.affine_velocities_numpy(), o.C[: o.num_particles],
                                  err_msg=what)


@pytest.mark.parametrize("case", ["box", "walls", "outside", "two_bodies", "neo_hookean"])
def test_sorted_scatter_bit_exact_against_cell_order(case):
    """The sorted scatter (p2g_mode="sorted") sums each node in the oracle's cell order
    (per-cell partials in ascending particle index, then ascending cell index), so with the
    device's float32 polar rotation every substep is bit-identical to the oracle."""
    kw = dict(gravity=(0.0, -1.0e-3, 0.0), dt=1.0e-2, youngs_modulus=1000.0, p2g_mode="sorted")
    rng = np.random.default_rng({"box": 4, "walls": 5, "outside": 6, "two_bodies": 7,
                                 "neo_hookean": 8}[case])
    if case == "walls":
        kw.update(nx=20, ny=13, nz=11, boundary_width=3, boundary_damping=0.5)
        pos = rng.uniform(0.6, 5.0, (3000, 3)).astype(np.float32)
    elif case == "outside":
        # Stencils that leave the grid: positions below 0.5 dx and beyond the last node.
        pos = rng.uniform(-3.0, 18.5, (2500, 3)).astype(np.float32)
    elif case == "two_bodies":
        kw.update(nx=24, ny=17, nz=18)
        a = rng.uniform(3.0, 7.0, (2000, 3))
        b = rng.uniform(12.0, 15.0, (1500, 3))
        pos = np.concatenate([a, b]).astype(np.float32)
    else:
        pos = np.stack(np.meshgrid(*[np.arange(6.0, 10.0, 0.5)] * 3, indexing="ij"),
                       -1).reshape(-1, 3).astype(np.float32)
        pos += rng.uniform(0, 0.25, pos.shape).astype(np.float32)
        if case == "neo_hookean":
            kw.update(constitutive_model="neo_hookean")
    cfg = mpm_cfg(**kw)
    vel = rng.normal(0, 2e-2, pos.shape).astype(np.float32)
    g = MPMSolver3D(cfg)
    o = O.MPMSolver3D(cfg, polar="device", cell_order=True)
    for s in (g, o):
        if case == "two_bodies":
            E = np.where(np.arange(len(pos)) < 2000, 800.0, 1500.0)
            s.initialize_particles_from_numpy(pos, vel, particle_volume=0.125, youngs_modulus=E)
        else:
            s.initialize_particles_from_numpy(pos, vel, particle_volume=0.125)
    assert g.sorted
    steps = 3 if case == "neo_hookean" else 12
    for k in range(steps):
        g.substep()
        o.substep()
        if case == "neo_hookean":
            # logf differs from the host's log in the last bit: hold the extension to float32 noise.
            assert rel_l2(g.positions_numpy(), o.positions_numpy()) < 1e-6
            continue
        _assert_state_equal(g, o, f"{case} substep {k}")


def test_sorted_scatter_repeats_bit_for_bit():
    """Two runs of the sorted scatter from the same state agree bit for bit, inactive
    particles included (the atomic scatter's sums depend on arrival order)."""
    cfg = mpm_cfg(gravity=(0.0, -1.0e-3, 0.0), dt=1.0e-2, youngs_modulus=1000.0,
                  p2g_mode="sorted")
    rng = np.random.default_rng(9)
    pos = rng.uniform(4.0, 12.0, (6000, 3)).astype(np.float32)
    vel = rng.normal(0, 1e-2, pos.shape).astype(np.float32)
    runs = []
    for _ in range(2):
        s = MPMSolver3D(cfg)
        s.initialize_particles_from_numpy(pos, vel, particle_volume=0.125)
        s._active[::7] = 0
        for _ in range(10):
            s.substep()
        runs.append((s.positions_numpy(), s.velocities_numpy(), s.deformation_gradients_numpy()))
    for a, b in zip(*runs):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(runs[0][0][::7], pos[::7])  # inactive particles stay put


def test_sorted_and_atomic_scatter_agree():
    cfg = dict(gravity=(0.0, -1.0e-3, 0.0), dt=1.0e-2, youngs_modulus=1000.0)
    rng = np.random.default_rng(10)
    pos = rng.uniform(3.0, 12.0, (5000, 3)).astype(np.float32)
    out = []
    for mode in ("sorted", "atomic"):
        s = MPMSolver3D(mpm_cfg(p2g_mode=mode, **cfg))
        s.initialize_particles_from_numpy(pos, particle_volume=0.125)
        for _ in range(10):
            s.substep()
        out.append(s)
    assert rel_l2(out[0].positions_numpy(), out[1].positions_numpy()) < 1e-6
    assert rel_l2(out[0].velocities_numpy(), out[1].velocities_numpy()) < 1e-3
