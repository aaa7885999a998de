"""The oracle's coupling kernels against independent float64 numpy restatements of the
reference's loops: the penalty coupling (fsi/coupling.py:314-406: fluid-node interpolation of
the lattice velocity, support tests, relative-velocity and force clipping, the gamma ramp, the
reaction spread and the solid-fraction build), the immersed-boundary drag (coupling.py:421-450)
and the contact detection and damping (coupling.py:463-496), on random lattice states, random
solid masks and fractions, and particles with full, partial and no fluid support. CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from fsi.config import CouplingConfig, LBMConfig, MPMConfig
from oracle import oracle as O


def reference_coupling(co, dt_ratio, build):
    """_compute_coupling_forces_kernel of the coupler ``co``'s state, loop for loop."""
    c, lbm, mpm = co.config, co.lbm, co.mpm
    n, inv_dx, vol_cell = mpm.num_particles, co.inv_dx, co.cell_volume
    shape = (co.nx, co.ny, co.nz)
    force = co.coupling_force.copy()
    phi = co.solid_volume_fraction.copy()
    fp = np.zeros((n, 3))
    valid = np.zeros(n)
    mask = np.zeros(n, np.int32)
    unsupported = partial = clipped_count = 0
    gamma = float(co._gamma_device())
    for p in range(n):
        gp = mpm.x[p] * inv_dx
        base = np.trunc(gp - 0.5).astype(np.int64)
        fx = gp - base
        w = np.array([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1.0) ** 2, 0.5 * (fx - 0.5) ** 2])
        nodes = []
        for off in np.ndindex(3, 3, 3):
            node = base + off
            if (node >= 0).all() and (node < shape).all() and lbm.solid[tuple(node)] == 0:
                nodes.append((tuple(node), w[off[0], 0] * w[off[1], 1] * w[off[2], 2]))
        total = sum(wt for _, wt in nodes)
        u = sum((wt * lbm.v[node] for node, wt in nodes), np.zeros(3))
        valid[p] = total
        if total <= c.min_valid_weight:
            unsupported += 1
            continue
        if total < 1.0 - 1.0e-5:
            partial += 1
        dv = u / total - mpm.v[p]
        clipped = False
        if c.relative_velocity_limit is not None:
            norm = np.linalg.norm(dv)
            if norm > c.relative_velocity_limit and norm > 0.0:
                dv = dv / norm * c.relative_velocity_limit
                clipped = True
        f = gamma * mpm.mass[p] * dv
        if c.force_limit is not None:
            norm = np.linalg.norm(f)
            if norm > c.force_limit and norm > 0.0:
                f = f / norm * c.force_limit
                clipped = True
        fp[p], mask[p] = f, 1
        clipped_count += clipped
        for node, wt in nodes:
            force[node] += -(wt / total) * f * dt_ratio / vol_cell
            if build:
                phi[node] += (wt / total) * mpm.volume[p] / vol_cell
    return force, phi, fp, valid, mask, (unsupported, partial, clipped_count)


@pytest.mark.parametrize("limits,ramp,build", [
    ((None, None), 0, True),
    ((0.05, 0.002), 4, False),
])
def test_coupling_matches_a_second_restatement(limits, ramp, build):
    n = 8
    lbm = O.LBMSolver3D(LBMConfig(nx=n, ny=n, nz=n, viscosity=1.0 / 30.0), dtype=np.float64)
    rng = np.random.default_rng(3)
    solid = (rng.random((n, n, n)) < 0.3).astype(np.int32)
    solid[5:, 5:, 5:] = 1  # a solid block: particles inside it have no fluid support
    lbm.initialize(solid)
    lbm.v[...] = 0.05 * rng.standard_normal((n, n, n, 3))
    mpm = O.MPMSolver3D(MPMConfig(nx=n, ny=n, nz=n, max_particles=80, dx=0.5),
                        dtype=np.float64)
    pos = rng.uniform(0.1, (n - 1.5) * 0.5, (80, 3))
    pos[:8] = rng.uniform(2.8, 3.2, (8, 3))  # inside the solid block
    mpm.initialize_particles_from_numpy(pos.astype(np.float32),
                                        velocities=rng.normal(0.0, 0.05, (80, 3)).astype(np.float32))
    mpm.x[:80] = pos
    cfg = CouplingConfig(gamma=0.3, relative_velocity_limit=limits[0], force_limit=limits[1],
                         gamma_ramp_steps=ramp, min_valid_weight=0.05)
    co = O.LBMMpmCoupler(cfg, lbm, mpm)
    co.coupled_step = 1
    co.clear_coupling_fields()
    co.coupling_force[...] = 1e-3 * rng.standard_normal(co.coupling_force.shape)  # accumulates
    want = reference_coupling(co, 0.1, build)
    co._coupling_kernel(0.1, build)
    got = (co.coupling_force, co.solid_volume_fraction, mpm.particle_force[:80],
           co.particle_valid_weight[:80], co.particle_coupling_mask[:80])
    for name, g, w in zip(("coupling_force", "phi", "f_p", "valid", "mask"), got, want):
        np.testing.assert_allclose(g, w, rtol=1e-12, atol=1e-15, err_msg=name)
    assert tuple(int(v) for v in co.counters) == want[5]
    unsupported, partial, clipped = want[5]
    assert unsupported > 0 and partial > 0
    assert (clipped > 0) == (limits != (None, None))


def reference_ib(co):
    """_compute_immersed_boundary_force_kernel (coupling.py:421-450), cell by cell."""
    c, lbm = co.config, co.lbm
    out = np.zeros_like(co.immersed_boundary_force)
    active = clipped = 0
    total = np.zeros(3)
    for cell in np.ndindex(co.nx, co.ny, co.nz):
        if lbm.solid[cell] != 0 or not c.immersed_boundary_drag > 0.0:
            continue
        phi = co.solid_volume_fraction[cell]
        if not (phi > 0.0 and phi >= c.immersed_boundary_fraction_threshold):
            continue
        f = -c.immersed_boundary_drag * phi * lbm.rho[cell] * lbm.v[cell]
        norm = np.linalg.norm(f)
        limit = c.immersed_boundary_max_force
        if limit is not None and norm > limit and norm > 0.0:
            f = f / norm * limit
            clipped += 1
        out[cell] = f
        active += 1
        total += f
    return out, (active, clipped), total


def reference_contact(co):
    """_compute_contact_diagnostics_kernel (coupling.py:463-496), particle by particle."""
    c, lbm, mpm = co.config, co.lbm, co.mpm
    v = mpm.v[:mpm.num_particles].copy()
    mask = np.zeros(mpm.num_particles, np.int32)
    cand = damped = 0
    for p in range(mpm.num_particles):
        gp = mpm.x[p] * co.inv_dx
        base = np.trunc(gp - 0.5).astype(np.int64)
        fx = gp - base
        w = np.array([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1.0) ** 2, 0.5 * (fx - 0.5) ** 2])
        dyn = stat = 0.0
        for off in np.ndindex(3, 3, 3):
            node = base + off
            if (node >= 0).all() and (node < (co.nx, co.ny, co.nz)).all():
                wt = w[off[0], 0] * w[off[1], 1] * w[off[2], 2]
                dyn += wt * co.solid_volume_fraction[tuple(node)]
                if lbm.solid[tuple(node)] != 0:
                    stat += wt
        thr = c.contact_fraction_threshold
        if dyn >= thr or stat >= thr:
            mask[p] = 1
            cand += 1
            if c.contact_velocity_damping > 0.0:
                v[p] *= 1.0 - c.contact_velocity_damping
                damped += 1
    return v, mask, (cand, damped)


@pytest.mark.parametrize("max_force", [None, 2e-4])
def test_ib_and_contact_match_a_second_restatement(max_force):
    n = 8
    rng = np.random.default_rng(7)
    lbm = O.LBMSolver3D(LBMConfig(nx=n, ny=n, nz=n, viscosity=1.0 / 30.0), dtype=np.float64)
    solid = (rng.random((n, n, n)) < 0.15).astype(np.int32)
    lbm.initialize(solid)
    lbm.rho[...] = 1.0 + 0.01 * rng.standard_normal((n, n, n))
    lbm.v[...] = 0.05 * rng.standard_normal((n, n, n, 3))
    mpm = O.MPMSolver3D(MPMConfig(nx=n, ny=n, nz=n, max_particles=60), dtype=np.float64)
    pos = rng.uniform(0.3, n - 1.5, (60, 3))
    mpm.initialize_particles_from_numpy(pos.astype(np.float32),
                                        velocities=rng.normal(0.0, 0.05, (60, 3)).astype(np.float32))
    mpm.x[:60] = pos
    cfg = CouplingConfig(immersed_boundary_enabled=True, immersed_boundary_drag=0.05,
                         immersed_boundary_fraction_threshold=0.2,
                         immersed_boundary_max_force=max_force, contact_enabled=True,
                         contact_fraction_threshold=0.4, contact_velocity_damping=0.25)
    co = O.LBMMpmCoupler(cfg, lbm, mpm)
    co.clear_coupling_fields()
    co.solid_volume_fraction[...] = np.clip(rng.uniform(-0.3, 1.0, (n, n, n)), 0.0, None)
    ib, counts, total = reference_ib(co)
    v, mask, contact = reference_contact(co)
    co._ib_kernel()
    co._contact_kernel()
    np.testing.assert_allclose(co.immersed_boundary_force, ib, rtol=1e-12, atol=1e-16)
    assert tuple(int(x) for x in co.ib_counters) == counts
    np.testing.assert_allclose(co.ib_total, total, rtol=1e-10, atol=1e-16)
    np.testing.assert_allclose(mpm.v[:60], v, rtol=1e-15, atol=0.0)
    np.testing.assert_array_equal(co.particle_contact_mask[:60], mask)
    assert tuple(int(x) for x in co.contact_counters) == contact
    assert counts[0] > 0 and (counts[1] > 0) == (max_force is not None)
    assert 0 < contact[0] < 60 and contact[1] == contact[0]
