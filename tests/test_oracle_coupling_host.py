"""The oracle's penalty-coupling kernel against an independent float64 numpy restatement of
the reference's loop (fsi/coupling.py:314-406: fluid-node interpolation of the lattice
velocity, support tests, relative-velocity and force clipping, the gamma ramp, the reaction
spread and the solid-fraction build), on random lattice velocities, a random solid mask and
particles with full, partial and no fluid support. CPU only."""
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
