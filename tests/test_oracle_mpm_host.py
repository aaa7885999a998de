"""The oracle's MLS-MPM substep against an independent float64 numpy restatement of the
reference's loops (fsi/mpm3d.py:189-328: clear_grid, p2g with the fixed-corotated stress and
the polar rotation from the SVD, grid_op with gravity and damped walls, g2p with APIC and the
position clamp), on random particle states: positions next to every wall and below 0.5 cells
(the truncating base-cell cast), a grid spacing other than 1 (the reference's unscaled
offset in the APIC term), sheared deformation gradients and particle forces. CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from fsi.config import MPMConfig
from oracle import oracle as O


def reference_substep(s, dt):
    """One substep of solver ``s``'s state in float64, loop for loop as mpm3d.py:189-328."""
    n, dx = s.num_particles, s.dx
    inv_dx = 1.0 / dx
    nx, ny, nz = s.nx, s.ny, s.nz
    x, v, C, F = s.x[:n].copy(), s.v[:n].copy(), s.C[:n].copy(), s.F[:n].copy()
    m, vol, fp = s.mass[:n], s.volume[:n], s.particle_force[:n]
    gv = np.zeros((nx, ny, nz, 3))
    gm = np.zeros((nx, ny, nz))
    eye = np.eye(3)

    def stencil(p):
        base = np.trunc(x[p] * inv_dx - 0.5).astype(np.int64)
        fx = x[p] * inv_dx - base
        w = np.array([0.5 * (1.5 - fx) ** 2, 0.75 - (fx - 1.0) ** 2, 0.5 * (fx - 0.5) ** 2])
        for off in np.ndindex(3, 3, 3):
            node = base + off
            if (node >= 0).all() and (node < (nx, ny, nz)).all():
                yield tuple(node), np.array(off, np.float64), fx, w[off[0], 0] * w[off[1], 1] * w[off[2], 2]

    for p in range(n):
        F[p] = (eye + dt * C[p]) @ F[p]
        J = np.linalg.det(F[p])
        U, _, Vt = np.linalg.svd(F[p])
        R = U @ Vt
        stress = 2.0 * s.mu * (F[p] - R) @ F[p].T + s.lam * J * (J - 1.0) * eye
        stress = -dt * vol[p] * 4.0 * inv_dx * inv_dx * stress
        affine = stress + m[p] * C[p]
        for node, off, fx, wt in stencil(p):
            dpos = (off - fx) * dx
            gv[node] += wt * (m[p] * v[p] + affine @ dpos + dt * fp[p])
            gm[node] += wt * m[p]
    g = np.asarray(s.config.gravity, np.float32).astype(np.float64)
    bw, damp = s.boundary_width, s.boundary_damping
    for node in zip(*np.nonzero(gm > 0.0)):
        gv[node] = gv[node] / gm[node] + dt * g
        for a, size in enumerate((nx, ny, nz)):
            if node[a] < bw and gv[node][a] < 0.0:
                gv[node][a] = -damp * gv[node][a]
            if node[a] >= size - bw and gv[node][a] > 0.0:
                gv[node][a] = -damp * gv[node][a]
    upper = np.array([(nx - 1.5) * dx, (ny - 1.5) * dx, (nz - 1.5) * dx])
    for p in range(n):
        new_v, new_c = np.zeros(3), np.zeros((3, 3))
        for node, off, fx, wt in stencil(p):
            new_v += wt * gv[node]
            new_c += 4.0 * inv_dx * wt * np.outer(gv[node], off - fx)
        v[p] = new_v
        C[p] = new_c if s.apic else 0.0
        x[p] = np.minimum(np.maximum(x[p] + dt * v[p], 0.5 * dx), upper)
    return x, v, C, F, gv, gm


@pytest.mark.parametrize("dx,damping", [(1.0, 0.0), (0.5, 0.3)])
def test_substep_matches_a_second_restatement(dx, damping):
    n_cells = 8
    cfg = MPMConfig(nx=n_cells, ny=n_cells, nz=n_cells, max_particles=64, particles_per_cell=2,
                    dx=dx, dt=0.05, density=1.5, youngs_modulus=2.0, poisson_ratio=0.3,
                    gravity=(0.0, -0.5, 0.1), boundary_width=2, boundary_damping=damping)
    s = O.MPMSolver3D(cfg, dtype=np.float64, polar="exact")
    rng = np.random.default_rng(11)
    lo, hi = 0.2 * dx, (n_cells - 1.5) * dx
    pos = rng.uniform(lo, hi, (48, 3))
    pos[:6, 0] = rng.uniform(0.0, 0.45 * dx, 6)       # base cell from a negative argument
    pos[6:12, 1] = hi - rng.uniform(0.0, 0.2 * dx, 6)  # against the upper walls
    s.initialize_particles_from_numpy(pos.astype(np.float32),
                                      velocities=rng.normal(0.0, 0.3, (48, 3)).astype(np.float32))
    n = s.num_particles
    s.x[:n] = pos  # float64 positions, as the float64 oracle carries them
    s.C[:n] = 0.2 * rng.standard_normal((n, 3, 3))
    s.F[:n] = np.eye(3) + 0.05 * rng.standard_normal((n, 3, 3))
    s.particle_force[:n] = 0.1 * rng.standard_normal((n, 3))
    want = reference_substep(s, 0.05)
    s.substep()
    got = (s.x[:n], s.v[:n], s.C[:n], s.F[:n], s.grid_v, s.grid_m)
    for name, g, w in zip(("x", "v", "C", "F", "grid_v", "grid_m"), got, want):
        np.testing.assert_allclose(g, w, rtol=1e-11, atol=1e-13, err_msg=name)
    gm = want[5]
    assert gm[:2].sum() > 0 and gm[:, -2:].sum() > 0  # the wall branches of grid_op ran
