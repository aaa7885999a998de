"""The oracle's lattice step with x-face conditions against an independent float64 numpy
restatement of the reference's step (fsi/lbm3d.py:269-433: collide, stream with half-way
bounce-back and periodic wrap, apply_boundary, update_macro), on random states of a small
lattice with solid cells next to both faces. No golden covers the x faces, so this pins the
oracle's face code, including the velocity condition's in-place update in q order, to a
second restatement. CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from fsi.config import BoundaryConfig, LBMConfig
from oracle import oracle as O

# D3Q19 velocities in the reference's q order (lbm3d.py:219-238)
E = np.array([[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
              [1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0], [1, 0, 1], [-1, 0, -1],
              [1, 0, -1], [-1, 0, 1], [0, 1, 1], [0, -1, -1], [0, 1, -1], [0, -1, 1]])
LR = np.array([int(np.flatnonzero((E == -e).all(axis=1))[0]) for e in E])


def feq(w, q, rho, u):
    eu = E[q] @ u
    return w[q] * rho * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * (u @ u))


def reference_step(f, F, rho, v, force, solid, M, invM, S, w, left, right, rho0):
    """One step in float64, loop for loop as lbm3d.py:269-433 (no fused arithmetic)."""
    nx, ny, nz = solid.shape
    f, Fn, rho, v = f.copy(), F.copy(), rho.copy(), v.copy()
    for i, j, k in np.ndindex(nx, ny, nz):
        if solid[i, j, k]:
            continue
        u, g = v[i, j, k], force[i, j, k]
        mom = np.empty(19)
        for m in range(19):
            val = M[m] @ F[i, j, k]
            meq = {0: rho[i, j, k], 1: u @ u, 3: u[0], 5: u[1], 7: u[2],
                   9: 2 * u[0] ** 2 - u[1] ** 2 - u[2] ** 2, 11: u[1] ** 2 - u[2] ** 2,
                   13: u[0] * u[1], 14: u[1] * u[2], 15: u[0] * u[2]}.get(m, 0.0)
            val -= S[m] * (val - meq)
            guo = sum(w[q] * ((E[q] - u) @ g + (E[q] @ u) * (E[q] @ g)) * M[m, q]
                      for q in range(19))
            mom[m] = val + (1.0 - 0.5 * S[m]) * guo
        f[i, j, k] = invM @ mom
    for i, j, k in np.ndindex(nx, ny, nz):
        if solid[i, j, k]:
            continue
        for q in range(19):
            t = ((i + E[q][0]) % nx, (j + E[q][1]) % ny, (k + E[q][2]) % nz)
            if solid[t] == 0:
                Fn[t + (q,)] = f[i, j, k, q]
            else:
                Fn[i, j, k, LR[q]] = f[i, j, k, q]
    for x, xin, bc in ((0, 1, left), (nx - 1, nx - 2, right)):
        for j, k in np.ndindex(ny, nz):
            if solid[x, j, k]:
                continue
            # face values live in float32 fields in the reference
            if bc[0] == "pressure":
                u = v[xin, j, k] if solid[xin, j, k] > 0 else v[x, j, k]
                for q in range(19):
                    Fn[x, j, k, q] = feq(w, q, float(np.float32(bc[1])), u)
            elif bc[0] == "velocity":
                ub = np.asarray(bc[1], np.float32).astype(np.float64)
                for q in range(19):  # in place, in q order
                    o = LR[q]
                    Fn[x, j, k, q] = feq(w, o, rho0, ub) - Fn[x, j, k, o] + feq(w, q, rho0, ub)
            elif bc[0] == "velocity-simultaneous":  # the extension: all partners read before
                ub = np.asarray(bc[1], np.float32).astype(np.float64)
                old = Fn[x, j, k].copy()
                for q in range(19):
                    o = LR[q]
                    Fn[x, j, k, q] = feq(w, o, rho0, ub) - old[o] + feq(w, q, rho0, ub)
    for i, j, k in np.ndindex(nx, ny, nz):
        if solid[i, j, k]:
            rho[i, j, k], v[i, j, k] = rho0, 0.0
            continue
        f[i, j, k] = Fn[i, j, k]
        rho[i, j, k] = Fn[i, j, k].sum()
        v[i, j, k] = (E.T @ Fn[i, j, k]) / rho[i, j, k] + force[i, j, k] * 0.5 / rho[i, j, k]
    return f, Fn, rho, v


def bc(kind, value):
    if kind == "pressure":
        return BoundaryConfig("pressure", rho=value)
    if kind == "velocity-simultaneous":
        return BoundaryConfig("velocity", velocity=value, velocity_update="simultaneous")
    return BoundaryConfig("velocity", velocity=value)


@pytest.mark.parametrize("left,right", [
    (("velocity", (0.05, 0.01, -0.02)), ("pressure", 1.02)),
    (("pressure", 0.98), ("velocity", (-0.03, 0.0, 0.01))),
    (("velocity-simultaneous", (0.05, 0.01, -0.02)), ("pressure", 1.02)),
])
def test_face_conditions_match_a_second_restatement(left, right):
    nx, ny, nz = 6, 5, 5
    cfg = LBMConfig(nx=nx, ny=ny, nz=nz, viscosity=1.0 / 60.0, x_left=bc(*left),
                    x_right=bc(*right))
    solid = np.zeros((nx, ny, nz), np.int32)
    solid[:, 0, :] = 1          # a wall plane
    solid[1, 2, 2] = 1          # inner neighbour of a left-face cell
    solid[nx - 2, 3, 1] = 1     # inner neighbour of a right-face cell
    solid[3, 2, 1] = 1
    lat = O.LBMSolver3D(cfg, dtype=np.float64)
    lat.initialize(solid)
    rng = np.random.default_rng(5)
    shape = (nx, ny, nz)
    lat.rho[...] = 1.0 + 0.02 * rng.standard_normal(shape)
    lat.v[...] = 0.03 * rng.standard_normal((*shape, 3))
    lat.force[...] = 1e-4 * rng.standard_normal((*shape, 3))
    lat.F[...] = lat.w * (1.0 + 0.05 * rng.standard_normal((*shape, 19)))
    lat.f[...] = lat.F
    start = [a.copy() for a in (lat.f, lat.F, lat.rho, lat.v, lat.force)]
    lat.step()
    want = reference_step(*start, solid, lat.M, lat.invM, lat.S, lat.w, left, right,
                          float(lat.rho0))
    for name, got, exp in zip(("f", "F", "rho", "v"), (lat.f, lat.F, lat.rho, lat.v), want):
        np.testing.assert_allclose(got, exp, rtol=1e-12, atol=1e-14, err_msg=name)
    # the two velocity updates differ at O(1) on the velocity face: the other one's result is
    # far from what the oracle computed
    swap = {"velocity": "velocity-simultaneous", "velocity-simultaneous": "velocity"}
    other_l = (swap.get(left[0], left[0]), left[1])
    other_r = (swap.get(right[0], right[0]), right[1])
    other = reference_step(*start, solid, lat.M, lat.invM, lat.S, lat.w, other_l, other_r,
                           float(lat.rho0))
    x = 0 if left[0].startswith("velocity") else nx - 1
    assert np.abs(other[1][x] - lat.F[x]).max() > 1e-3
    np.testing.assert_allclose(other[1][2:4], lat.F[2:4], rtol=1e-12)  # interior cells agree
