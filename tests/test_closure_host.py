"""Host logic of the learned closure (no GPU): the coarse lattice in acoustic scaling, the
coarse mask rule, the solid-fraction occupancy feature and the prolongation of a coarse
state onto the fine lattice."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from fsi import closure as cl
from fsi.config import LBMConfig
from helpers import PERIODIC


def test_coarse_config_is_acoustic_scaling():
    fine = LBMConfig(nx=24, ny=12, nz=16, viscosity=0.04, force=(2e-5, -1e-6, 0.0), **PERIODIC)
    c = cl.coarse_config(fine)
    assert (c.nx, c.ny, c.nz) == (12, 6, 8)
    assert c.viscosity == pytest.approx(0.02)
    assert c.force == pytest.approx((4e-5, -2e-6, 0.0))
    assert c.population_storage == "f32" and c.collision_arithmetic == "fast"
    assert c.rho0 == fine.rho0
    with pytest.raises(ValueError):
        cl.coarse_config(LBMConfig(nx=23, ny=12, nz=16, viscosity=0.04, **PERIODIC))


def test_coarse_mask_needs_four_of_eight_solid_children():
    rng = np.random.default_rng(3)
    fine = (rng.uniform(size=(8, 6, 4)) < 0.45).astype(np.int32)
    got = cl.coarse_mask(fine)
    assert got.shape == (4, 3, 2) and got.dtype == np.int32
    for I in range(4):
        for J in range(3):
            for K in range(2):
                n = int(fine[2 * I:2 * I + 2, 2 * J:2 * J + 2, 2 * K:2 * K + 2].sum())
                assert got[I, J, K] == (1 if n >= 4 else 0)


def test_solid_fraction_is_the_share_of_solid_children():
    rng = np.random.default_rng(5)
    fine = (rng.uniform(size=(6, 4, 8)) < 0.3).astype(np.int32)
    frac = cl.solid_fraction(fine, device="cpu").numpy().reshape(3, 2, 4)
    for I in range(3):
        for J in range(2):
            for K in range(4):
                want = fine[2 * I:2 * I + 2, 2 * J:2 * J + 2, 2 * K:2 * K + 2].mean()
                assert frac[I, J, K] == np.float32(want)
    # the fraction and the coarse mask agree on which cells are solid
    assert np.array_equal(frac >= 0.5, cl.coarse_mask(fine).astype(bool))


def test_prolongation_copies_each_parent_to_its_eight_children():
    nx, ny, nz = 4, 6, 2
    coarse = torch.arange((nx // 2) * (ny // 2) * (nz // 2) * 19, dtype=torch.float32).reshape(-1, 19)
    fine = cl.prolongate(coarse, (nx, ny, nz)).reshape(nx, ny, nz, 19)
    c = coarse.reshape(nx // 2, ny // 2, nz // 2, 19)
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                assert torch.equal(fine[i, j, k], c[i // 2, j // 2, k // 2])


def test_restrict_rows_sums_fluid_children_in_kernel_order():
    """restrict_rows: fluid children added one by one in child order 4 di + 2 dj + dk (float32),
    divided by their count; w_q rho0 where all eight children are solid."""
    import torch
    from fsi import closure as cl
    rng = np.random.default_rng(0)
    nx, ny, nz = 8, 6, 4
    dist = rng.random((nx * ny * nz, 19)).astype(np.float32)
    solid = rng.random((nx, ny, nz)) < 0.4
    solid[0:2, 0:2, 0:2] = True
    rows = cl.restrict_rows(torch.from_numpy(dist), (nx, ny, nz), torch.from_numpy(solid),
                            1.25).numpy()
    f = dist.reshape(nx, ny, nz, 19)
    ref = np.zeros((nx // 2, ny // 2, nz // 2, 19), np.float32)
    for I in range(nx // 2):
        for J in range(ny // 2):
            for K in range(nz // 2):
                acc, n = np.zeros(19, np.float32), 0
                for ch in range(8):
                    i, j, k = 2 * I + (ch >> 2), 2 * J + ((ch >> 1) & 1), 2 * K + (ch & 1)
                    if not solid[i, j, k]:
                        acc, n = (acc + f[i, j, k]).astype(np.float32), n + 1
                ref[I, J, K] = acc / np.float32(n) if n else \
                    np.array(cl._W, np.float32) * np.float32(1.25)
    np.testing.assert_array_equal(rows, ref.reshape(-1, 19))
