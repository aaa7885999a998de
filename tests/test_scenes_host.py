"""Seeded scene generators of the benchmark workloads (no GPU): masks, sphere packings and
particle sets are deterministic per seed, non-overlapping, inside their domains and of the
stated sizes."""
from __future__ import annotations

import numpy as np

from fsi import scenes


def test_wall_mask_and_sphere():
    m = scenes.wall_mask(5, 6, 7)
    assert m.shape == (5, 6, 7) and m.dtype == np.int32
    assert m[:, 0].all() and m[:, -1].all() and m[:, :, 0].all() and m[:, :, -1].all()
    assert not m[:, 1:-1, 1:-1].any()
    s = np.zeros((12, 12, 12), np.int32)
    added = scenes.add_sphere(s, (6.0, 6.0, 6.0), 3.0)
    ii, jj, kk = np.meshgrid(*[np.arange(12)] * 3, indexing="ij")
    inside = (ii - 6.0) ** 2 + (jj - 6.0) ** 2 + (kk - 6.0) ** 2 <= 9.0
    assert added == inside.sum() and np.array_equal(s.astype(bool), inside)
    assert scenes.add_sphere(s, (6.0, 6.0, 6.0), 3.0) == 0


def test_sphere_packing_is_seeded_disjoint_and_fills_the_fraction():
    shape = (48, 40, 44)
    mask, c, r = scenes.sphere_packing(shape, 0.10, 3.0, 6.0, seed=5)
    mask2, c2, r2 = scenes.sphere_packing(shape, 0.10, 3.0, 6.0, seed=5)
    assert np.array_equal(mask, mask2) and np.array_equal(c, c2) and np.array_equal(r, r2)
    assert mask.sum() >= 0.10 * np.prod(shape)
    assert np.all((r >= 3.0) & (r <= 6.0))
    d = np.linalg.norm(c[:, None] - c[None], axis=-1)
    iu = np.triu_indices(len(r), 1)
    assert np.all(d[iu] >= (r[:, None] + r[None])[iu])
    for a in range(3):  # centres keep the margin of one cell plus the radius
        assert np.all(c[:, a] - r >= 1.0 - 1e-9) and np.all(c[:, a] + r <= shape[a] - 2 + 1e-9)


def test_cube_particles_order_and_positions():
    p = scenes.cube_particles((3, 4, 5), 2, 2)
    assert p.shape == (64, 3) and p.dtype == np.float32
    # cell by cell: the first 8 particles are the sub-cell centres of cell (3, 4, 5)
    assert np.all(np.floor(p[:8]) == [3, 4, 5])
    assert sorted(map(tuple, p[:8] - [3, 4, 5])) == sorted(
        (a, b, c) for a in (0.25, 0.75) for b in (0.25, 0.75) for c in (0.25, 0.75))
    rng = np.random.default_rng(0)
    q = scenes.cube_particles((3, 4, 5), 2, 2, rng)
    assert np.all(np.floor(q * 2) == np.floor(p * 2))  # jitter stays within the sub-cell


def test_random_cubes_are_disjoint_and_seeded():
    a = scenes.random_cubes(64, 5, 8, seed=9)
    assert np.array_equal(a, scenes.random_cubes(64, 5, 8, seed=9))
    assert a.shape == (5 * 8 ** 3 * 8, 3)
    cells = [set(map(tuple, np.floor(blk).astype(int))) for blk in np.split(a, 5)]
    for i in range(5):
        for j in range(i + 1, 5):
            assert not cells[i] & cells[j]
    assert a.min() >= 4 and a.max() < 64 - 4


def test_headline_solid_workload_has_2097152_particles():
    cfg, pos = scenes.cubes_mpm()
    assert pos.shape == (2_097_152, 3) and cfg.max_particles == 2_097_152
    assert (cfg.nx, cfg.ny, cfg.nz) == (256, 256, 256)
    assert pos.min() >= 0 and pos.max() < 256


def test_coupled_workloads():
    cfg, mask, pos = scenes.coupled_smoke(steps=10)
    assert pos.shape == (4096, 3) and pos.min() >= 12.0 and pos.max() < 20.0
    assert mask.shape == (48, 32, 32) and cfg.coupling.mpm_substeps_per_lbm_step == 10
    cfg, mask, pos, young = scenes.coupled_bodies(nx=112, ny=48, nz=48, bodies=4, seed=7)
    assert len(pos) == len(young) and cfg.mpm.max_particles == len(pos)
    assert cfg.lbm.x_left.boundary_type == "velocity" and cfg.lbm.x_right.boundary_type == "pressure"
    assert np.all((pos >= 0) & (pos < [112, 48, 48]))
    assert 1 <= len(np.unique(young)) <= 4 and np.all((young >= 0.02) & (young <= 0.1))
    assert cfg.lbm.initial_velocity == (0.05, 0.0, 0.0)  # the channel starts at its inflow


def test_batch_scenes_are_seeded_and_within_bounds():
    a = scenes.batch_scenes(count=6, seed=4, edges=(32, 48))
    b = scenes.batch_scenes(count=6, seed=4, edges=(32, 48))
    for (ca, ma, pa, ya), (cb, mb, pb, yb) in zip(a, b):
        assert ca.lbm.nx == cb.lbm.nx and np.array_equal(pa, pb) and np.array_equal(ya, yb)
        n = ca.lbm.nx
        assert n in (32, 48) and ca.lbm.population_storage == "f16"
        assert ma.shape == (n, n, n) and len(pa) == len(ya) == ca.mpm.max_particles
        assert np.all((pa >= 0) & (pa < n))
        assert 1 <= len(np.unique(ya)) <= 4


def test_closure_channel_scenes():
    """The learned closure's data-set scenes: seeded, four balls inside the walls, walls and
    balls together in the solid mask, different geometry per seed."""
    from fsi import scenes

    cfg, mask, body = scenes.closure_channel(100)
    cfg2, mask2, body2 = scenes.closure_channel(100)
    assert (mask == mask2).all() and (body == body2).all()
    assert mask.shape == body.shape == (48, 24, 24) == (cfg.nx, cfg.ny, cfg.nz)
    assert 0.005 < body.mean() < 0.1
    assert ((mask >= body) & (mask >= scenes.wall_mask(48, 24, 24))).all()
    assert not body[:, 0, :].any() and not body[:, :, -1].any()
    _, _, other = scenes.closure_channel(300)
    assert (other != body).any()
    assert cfg.force == (2e-5, 0.0, 0.0)
