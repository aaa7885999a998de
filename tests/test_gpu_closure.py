"""Learned coarse-grid closure (fsi.closure): the tcgen05 GEMM epilogues, the features, the
fused inference and the gradients against the CPU restatement (oracle/closure_oracle.py),
training, the gain over the coarse run without the network, and the guard fallback."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from fsi import _native as nat
from fsi import closure as cl
from fsi.config import LBMConfig
from fsi.lbm3d import LBMSolver3D
from helpers import PERIODIC, channel_mask, rel_l2
from oracle import closure_oracle as O

pytestmark = pytest.mark.gpu


def bf(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.asarray(a, np.float32)).cuda().to(torch.bfloat16)


def host(t: torch.Tensor) -> np.ndarray:
    return t.float().cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("m,n,k", [(300, 64, 656), (128, 32, 64), (257, 128, 96), (64, 656, 1024)])
def test_gemm_store_and_atomic(m, n, k):
    rng = np.random.default_rng(m + n + k)
    a, b = bf(rng.standard_normal((m, k))), bf(rng.standard_normal((n, k)))
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    want = host(a) @ host(b).T
    c = torch.zeros((m, n), dtype=torch.float32, device="cuda")
    cl._gemm(a, b, k, k, m, n, k, nat.GEMM_STORE, err, c=c, ldc=n)
    np.testing.assert_allclose(c.cpu().numpy(), want, rtol=1e-5, atol=1e-4)
    c.zero_()
    cl._gemm(a, b, k, k, m, n, k, nat.GEMM_ATOMIC, err, c=c, ldc=n, k_chunk=64)  # split-K
    np.testing.assert_allclose(c.cpu().numpy(), want, rtol=1e-5, atol=1e-4)
    assert int(err.item()) == 0


def test_gemm_gelu_epilogues():
    rng = np.random.default_rng(7)
    m, n, k = 384, 64, 656
    a, b = bf(rng.standard_normal((m, k)) * 0.1), bf(rng.standard_normal((n, k)) * 0.1)
    bias = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    h = torch.empty((m, n), dtype=torch.bfloat16, device="cuda")
    ht = torch.empty((n, m), dtype=torch.bfloat16, device="cuda")
    z = torch.empty((m, n), dtype=torch.float32, device="cuda")
    cl._gemm(a, b, k, k, m, n, k, nat.GEMM_GELU_FWD, err, bias=bias, h=h, ht=ht, ldht=m, zout=z)
    zw = host(a) @ host(b).T + bias.double().cpu().numpy()
    np.testing.assert_allclose(z.cpu().numpy(), zw, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(host(h), O.gelu(zw), rtol=1e-2, atol=1e-2)
    np.testing.assert_array_equal(host(ht), host(h).T)
    g = bf(rng.standard_normal((m, 32)))
    w = bf(rng.standard_normal((n, 32)))
    d = torch.empty((m, n), dtype=torch.bfloat16, device="cuda")
    dt = torch.empty((n, m), dtype=torch.bfloat16, device="cuda")
    cl._gemm(g, w, 32, 32, m, n, 32, nat.GEMM_GELU_BWD, err, h=d, ht=dt, ldht=m, zin=z)
    want = (host(g) @ host(w).T) * O.gelu_grad(z.double().cpu().numpy())
    np.testing.assert_allclose(host(d), want, rtol=1e-2, atol=1e-2)
    np.testing.assert_array_equal(host(dt), host(d).T)
    assert int(err.item()) == 0


def small_lattice(seed=0, steps=5):
    cfg = LBMConfig(nx=10, ny=9, nz=8, viscosity=0.05, force=(1e-4, 2e-5, 0.0), **PERIODIC)
    mask = channel_mask(10, 9, 8)
    mask[4:6, 3:5, 3:5] = 1
    lbm = LBMSolver3D(cfg)
    lbm.initialize(mask)
    for _ in range(steps):
        lbm.step()
    return lbm, mask


def numpy_features(lbm, mask, cells, pop_scale, force_scale, frac=None):
    f = lbm.distribution_numpy()
    g = lbm.force_numpy()
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, np.float32)
    nx, ny, nz = mask.shape
    out = np.zeros((len(cells), 656))
    for r, c in enumerate(cells):
        i, j, k = c // (ny * nz), (c // nz) % ny, c % nz
        col = 0
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    a, b, e = (i + dx) % nx, (j + dy) % ny, (k + dz) % nz
                    solid = mask[a, b, e] > 0
                    pops = np.zeros(19) if solid else (f[a, b, e] - w * np.float32(lbm.config.rho0)) * pop_scale
                    out[r, col:col + 19] = pops
                    out[r, col + 19] = (frac[a, b, e] if frac is not None else (1.0 if solid else 0.0))
                    out[r, col + 20:col + 23] = g[a, b, e] * force_scale
                    col += 24
    return out


def test_features_match_numpy():
    lbm, mask = small_lattice()
    cells = np.array([0, 17, 123, 300, 555, 719])
    x = cl.features(lbm, torch.from_numpy(cells.astype(np.int32)).cuda(), 30.0, 1e3)
    want = numpy_features(lbm, mask, cells, 30.0, 1e3)
    np.testing.assert_allclose(host(x), O.bf16(want.astype(np.float32)), rtol=0, atol=1e-6)


def test_solid_fraction_feature_and_inference():
    """With a per-cell solid fraction the occupancy feature is that fraction, in the training
    features and in the fused inference alike."""
    lbm, mask = small_lattice()
    rng = np.random.default_rng(7)
    frac_np = np.where(mask > 0, rng.uniform(0.5, 1.0, mask.shape), rng.uniform(0.0, 0.49, mask.shape))
    frac_np = frac_np.astype(np.float32)
    frac = torch.from_numpy(frac_np.reshape(-1)).cuda()
    cells = np.array([0, 17, 123, 300, 555, 719])
    x = cl.features(lbm, torch.from_numpy(cells.astype(np.int32)).cuda(), 30.0, 1e3, frac)
    want = numpy_features(lbm, mask, cells, 30.0, 1e3, frac_np)
    np.testing.assert_allclose(host(x), O.bf16(want.astype(np.float32)), rtol=0, atol=1e-6)
    net = cl.ClosureMLP(seed=3)
    net.pop_scale, net.force_scale, net.out_scale = 30.0, 1e3, 250.0
    corr = torch.zeros((19, lbm.n_cells), dtype=torch.float32, device="cuda")
    cl.infer(lbm, net.weights_struct(), corr, cl.rows_buffer(lbm), net.err, frac)
    net.check()
    fluid = np.nonzero(mask.reshape(-1) == 0)[0]
    xf = cl.features(lbm, torch.from_numpy(fluid.astype(np.int32)).cuda(), net.pop_scale, net.force_scale, frac)
    pad = (-len(fluid)) % 128
    xp = torch.cat([xf, torch.zeros((pad, 656), dtype=xf.dtype, device="cuda")])
    y = net.predict(xp)[:len(fluid)] / net.out_scale
    got = corr[:, torch.from_numpy(fluid).cuda()].t()
    assert rel_l2(got.cpu().numpy(), y.cpu().numpy()) < 2e-3


def test_fused_inference_matches_unfused_passes():
    lbm, mask = small_lattice()
    net = cl.ClosureMLP(seed=3)
    net.pop_scale, net.force_scale, net.out_scale = 30.0, 1e3, 250.0
    corr = torch.zeros((19, lbm.n_cells), dtype=torch.float32, device="cuda")
    cl.infer(lbm, net.weights_struct(), corr, cl.rows_buffer(lbm), net.err)
    net.check()
    fluid = np.nonzero(mask.reshape(-1) == 0)[0]
    cells = torch.from_numpy(fluid.astype(np.int32)).cuda()
    x = cl.features(lbm, cells, net.pop_scale, net.force_scale)
    pad = (-len(fluid)) % 128
    xp = torch.cat([x, torch.zeros((pad, 656), dtype=x.dtype, device="cuda")])
    y = net.predict(xp)[:len(fluid)] / net.out_scale
    got = corr[:, torch.from_numpy(fluid).cuda()].t()
    assert rel_l2(got.cpu().numpy(), y.cpu().numpy()) < 2e-3
    solid = np.nonzero(mask.reshape(-1))[0]
    assert float(corr[:, torch.from_numpy(solid).cuda()].abs().max()) == 0.0


@pytest.mark.parametrize("steps", [6, 7])
def test_fused_inference_on_a_lattice_of_many_columns(steps):
    """40x30x70: several inference columns in y and z, partial last blocks on both axes, many
    segments per CTA; every fluid cell's correction against the unfused feature rows + GEMMs,
    on both AA parities; solid cells get no correction."""
    nx, ny, nz = 40, 30, 70
    cfg = LBMConfig(nx=nx, ny=ny, nz=nz, viscosity=0.04, force=(5e-5, 1e-5, -2e-5), **PERIODIC)
    mask = channel_mask(nx, ny, nz)
    rng = np.random.default_rng(11)
    for _ in range(12):
        c = rng.integers([2, 3, 3], [nx - 2, ny - 3, nz - 3])
        mask[c[0] - 1:c[0] + 2, c[1] - 1:c[1] + 2, c[2] - 2:c[2] + 1] = 1
    lbm = LBMSolver3D(cfg)
    lbm.initialize(mask)
    for _ in range(steps):
        lbm.step()
    net = cl.ClosureMLP(seed=9)
    net.pop_scale, net.force_scale, net.out_scale = 30.0, 1e3, 250.0
    frac = torch.from_numpy(np.where(mask > 0, 0.75, 0.125).astype(np.float32).reshape(-1)).cuda()
    corr = torch.full((19, lbm.n_cells), 7.0, dtype=torch.float32, device="cuda")
    cl.infer(lbm, net.weights_struct(), corr, cl.rows_buffer(lbm), net.err, frac)
    net.check()
    fluid = np.nonzero(mask.reshape(-1) == 0)[0]
    x = cl.features(lbm, torch.from_numpy(fluid.astype(np.int32)).cuda(), net.pop_scale, net.force_scale, frac)
    pad = (-len(fluid)) % 128
    xp = torch.cat([x, torch.zeros((pad, 656), dtype=x.dtype, device="cuda")])
    y = net.predict(xp)[:len(fluid)] / net.out_scale
    got = corr[:, torch.from_numpy(fluid).cuda()].t()
    assert rel_l2(got.cpu().numpy(), y.cpu().numpy()) < 2e-3
    solid = np.nonzero(mask.reshape(-1))[0]
    assert float(corr[:, torch.from_numpy(solid).cuda()].abs().max()) == 0.0


def test_in_place_inference_equals_inference_then_apply():
    """fsi_closure_infer_apply gives bit for bit the populations of fsi_closure_infer followed
    by fsi_closure_apply (both parities of the AA layout)."""
    for steps in (4, 5):
        lbm, mask = small_lattice(steps=steps)
        net = cl.ClosureMLP(seed=5)
        net.pop_scale, net.force_scale, net.out_scale = 30.0, 1e3, 250.0
        w = net.weights_struct()
        rows = cl.rows_buffer(lbm)
        before = lbm._pops.clone()
        corr = torch.zeros((19, lbm.n_cells), dtype=torch.float32, device="cuda")
        cl.infer(lbm, w, corr, rows, net.err)
        nat.call("fsi_closure_apply", lbm._desc, nat.ptr(lbm._pops), nat.ptr(lbm.flags), lbm.steps_done,
                 nat.ptr(corr), nat.stream_ptr())
        want = lbm._pops.clone()
        lbm._pops.copy_(before)
        cl.infer_apply(lbm, w, rows, net.err)
        net.check()
        assert torch.equal(lbm._pops, want), steps
        assert not torch.equal(want, before)


def test_gradients_match_the_oracle():
    rng = np.random.default_rng(11)
    net = cl.ClosureMLP(seed=5)
    m = 256
    xh = O.bf16(rng.standard_normal((m, 656)).astype(np.float32) * 0.5)
    xh[:, cl._ZERO_COLS] = 0.0
    target = rng.standard_normal((m, 19)) * 0.5
    x = torch.from_numpy(xh.astype(np.float32)).cuda().to(torch.bfloat16)
    y, acts = net.forward(x, keep=True)
    t = torch.from_numpy(target.astype(np.float32)).cuda()
    loss = net.backward(x, y, acts, t, xt=x.t().contiguous())
    net.check()
    P = [v.double().cpu().numpy() for v in net.views]
    yw, aw = O.forward(xh, P[0], P[1], P[2], P[3], P[4], P[5], P[6])
    np.testing.assert_allclose(y.cpu().numpy(), yw, rtol=2e-2, atol=2e-3)
    lw, gw = O.backward(xh, yw, aw, target, P[2], P[4], P[6], P[7])
    assert loss == pytest.approx(lw, rel=1e-3)
    names = ["W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"]
    for name, g in zip(names, net.gviews):
        want = gw[name]
        got = g.double().cpu().numpy()
        if name == "W4":
            want, got = want[:19], got[:19]
        if name == "b4":
            want, got = want[:19], got[:19]
        if name == "W1":
            keep = [c for c in range(656) if c not in set(cl._ZERO_COLS)]
            want, got = want[:, keep], got[:, keep]
        assert rel_l2(got, want) < 3e-2, name


def test_training_fits_a_teacher_network():
    rng = np.random.default_rng(2)
    teacher = cl.ClosureMLP(seed=9)
    m = 8192
    xh = rng.standard_normal((m, 656)).astype(np.float32)
    xh[:, cl._ZERO_COLS] = 0
    x = torch.from_numpy(xh).cuda().to(torch.bfloat16)
    t = teacher.predict(x).contiguous()
    student = cl.ClosureMLP(seed=1)
    tr = cl.ClosureTrainer(student)
    tr.x, tr.t = x, t
    hist = tr.fit(steps=300, batch=4096, lr=3e-3)
    assert hist[-1] < 0.2 * hist[0], (hist[0], hist[-1])


def channel_scene(seed, n=(32, 16, 16)):
    from fsi import scenes
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    mask = scenes.wall_mask(nx, ny, nz)
    for _ in range(3):
        c = [rng.uniform(4, nx - 4), rng.uniform(5, ny - 5), rng.uniform(5, nz - 5)]
        scenes.add_sphere(mask, c, rng.uniform(2.0, 3.5))
    cfg = LBMConfig(nx=nx, ny=ny, nz=nz, viscosity=(0.6 - 0.5) / 3.0, force=(2e-5, 0.0, 0.0),
                    **PERIODIC)
    return cfg, mask


def coarse_errors(cfg, mask, net, steps=40):
    """rel-L2 velocity error of the plain coarse run and of the closure run against the
    restricted fine run, after `steps` coarse steps."""
    fine = LBMSolver3D(cfg)
    fine.initialize(mask)
    ccfg = cl.coarse_config(cfg)
    plain = LBMSolver3D(ccfg)
    plain.initialize(cl.coarse_mask(mask))
    sim = cl.ClosureSimulation(cfg, mask, net, check_every=0)
    for _ in range(steps):
        fine.step()
        fine.step()
        plain.step()
        sim.step()
    ref = cl.restrict(fine, plain)
    tmp = LBMSolver3D(ccfg)
    tmp.initialize(cl.coarse_mask(mask))
    tmp.load_populations(ref)
    u_ref = tmp.velocity_numpy()
    return rel_l2(plain.velocity_numpy(), u_ref), rel_l2(sim.velocity_numpy(), u_ref)


def test_trained_closure_beats_the_plain_coarse_run():
    net = cl.ClosureMLP(seed=0)
    tr = cl.ClosureTrainer(net)
    for seed in (100, 101, 102, 103):
        cfg, mask = channel_scene(seed)
        tr.add_run(cfg, mask, warmup=20, snapshots=12, every=4)
    rows = tr.build()
    assert rows > 10_000
    hist = tr.fit(steps=400, batch=8192, lr=2e-3)
    assert hist[-1] < hist[0]
    cfg, mask = channel_scene(300)  # held out
    e_plain, e_closure = coarse_errors(cfg, mask, net)
    assert e_closure < e_plain, (e_plain, e_closure)


def test_guard_falls_back_to_the_fine_grid():
    cfg, mask = channel_scene(7)
    net = cl.ClosureMLP(seed=0)
    sim = cl.ClosureSimulation(cfg, mask, net, mach_tol=1e-12, check_every=3)
    for _ in range(5):
        sim.step()
    assert sim.on_fine_grid and sim.fallback_step == 3 and "Mach" in sim.fallback_reason
    assert sim.fine.steps_done == 4
    u = sim.velocity_numpy()
    assert u.shape == (16, 8, 8, 3) and np.all(np.isfinite(u))


def test_bounded_wait_gives_up_reports_and_releases_the_other_role():
    """A wait on an mbarrier that nothing arrives on ends after its clock limit with error code
    7 (no fault, no hang); the abortable wait of a second role returns on the first role's abort
    flag without a code of its own; the context stays usable afterwards."""
    import time

    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nat.call("fsi_selftest_wait_limit", nat.ptr(err), nat.ptr(out), nat.stream_ptr())
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    assert err.item() == 7
    assert out.tolist() == [0, 0]
    assert 0.2 < elapsed < 20.0  # 2^31 SM clock cycles
    x = torch.arange(8, device="cuda", dtype=torch.float32)
    assert float((x * 2).sum()) == 56.0


def test_momentum_exchange_drag_matches_link_sum_of_the_oracle():
    """fsi.closure.momentum_exchange on the GPU lattice against an explicit loop over the
    bounce-back links of the oracle's (bit-identical) populations: 2 c_q f_q* per link, summed
    over fluid cells next to a body cell; the drive pushes the bodies downstream (+x)."""
    from fsi import scenes
    from oracle import oracle as OR

    cfg, mask, body = scenes.closure_channel(5, nx=24, ny=16, nz=16, rmin=2.0, rmax=3.5)
    assert body.sum() > 0
    lbm = LBMSolver3D(cfg)
    lbm.initialize(mask)
    ref = OR.LBMSolver3D(cfg)
    ref.initialize(mask)
    for _ in range(30):
        lbm.step()
        ref.step()
    f = ref.distribution_numpy()
    fluid = mask == 0
    expect = np.zeros(3)
    nx, ny, nz = mask.shape
    for i, j, k in zip(*np.nonzero(fluid)):
        for q in range(1, 19):
            c = (cl._EX[q], cl._EY[q], cl._EZ[q])
            if body[(i + c[0]) % nx, (j + c[1]) % ny, (k + c[2]) % nz]:
                expect += 2.0 * float(f[i, j, k, cl._OPP[q]]) * np.array(c, np.float64)
    got = cl.momentum_exchange(lbm, body)
    np.testing.assert_allclose(got, expect, rtol=1e-12, atol=1e-18)
    assert got[0] > 0.0


def test_evaluation_reports_drag_and_fallback():
    from fsi import scenes

    cfg, mask, body = scenes.closure_channel(301, nx=32, ny=16, nz=16, rmin=2.0, rmax=3.5)
    net = cl.ClosureMLP(seed=0)
    r = cl.evaluate(cfg, mask, net, coarse_steps=6, body_mask=body, check_every=3)
    for k in ("drag_fine", "drag_plain", "drag_closure", "drag_error_plain",
              "drag_error_closure", "velocity_l2_plain", "velocity_l2_closure"):
        assert np.isfinite(r[k]), k
    assert r["drag_fine"] > 0.0
    assert r["fallback"] is None or isinstance(r["fallback"], str)


def test_restrict_rows_is_the_restriction_kernel():
    from fsi import scenes
    cfg, mask, _ = scenes.closure_channel(7, nx=16, ny=12, nz=12, balls=2, rmin=2.0, rmax=3.0)
    fine = LBMSolver3D(cfg)
    fine.initialize(mask)
    for _ in range(5):
        fine.step()
    coarse = LBMSolver3D(cl.coarse_config(cfg))
    coarse.initialize(cl.coarse_mask(mask))
    dist = torch.from_numpy(fine.distribution_numpy().reshape(-1, 19)).cuda()
    rows = cl.restrict_rows(dist, (cfg.nx, cfg.ny, cfg.nz),
                            torch.from_numpy(mask > 0).cuda(), cfg.rho0)
    assert torch.equal(rows, cl.restrict(fine, coarse))


def test_batched_training_rows_are_the_per_scene_rows(tmp_path, monkeypatch):
    """ClosureTrainer.add_batch (the scenes' fine runs as one autotuned LatticeBatch) gives
    the rows of add_run scene by scene, bit for bit, and keeps the autotuner's record."""
    from fsi import scenes
    monkeypatch.setenv("FSI_AUTOTUNE_CACHE", str(tmp_path / "autotune.json"))
    seeds = [100, 101, 102]
    scenes_ = [scenes.closure_channel(sd, nx=24, ny=12, nz=12, balls=2, rmin=2.0, rmax=3.0)
               for sd in seeds]
    kw = dict(warmup=2, snapshots=3, every=3, cell_fraction=0.5)
    one = cl.ClosureTrainer(cl.ClosureMLP(seed=0))
    for sd, (cfg, mask, _) in zip(seeds, scenes_):
        one.add_run(cfg, mask, seed=sd, **kw)
    many = cl.ClosureTrainer(cl.ClosureMLP(seed=0))
    rec = many.add_batch([c for c, _, _ in scenes_], [m for _, m, _ in scenes_], seeds=seeds,
                         **kw)
    assert rec["scenes"] == 3 and rec["fine_steps"] == 2 + 3 * 3
    assert rec["tuning"]["best"] is not None and rec["tuning"]["ms"]
    assert many.batch_records == [rec]
    assert one.build() == many.build() > 0
    assert torch.equal(one.x, many.x)
    assert torch.equal(one.t, many.t)
    assert (one.net.pop_scale, one.net.force_scale, one.net.out_scale) == \
        (many.net.pop_scale, many.net.force_scale, many.net.out_scale)
