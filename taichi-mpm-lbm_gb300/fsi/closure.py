"""Learned coarse-grid closure (no reference counterpart).

A lattice run on a grid 2x coarser than a reference ("fine") run, with lattice units kept
(acoustic scaling: dx and dt double, so velocities in lattice units are unchanged, the
lattice viscosity halves and a body force doubles), is corrected after every step by a
per-cell MLP: 621 features of the cell's 3^3 neighbourhood (19 populations, occupancy and
3 force components per neighbour, laid out in 27 groups of 24 columns, 656 columns in all)
-> 64 -> 64 -> 64 -> 19 corrections of the post-stream
populations, GELU activations, BF16 weights with FP32 accumulation. Training pairs come
from restricted fine runs of the plain solver: the correction is what the coarse step
misses, R(f(t + 2 dt_f)) - C(R(f(t))), with R the 2x2x2 restriction and C one coarse step.

Every matrix product (forward, backward and weight gradients) runs on the tcgen05 tensor
cores through ``fsi_closure_gemm``; inference during stepping is one fused kernel
(``fsi_closure_infer``). ``ClosureSimulation`` watches mass drift and the local Mach number
and falls back to the plain fine-grid solver (prolongating the coarse state) when a guard
trips.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math

import numpy as np
import torch

from . import _native as nat
from .config import LBMConfig
from .lbm3d import LBMSolver3D

FEATURES = 656  # 27 groups of 24 columns (23 values + 1 zero) + 8 zero columns
# feature columns that always hold zero (the last of each group, and the tail)
_ZERO_COLS = [c for c in range(FEATURES) if c >= 27 * 24 or c % 24 == 23]
HIDDEN = 64
OUT = 19
OUT_PAD = 32
_CS = 1.0 / math.sqrt(3.0)


# ----------------------------------------------------------------- grids
def coarse_config(fine: LBMConfig) -> LBMConfig:
    """The 2x coarser lattice in acoustic scaling: half the cells per axis, half the lattice
    viscosity, twice the body force, FP32 populations with the reduced-operation collision
    (the learned correction is trained against this same coarse step)."""
    for n in (fine.nx, fine.ny, fine.nz):
        if n % 2:
            raise ValueError("the fine lattice needs even sizes.")
    return dataclasses.replace(fine, nx=fine.nx // 2, ny=fine.ny // 2, nz=fine.nz // 2,
                               viscosity=fine.viscosity / 2.0,
                               force=tuple(2.0 * g for g in fine.force),
                               population_storage="f32", collision_arithmetic="fast",
                               mrt_rates=None)


def coarse_mask(fine_mask: np.ndarray) -> np.ndarray:
    """A coarse cell is solid when at least 4 of its 8 children are."""
    m = np.asarray(fine_mask) > 0
    nx, ny, nz = m.shape
    c = m.reshape(nx // 2, 2, ny // 2, 2, nz // 2, 2).sum(axis=(1, 3, 5))
    return (c >= 4).astype(np.int32)


def solid_fraction(fine_mask: np.ndarray, device=None) -> torch.Tensor:
    """Share of each coarse cell's 8 fine children that are solid (float32 [Nc], device): the
    occupancy feature of the network, which keeps the sub-cell geometry the coarse mask
    loses."""
    m = np.asarray(fine_mask) > 0
    nx, ny, nz = m.shape
    f = m.reshape(nx // 2, 2, ny // 2, 2, nz // 2, 2).mean(axis=(1, 3, 5)).astype(np.float32)
    return torch.from_numpy(f.reshape(-1)).to(device if device is not None else nat.device())


def restrict(fine: LBMSolver3D, coarse: LBMSolver3D) -> torch.Tensor:
    """Mean post-stream populations of the fluid children, [Nc, 19] (device)."""
    out = torch.empty((coarse.n_cells, OUT), dtype=torch.float32, device=fine._device)
    nat.call("fsi_closure_restrict", fine._desc, nat.ptr(fine._pops), nat.ptr(fine.flags),
             fine.steps_done, coarse._desc, nat.ptr(out), nat.stream_ptr())
    return out


_W = (1.0 / 3.0,) + (1.0 / 18.0,) * 6 + (1.0 / 36.0,) * 12


def restrict_rows(dist: torch.Tensor, shape, solid: torch.Tensor, rho0: float) -> torch.Tensor:
    """``restrict`` of fine lattices given as their post-stream populations in the reference
    layout: ``dist`` device float32 [k*nx*ny*nz][19] holds k lattices of one shape one after
    another (e.g. consecutive lattices of ``LatticeBatch.distribution``), ``solid`` their
    solid masks (device bool [k, nx, ny, nz], or [nx, ny, nz] for k = 1). The fluid children of
    each coarse cell are summed in the kernel's order (child (di, dj, dk) = 4 di + 2 dj + dk)
    and divided by their count, w_q rho0 where all eight are solid: bit for bit the kernel's
    result. Returns [k*Nc][19]."""
    nx, ny, nz = shape
    k = dist.shape[0] // (nx * ny * nz)
    f = dist.view(k, nx // 2, 2, ny // 2, 2, nz // 2, 2, OUT)
    fluid = (~solid).reshape(k, nx // 2, 2, ny // 2, 2, nz // 2, 2, 1)
    acc = torch.zeros((k, nx // 2, ny // 2, nz // 2, OUT), dtype=torch.float32,
                      device=dist.device)
    nf = torch.zeros((k, nx // 2, ny // 2, nz // 2, 1), dtype=torch.float32, device=dist.device)
    for ch in range(8):
        di, dj, dk = ch >> 2, (ch >> 1) & 1, ch & 1
        keep = fluid[:, :, di, :, dj, :, dk, :]
        acc = acc + torch.where(keep, f[:, :, di, :, dj, :, dk, :], 0.0)
        nf = nf + keep.to(torch.float32)
    rest = torch.tensor(_W, dtype=torch.float32, device=dist.device) * np.float32(rho0)
    return torch.where(nf > 0, acc / nf.clamp(min=1.0), rest).reshape(-1, OUT)


def prolongate(coarse_f: torch.Tensor, shape) -> torch.Tensor:
    """Each fine cell takes its parent's populations, [Nf, 19]."""
    nx, ny, nz = shape
    f = coarse_f.reshape(nx // 2, ny // 2, nz // 2, OUT)
    f = f.repeat_interleave(2, 0).repeat_interleave(2, 1).repeat_interleave(2, 2)
    return f.reshape(-1, OUT).contiguous()


# D3Q19 velocities in the reference's order (fsi/lbm3d.py:221-239) and opposite directions.
_EX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
_EY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1])
_EZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1])
_OPP = np.array([0] + [q + 1 if q % 2 else q - 1 for q in range(1, 19)])


def _near(body: np.ndarray) -> np.ndarray:
    """Cells with a cell of ``body`` in their periodic 3^3 neighbourhood (bool)."""
    b = np.asarray(body) > 0
    out = np.zeros_like(b)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                out |= np.roll(b, (dx, dy, dz), axis=(0, 1, 2))
    return out


def momentum_exchange(lbm: LBMSolver3D, body_mask: np.ndarray) -> np.ndarray:
    """Hydrodynamic force on the bodies of ``body_mask`` (bool/0-1 (nx, ny, nz)), in the
    lattice's units, by momentum exchange over the half-way bounce-back links: every
    population that left a fluid cell x towards a body cell x + c_q came back reversed, so the
    body received 2 c_q f_q*(x); after the step that population is the post-stream f_opp(q)(x).
    Float64 sums of the float32 populations."""
    f = lbm.distribution_numpy()
    body = np.asarray(body_mask) > 0
    fluid = lbm.solid_numpy() == 0
    out = np.zeros(3)
    for q in range(1, 19):
        c = (int(_EX[q]), int(_EY[q]), int(_EZ[q]))
        links = fluid & np.roll(body, shift=(-c[0], -c[1], -c[2]), axis=(0, 1, 2))
        total = float(f[..., _OPP[q]][links].astype(np.float64).sum())
        out += 2.0 * total * np.array(c, np.float64)
    return out


# ------------------------------------------------------------------- net
def _gemm(a, b, lda, ldb, m, n, k, mode, err, c=None, ldc=0, bias=None, h=None, ht=None,
          ldht=0, zout=None, zin=None, k_chunk=None):
    d = nat.ClosureGemmDesc()
    d.a, d.b = a.data_ptr(), b.data_ptr()
    d.lda, d.ldb, d.m, d.n, d.k = lda, ldb, m, n, k
    d.k_chunk = k_chunk or ((k + 63) // 64 * 64)
    d.mode = mode
    d.ldc = ldc
    for name, t in (("c", c), ("bias", bias), ("h", h), ("ht", ht), ("zout", zout), ("zin", zin)):
        setattr(d, name, None if t is None else t.data_ptr())
    d.ldht = ldht
    d.err = err.data_ptr()
    nat.call("fsi_closure_gemm", ctypes.byref(d), nat.stream_ptr())


class ClosureMLP:
    """Parameters (FP32 master, BF16 copies), Adam state and the tensor-core passes."""

    def __init__(self, seed: int = 0, device=None, use_fraction: bool = True):
        self.device = device or nat.device()
        # Occupancy feature: the solid fraction of each coarse cell (from the fine mask) when
        # True, else the coarse cell's 0/1 flag.
        self.use_fraction = use_fraction
        nat.load()
        g = torch.Generator().manual_seed(seed)
        sizes = [(HIDDEN, FEATURES), (HIDDEN,), (HIDDEN, HIDDEN), (HIDDEN,), (HIDDEN, HIDDEN),
                 (HIDDEN,), (OUT_PAD, HIDDEN), (OUT_PAD,)]
        total = sum(int(np.prod(s)) for s in sizes)
        self.params = torch.zeros(total, dtype=torch.float32, device=self.device)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.views, self.gviews, off = [], [], 0
        for s in sizes:
            n = int(np.prod(s))
            self.views.append(self.params[off:off + n].view(*s))
            self.gviews.append(self.grads[off:off + n].view(*s))
            off += n
        W1, _, W2, _, W3, _, W4, _ = self.views
        for W, fan_in in ((W1, 621), (W2, HIDDEN), (W3, HIDDEN), (W4, HIDDEN)):
            W.copy_(torch.randn(W.shape, generator=g) * math.sqrt(2.0 / fan_in))
        W1[:, _ZERO_COLS] = 0.0
        W4[OUT:] = 0.0
        W4.mul_(0.1)
        self.pop_scale = self.force_scale = self.out_scale = 1.0
        self.step_count = 0
        self.err = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.refresh()

    def refresh(self) -> None:
        """BF16 copies of the weights and the transposes used by the backward pass."""
        W1, b1, W2, b2, W3, b3, W4, b4 = self.views
        bf = torch.bfloat16
        self.w1, self.w2, self.w3, self.w4 = (W.to(bf).contiguous() for W in (W1, W2, W3, W4))
        self.w2t, self.w3t = W2.t().contiguous().to(bf), W3.t().contiguous().to(bf)
        self.w4t = W4.t().contiguous().to(bf)  # [64][32]
        self.bias = torch.cat([b1, b2, b3, b4]).contiguous()

    def weights_struct(self) -> nat.ClosureWeights:
        w = nat.ClosureWeights()
        w.w1, w.w2, w.w3, w.w4 = (t.data_ptr() for t in (self.w1, self.w2, self.w3, self.w4))
        w.bias = self.bias.data_ptr()
        w.pop_scale, w.force_scale, w.out_scale = self.pop_scale, self.force_scale, self.out_scale
        return w

    # -- forward / backward over a batch of feature rows (BF16 [m][656]) ------------
    def forward(self, x: torch.Tensor, keep: bool = False):
        m = x.shape[0]
        dev, bf = self.device, torch.bfloat16
        b1, b2, b3 = self.views[1], self.views[3], self.views[5]
        acts = {}
        h_in = x
        for i, (w, b) in enumerate(((self.w1, b1), (self.w2, b2), (self.w3, b3)), start=1):
            k = w.shape[1]
            h = torch.empty((m, HIDDEN), dtype=bf, device=dev)
            ht = torch.empty((HIDDEN, m), dtype=bf, device=dev) if keep else None
            z = torch.empty((m, HIDDEN), dtype=torch.float32, device=dev) if keep else None
            _gemm(h_in, w, k, k, m, HIDDEN, k, nat.GEMM_GELU_FWD, self.err, bias=b, h=h, ht=ht,
                  ldht=m, zout=z)
            acts[i] = (h, ht, z)
            h_in = h
        y = torch.empty((m, OUT_PAD), dtype=torch.float32, device=dev)
        _gemm(h_in, self.w4, HIDDEN, HIDDEN, m, OUT_PAD, HIDDEN, nat.GEMM_STORE, self.err, c=y,
              ldc=OUT_PAD)
        return (y, acts) if keep else y

    def predict(self, x: torch.Tensor) -> torch.Tensor:
        """Network output (normalised corrections) [m][19], FP32."""
        return self.forward(x)[:, :OUT] + self.views[7][:OUT]

    def backward(self, x: torch.Tensor, y: torch.Tensor, acts: dict, target: torch.Tensor,
                 xt: torch.Tensor | None = None, k_chunk: int = 1024) -> float:
        """Gradients of the mean-square loss into self.grads; returns the loss."""
        m = x.shape[0]
        dev, bf = self.device, torch.bfloat16
        self.grads.zero_()
        loss = torch.zeros(1, dtype=torch.float64, device=dev)
        dy = torch.empty((m, OUT_PAD), dtype=bf, device=dev)
        dyt = torch.empty((OUT_PAD, m), dtype=bf, device=dev)
        nat.call("fsi_closure_loss", nat.ptr(y), nat.ptr(target), nat.ptr(self.views[7]), m,
                 nat.ptr(dy), nat.ptr(dyt), m, nat.ptr(loss), nat.stream_ptr())
        gW1, gb1, gW2, gb2, gW3, gb3, gW4, gb4 = self.gviews
        kc = k_chunk
        # output layer
        h3, h3t, z3 = acts[3]
        _gemm(dyt, h3t, m, m, OUT_PAD, HIDDEN, m, nat.GEMM_ATOMIC, self.err, c=gW4, ldc=HIDDEN,
              k_chunk=kc)
        nat.call("fsi_closure_colsum", nat.ptr(dy), m, OUT_PAD, nat.ptr(gb4), nat.stream_ptr())
        # hidden layers, from the top
        g_in, g_ld, w_t = dy, OUT_PAD, self.w4t
        for layer, (gW, gb) in ((3, (gW3, gb3)), (2, (gW2, gb2)), (1, (gW1, gb1))):
            h, ht, z = acts[layer]
            dz = torch.empty((m, HIDDEN), dtype=bf, device=dev)
            dzt = torch.empty((HIDDEN, m), dtype=bf, device=dev)
            _gemm(g_in, w_t, g_ld, g_ld, m, HIDDEN, g_ld, nat.GEMM_GELU_BWD, self.err, h=dz, ht=dzt,
                  ldht=m, zin=z)
            below_t = xt if layer == 1 else acts[layer - 1][1]
            n_below = FEATURES if layer == 1 else HIDDEN
            _gemm(dzt, below_t, m, m, HIDDEN, n_below, m, nat.GEMM_ATOMIC, self.err, c=gW,
                  ldc=n_below, k_chunk=kc)
            nat.call("fsi_closure_colsum", nat.ptr(dz), m, HIDDEN, nat.ptr(gb), nat.stream_ptr())
            g_in, g_ld = dz, HIDDEN
            w_t = self.w3t if layer == 3 else self.w2t
        gW4[OUT:] = 0.0
        gb4[OUT:] = 0.0
        gW1[:, _ZERO_COLS] = 0.0
        return float(loss.item())

    def adam_step(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999,
                  eps: float = 1e-8) -> None:
        self.step_count += 1
        nat.call("fsi_closure_adam", nat.ptr(self.params), nat.ptr(self.grads), nat.ptr(self.m),
                 nat.ptr(self.v), self.params.numel(), lr, beta1, beta2, eps, self.step_count,
                 nat.stream_ptr())
        self.refresh()

    def check(self) -> None:
        if int(self.err.item()) != 0:
            raise nat.NativeError(f"tensor-core wait timed out (code {int(self.err.item())})")

    def state_dict(self) -> dict:
        return {"params": self.params.cpu(), "scales": (self.pop_scale, self.force_scale,
                                                        self.out_scale),
                "use_fraction": self.use_fraction}

    def load_state_dict(self, state: dict) -> None:
        self.params.copy_(state["params"])
        self.pop_scale, self.force_scale, self.out_scale = state["scales"]
        self.use_fraction = bool(state.get("use_fraction", False))
        self.refresh()


# ------------------------------------------------------------------ data
def _ptr_or_null(t: torch.Tensor | None):
    return None if t is None else nat.ptr(t)


def features(lbm: LBMSolver3D, cells: torch.Tensor, pop_scale: float, force_scale: float,
             frac: torch.Tensor | None = None):
    """BF16 feature rows [m][656] of the given cells (int32 device tensor) of `lbm`; the
    occupancy feature is ``frac`` (solid fraction per cell) when given, else 0/1."""
    m = int(cells.numel())
    x = torch.empty((m, FEATURES), dtype=torch.bfloat16, device=lbm._device)
    nat.call("fsi_closure_features", lbm._desc, nat.ptr(lbm._pops), nat.ptr(lbm.flags),
             nat.ptr(lbm.force), _ptr_or_null(frac), lbm.steps_done, nat.ptr(cells), m, pop_scale,
             force_scale, nat.ptr(x), nat.stream_ptr())
    return x


def training_pairs(fine_cfg: LBMConfig, fine_mask: np.ndarray, warmup: int, snapshots: int,
                   every: int = 2):
    """Run the plain fine solver and collect (coarse post-step state, correction target)
    pairs: for each snapshot, the coarse solver is loaded with the restricted fine state,
    takes one step, and the target is the restricted fine state two fine steps later minus
    the coarse result. Yields (coarse solver after its step, fluid cells, target [m][19])."""
    fine = LBMSolver3D(fine_cfg)
    fine.initialize(fine_mask)
    ccfg = coarse_config(fine_cfg)
    coarse = LBMSolver3D(ccfg)
    cmask = coarse_mask(fine_mask)
    coarse.initialize(cmask)
    fluid = torch.nonzero(torch.from_numpy(cmask.reshape(-1) == 0)).reshape(-1).to(
        torch.int32).to(fine._device)
    for _ in range(warmup):
        fine.step()
    for _ in range(snapshots):
        r0 = restrict(fine, coarse)
        fine.step()
        fine.step()
        r1 = restrict(fine, coarse)
        coarse.load_populations(r0)
        coarse.step()
        cstate = torch.from_numpy(coarse.distribution_numpy().reshape(-1, OUT)).to(fine._device)
        target = (r1 - cstate)[fluid.long()]
        yield coarse, fluid, target
        for _ in range(every - 2):
            fine.step()


def batched_training_pairs(batch, fine_masks: list[np.ndarray], warmup: int, snapshots: int,
                           every: int = 2):
    """``training_pairs`` of every lattice of ``batch`` (an initialised ``LatticeBatch`` of
    the fine scenes, periodic faces, masks ``fine_masks``), the fine runs advancing together
    as one batched launch per step. Yields (lattice index, coarse solver after its step,
    fluid cells, target [m][19]) for each snapshot and lattice; with exact float32
    arithmetic these are the pairs ``training_pairs`` gives scene by scene."""
    dev = batch._device
    coarse, fluid = [], []
    for s, cfg in enumerate(batch.configs):
        c = LBMSolver3D(coarse_config(cfg))
        cmask = coarse_mask(fine_masks[s])
        c.initialize(cmask)
        coarse.append(c)
        fluid.append(torch.nonzero(torch.from_numpy(cmask.reshape(-1) == 0)).reshape(-1).to(
            torch.int32).to(dev))
    # runs of consecutive lattices of one shape and rho0 are restricted in one call
    groups, s = [], 0
    while s < batch.count:
        e = s + 1
        while (e < batch.count and batch.shapes[e] == batch.shapes[s]
               and batch.configs[e].rho0 == batch.configs[s].rho0):
            e += 1
        solid = torch.from_numpy(np.stack([np.asarray(m) > 0 for m in fine_masks[s:e]])).to(dev)
        groups.append((s, e, solid))
        s = e

    def restricted(d):
        out = []
        for a, e, solid in groups:
            rows = d[int(batch.offsets[a]):int(batch.offsets[e])]
            r = restrict_rows(rows, batch.shapes[a], solid, batch.configs[a].rho0)
            out.extend(r.view(e - a, -1, OUT).unbind(0))
        return out

    for _ in range(warmup):
        batch.step()
    for _ in range(snapshots):
        r0s = restricted(batch.distribution())
        batch.step()
        batch.step()
        r1s = restricted(batch.distribution())
        for s in range(batch.count):
            r0, r1 = r0s[s], r1s[s]
            c = coarse[s]
            c.load_populations(r0)
            c.step()
            cstate = torch.from_numpy(c.distribution_numpy().reshape(-1, OUT)).to(dev)
            yield s, c, fluid[s], (r1 - cstate)[fluid[s].long()]
        for _ in range(every - 2):
            batch.step()


def rollout_pairs(fine_cfg: LBMConfig, fine_mask: np.ndarray, net: "ClosureMLP",
                  coarse_steps: int, every: int = 2):
    """Training pairs along the closure's own trajectory (solver in the loop): the coarse run
    with ``net``'s corrections and the plain fine run advance together from rest; every
    ``every`` coarse steps, the coarse state s is stepped once without correction and the
    target is the restricted fine state of the same time minus that step, R(f(t + 2 dt_f)) -
    C(s). One-step pairs from restricted fine states alone teach no recovery from the
    network's own drift, which in rollouts can grow step by step.
    Yields (coarse solver after its uncorrected step, fluid cells, target [m][19])."""
    fine = LBMSolver3D(fine_cfg)
    fine.initialize(fine_mask)
    sim = ClosureSimulation(fine_cfg, fine_mask, net, check_every=0)
    probe = LBMSolver3D(sim.coarse.config)
    cmask = coarse_mask(fine_mask)
    probe.initialize(cmask)
    fluid = torch.nonzero(torch.from_numpy(cmask.reshape(-1) == 0)).reshape(-1).to(
        torch.int32).to(fine._device)
    for k in range(coarse_steps):
        if k % every == 0:
            probe.load_state_dict(sim.coarse.state_dict())
            probe.step()
        fine.step()
        fine.step()
        if k % every == 0:
            r1 = restrict(fine, probe)
            cstate = torch.from_numpy(probe.distribution_numpy().reshape(-1, OUT)).to(fine._device)
            yield probe, fluid, (r1 - cstate)[fluid.long()]
        sim.step()


class ClosureTrainer:
    """Collects training rows from restricted fine runs and fits a ClosureMLP."""

    def __init__(self, net: ClosureMLP):
        self.net = net
        self.rows_x: list[torch.Tensor] = []
        self.rows_t: list[torch.Tensor] = []
        self._pending = []  # (coarse state copy, cells, raw target) before scales are known
        self.batch_records: list[dict] = []  # add_batch: scene count, steps, autotuner record

    def add_run(self, fine_cfg: LBMConfig, fine_mask: np.ndarray, warmup: int = 40,
                snapshots: int = 10, every: int = 4, cell_fraction: float = 1.0,
                seed: int = 0) -> None:
        """Pairs of one restricted fine run; ``cell_fraction`` < 1 keeps a seeded random share
        of each snapshot's fluid cells (bounding the rows of large data sets)."""
        frac = solid_fraction(fine_mask, self.net.device) if self.net.use_fraction else None
        g = torch.Generator(device="cpu").manual_seed(seed)
        for coarse, cells, target in training_pairs(fine_cfg, fine_mask, warmup, snapshots, every):
            if cell_fraction < 1.0:
                keep = torch.rand(cells.numel(), generator=g) < cell_fraction
                keep = keep.to(cells.device)
                cells, target = cells[keep], target[keep]
            self._pending.append((coarse.state_dict(), coarse.config, cells, target.clone(), frac))

    def add_batch(self, fine_cfgs: list[LBMConfig], fine_masks: list[np.ndarray],
                  warmup: int = 40, snapshots: int = 10, every: int = 4,
                  cell_fraction: float = 1.0, seeds: list[int] | None = None,
                  tune: bool = True) -> dict:
        """``add_run`` for many scenes at once: their fine runs advance as one
        ``LatticeBatch``, whose launch the batch autotuner first picks on these scenes
        (``fsi.autotune.tune_lattice_batch``; the state is restored after tuning). Rows are
        kept per scene in the order ``add_run`` would give them, scene ``s`` subsampled with
        ``seeds[s]``. Returns the tuning record, also kept in ``batch_records``."""
        from .batch import LatticeBatch

        n = len(fine_cfgs)
        seeds = list(range(n)) if seeds is None else list(seeds)
        if len(fine_masks) != n or len(seeds) != n:
            raise ValueError("one mask and one seed per scene.")
        batch = LatticeBatch(fine_cfgs)
        batch.initialize(fine_masks)
        record = batch.autotune() if tune else {"best": None, "ms": {}}
        fracs = [solid_fraction(m, self.net.device) if self.net.use_fraction else None
                 for m in fine_masks]
        gens = [torch.Generator(device="cpu").manual_seed(sd) for sd in seeds]
        per_scene = [[] for _ in range(n)]
        for s, coarse, cells, target in batched_training_pairs(batch, fine_masks, warmup,
                                                                snapshots, every):
            if cell_fraction < 1.0:
                keep = (torch.rand(cells.numel(), generator=gens[s]) < cell_fraction)
                keep = keep.to(cells.device)
                cells, target = cells[keep], target[keep]
            per_scene[s].append((coarse.state_dict(), coarse.config, cells, target.clone(),
                                 fracs[s]))
        for pending in per_scene:
            self._pending.extend(pending)
        del batch
        rec = {"scenes": n, "fine_steps": warmup + snapshots * max(every, 2),
               "tuning": record}
        self.batch_records.append(rec)
        return rec

    def add_rollout_run(self, fine_cfg: LBMConfig, fine_mask: np.ndarray, coarse_steps: int,
                        every: int = 2, cell_fraction: float = 1.0, seed: int = 0) -> None:
        """Pairs along the current network's own closure trajectory (``rollout_pairs``), built
        with the scales already fitted; call after a first ``build`` / ``fit``."""
        frac = solid_fraction(fine_mask, self.net.device) if self.net.use_fraction else None
        g = torch.Generator(device="cpu").manual_seed(seed)
        for probe, cells, target in rollout_pairs(fine_cfg, fine_mask, self.net, coarse_steps,
                                                   every):
            if cell_fraction < 1.0:
                keep = (torch.rand(cells.numel(), generator=g) < cell_fraction).to(cells.device)
                cells, target = cells[keep], target[keep]
            self.rows_x.append(features(probe, cells, self.net.pop_scale, self.net.force_scale,
                                        frac))
            self.rows_t.append((target * self.net.out_scale).float())

    def merge(self) -> int:
        """Append the rows of add_rollout_run to the data set; returns the row count."""
        if self.rows_x:
            self.x = torch.cat([self.x, *self.rows_x])
            self.t = torch.cat([self.t, *self.rows_t]).contiguous()
            self.rows_x.clear()
            self.rows_t.clear()
        return int(self.x.shape[0])

    def _fit_scales(self) -> None:
        devs, forces, targets = [], [], []
        for state, cfg, cells, target, _ in self._pending:
            f = state["pops"]
            w = torch.tensor([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, device=f.device).view(OUT, 1)
            devs.append((f - w * cfg.rho0)[:, cells.long()].flatten())
            forces.append(torch.tensor(cfg.force).abs().max())
            targets.append(target.flatten())
        self.net.pop_scale = float(1.0 / max(torch.cat(devs).std().item(), 1e-12))
        self.net.force_scale = float(1.0 / max(max(float(f) for f in forces), 1e-12))
        self.net.out_scale = float(1.0 / max(torch.cat(targets).std().item(), 1e-20))

    def build(self) -> int:
        """Feature rows of every collected pair with the fitted scales; returns the row count."""
        self._fit_scales()
        for state, cfg, cells, target, frac in self._pending:
            lbm = LBMSolver3D(cfg)
            lbm.load_state_dict(state)
            self.rows_x.append(features(lbm, cells, self.net.pop_scale, self.net.force_scale, frac))
            self.rows_t.append((target * self.net.out_scale).float())
        self._pending.clear()
        self.x = torch.cat(self.rows_x)
        self.t = torch.cat(self.rows_t).contiguous()
        self.rows_x.clear()
        self.rows_t.clear()
        return int(self.x.shape[0])

    def fit(self, steps: int = 500, batch: int = 16384, lr: float = 2e-3, seed: int = 0,
            halvings: float = 3.0) -> list[float]:
        """Adam on random mini-batches (multiples of 128 rows), the learning rate halving
        ``halvings`` times over the run; returns the loss history."""
        g = torch.Generator(device="cpu").manual_seed(seed)
        n = self.x.shape[0]
        batch = max(128, min(batch, n) // 128 * 128)
        hist = []
        for it in range(steps):
            idx = torch.randint(0, n, (batch,), generator=g).to(self.x.device)
            x = self.x[idx].contiguous()
            xt = x.t().contiguous()
            t = self.t[idx].contiguous()
            y, acts = self.net.forward(x, keep=True)
            hist.append(self.net.backward(x, y, acts, t, xt=xt))
            self.net.adam_step(lr=lr * (0.5 ** (it / max(steps, 1) * halvings)))
        self.net.check()
        return hist


# ------------------------------------------------------------ simulation
def rows_buffer(lbm: LBMSolver3D) -> torch.Tensor:
    """Scratch for the feature rows the fused inference stages (``fsi_closure_rows_bytes``)."""
    nbytes = int(nat.load().fsi_closure_rows_bytes(lbm._desc))
    if nbytes <= 0:
        raise ValueError(f"lattice unsupported by the closure: {nat.last_error()}")
    return torch.empty(nbytes, dtype=torch.uint8, device=lbm._device)


def infer(lbm: LBMSolver3D, weights: nat.ClosureWeights, corr: torch.Tensor, rows: torch.Tensor,
          err: torch.Tensor, frac: torch.Tensor | None = None) -> None:
    """Corrections corr [19][N] of every cell of ``lbm`` by the fused tensor-core inference."""
    nat.call("fsi_closure_infer", lbm._desc, nat.ptr(lbm._pops), nat.ptr(lbm.flags), nat.ptr(lbm.force),
             _ptr_or_null(frac), lbm.steps_done, ctypes.byref(weights), nat.ptr(rows), nat.ptr(corr),
             nat.ptr(err), nat.stream_ptr())


def infer_apply(lbm: LBMSolver3D, weights: nat.ClosureWeights, rows: torch.Tensor,
                err: torch.Tensor, frac: torch.Tensor | None = None) -> None:
    """The fused inference with each cell's mass-conserving correction added to its populations
    in place (``infer`` then ``fsi_closure_apply``, in one pass)."""
    nat.call("fsi_closure_infer_apply", lbm._desc, nat.ptr(lbm._pops), nat.ptr(lbm.flags),
             nat.ptr(lbm.force), _ptr_or_null(frac), lbm.steps_done, ctypes.byref(weights), nat.ptr(rows),
             nat.ptr(err), nat.stream_ptr())
    lbm._mass_speed_cache = None


class ClosureSimulation:
    """The coarse lattice with the learned correction after every step; guards on mass drift
    and local Mach number fall back to the plain fine-grid solver."""

    def __init__(self, fine_cfg: LBMConfig, fine_mask: np.ndarray, net: ClosureMLP,
                 mass_tol: float = 1e-3, mach_tol: float = 0.3, check_every: int = 10):
        self.fine_cfg = fine_cfg
        self.fine_mask = np.asarray(fine_mask)
        self.net = net
        self.coarse = LBMSolver3D(coarse_config(fine_cfg))
        self.coarse.initialize(coarse_mask(fine_mask))
        self.mass_tol, self.mach_tol, self.check_every = mass_tol, mach_tol, check_every
        self.mass0 = self.coarse.total_mass()
        self.fine: LBMSolver3D | None = None
        self.fallback_step: int | None = None
        self.fallback_reason = ""
        self.coarse_steps = 0
        self._weights = net.weights_struct()
        self._rows = rows_buffer(self.coarse)
        self._frac = solid_fraction(fine_mask, self.coarse._device) if net.use_fraction else None

    @property
    def on_fine_grid(self) -> bool:
        return self.fine is not None

    def _guard(self) -> str:
        mass = self.coarse.total_mass()
        if abs(mass - self.mass0) > self.mass_tol * abs(self.mass0):
            return f"mass drift {abs(mass - self.mass0) / abs(self.mass0):.2e}"
        mach = self.coarse.max_velocity_norm() / _CS
        if not math.isfinite(mach) or mach > self.mach_tol:
            return f"local Mach {mach:.3f}"
        return ""

    def _fall_back(self, reason: str) -> None:
        f = torch.from_numpy(self.coarse.distribution_numpy().reshape(-1, OUT)).to(self.coarse._device)
        self.fine = LBMSolver3D(self.fine_cfg)
        self.fine.initialize(self.fine_mask)
        self.fine.load_populations(prolongate(f, (self.fine_cfg.nx, self.fine_cfg.ny, self.fine_cfg.nz)))
        self.fallback_step = self.coarse_steps
        self.fallback_reason = reason

    def step(self, drag_mask: np.ndarray | None = None) -> np.ndarray | None:
        """One coarse step (= two fine steps of time), or two fine steps after a fallback.
        With ``drag_mask`` (the fine-grid body mask) returns the momentum-exchange force on
        those bodies in fine-lattice units: on the coarse grid it is taken after the coarse
        step and before the learned correction (the populations the bounce-back links
        produced; the correction is a volume term and no link exchange), times 4 for the
        coarse lattice's units under acoustic scaling."""
        if self.fine is not None:
            self.fine.step()
            self.fine.step()
            return None if drag_mask is None else momentum_exchange(self.fine, drag_mask)
        c = self.coarse
        c.step()
        if drag_mask is None:
            drag = None
            infer_apply(c, self._weights, self._rows, self.net.err, self._frac)
        else:
            cbody = coarse_mask(drag_mask)
            drag = 4.0 * momentum_exchange(c, cbody)
            # The correction is the closure's sub-grid force: the momentum it removes from the
            # cells next to the bodies (those with a body cell in their 3^3 neighbourhood) is
            # drag on the bodies that no bounce-back link carries.
            corr = torch.zeros((OUT, c.n_cells), dtype=torch.float32, device=c._device)
            infer(c, self._weights, corr, self._rows, self.net.err, self._frac)
            near = torch.from_numpy(_near(cbody).reshape(-1)).to(c._device)
            e = torch.tensor(np.stack([_EX, _EY, _EZ]), dtype=torch.float64, device=c._device)
            q = (e @ corr[:, near].double()).sum(dim=1).cpu().numpy()
            self.last_correction_momentum = 4.0 * q
            drag = drag - 4.0 * q
            nat.call("fsi_closure_apply", c._desc, nat.ptr(c._pops), nat.ptr(c.flags),
                     c.steps_done, nat.ptr(corr), nat.stream_ptr())
            c._mass_speed_cache = None
        self.coarse_steps += 1
        if self.check_every and self.coarse_steps % self.check_every == 0:
            reason = self._guard()
            if reason:
                self._fall_back(reason)
        return drag

    def velocity_numpy(self) -> np.ndarray:
        """Velocity on the coarse grid (restricting the fine field after a fallback)."""
        if self.fine is None:
            return self.coarse.velocity_numpy()
        u = self.fine.velocity_numpy()
        nx, ny, nz = (n // 2 for n in u.shape[:3])
        return u.reshape(nx, 2, ny, 2, nz, 2, 3).mean(axis=(1, 3, 5))


def evaluate(fine_cfg: LBMConfig, fine_mask: np.ndarray, net: ClosureMLP, coarse_steps: int,
             flow_axis: int = 0, body_mask: np.ndarray | None = None,
             check_every: int = 10) -> dict:
    """Error of the coarse runs against the restricted plain fine run after ``coarse_steps``
    coarse steps (2 * coarse_steps fine steps): rel-L2 velocity of the plain coarse run and
    of the closure run, the relative error of the mean flow along ``flow_axis`` (the
    channel's flow rate), and with ``body_mask`` the relative error of the drag on the bodies
    along ``flow_axis``: momentum exchange on each run's own body mask (a coarse lattice force
    is 4x the fine-lattice force of the same physical force under acoustic scaling), for the
    closure run taken before its last correction and less the momentum that correction adds
    next to the bodies (ClosureSimulation.step). The closure run keeps its guards
    (``check_every``); ``fallback`` names the tripped guard."""
    fine = LBMSolver3D(fine_cfg)
    fine.initialize(fine_mask)
    ccfg = coarse_config(fine_cfg)
    cmask = coarse_mask(fine_mask)
    plain = LBMSolver3D(ccfg)
    plain.initialize(cmask)
    sim = ClosureSimulation(fine_cfg, fine_mask, net, check_every=check_every)
    d_sim = None
    for k in range(coarse_steps):
        fine.step()
        fine.step()
        plain.step()
        d_sim = sim.step(body_mask if k == coarse_steps - 1 else None)
    drag = {}
    if body_mask is not None:
        d_ref = momentum_exchange(fine, body_mask)[flow_axis]
        d_plain = 4.0 * momentum_exchange(plain, coarse_mask(body_mask))[flow_axis]
        d_cl = float(d_sim[flow_axis])
        q = 0.0 if sim.fine is not None else float(sim.last_correction_momentum[flow_axis])
        drag = {"drag_fine": d_ref, "drag_plain": d_plain, "drag_closure": d_cl,
                "drag_closure_links_only": d_cl + q,
                "drag_error_plain": abs(d_plain - d_ref) / abs(d_ref),
                "drag_error_closure": abs(d_cl - d_ref) / abs(d_ref)}
    ref = LBMSolver3D(ccfg)
    ref.initialize(cmask)
    ref.load_populations(restrict(fine, plain))
    u_ref, u_plain, u_cl = ref.velocity_numpy(), plain.velocity_numpy(), sim.velocity_numpy()
    fluid = cmask == 0

    def l2(u):
        return float(np.linalg.norm((u - u_ref)[fluid]) / max(np.linalg.norm(u_ref[fluid]), 1e-30))

    def flow(u):
        return float(u[..., flow_axis][fluid].mean())

    q_ref = flow(u_ref)
    return {"coarse_steps": coarse_steps, "velocity_l2_plain": l2(u_plain),
            "velocity_l2_closure": l2(u_cl),
            "flow_rate_error_plain": abs(flow(u_plain) - q_ref) / abs(q_ref),
            "flow_rate_error_closure": abs(flow(u_cl) - q_ref) / abs(q_ref),
            "fallback": sim.fallback_reason or None, **drag}
