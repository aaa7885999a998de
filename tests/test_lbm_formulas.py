"""The generated MRT register formulas equal the literal float32 19x19 sums of the reference."""
from __future__ import annotations

import importlib.util
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GEN = ROOT / "taichi-mpm-lbm_gb300" / "csrc" / "gen_lbm_formulas.py"


def load_gen():
    spec = importlib.util.spec_from_file_location("gen_lbm_formulas", GEN)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_generated_header_is_current():
    gen = load_gen()
    assert (GEN.parent / "lbm_formulas.cuh").read_text() == gen.gen()


def test_planned_inverse_is_bit_exact():
    load_gen().self_check(n=50_000, seed=7)


def test_tables_match_the_oracle():
    gen = load_gen()
    from oracle import oracle as O
    M, invM, S, w = O.lattice_tables(0.1)
    assert np.array_equal(gen.M, M) and np.array_equal(gen.INV, invM)
    # The device constants for the weights are float32(1/3), float32(1/18), float32(1/36).
    assert float(w[0]).hex() == "0x1.5555560000000p-2"
    assert float(w[1]).hex() == "0x1.c71c720000000p-5"
    assert float(w[7]).hex() == "0x1.c71c720000000p-6"


def _split_top(text: str) -> list[str]:
    """Split at commas outside parentheses/brackets."""
    parts, depth, cur = [], 0, ""
    for ch in text:
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def _fast_as_python(src: str) -> str:
    """Body of the generated mrt_collide_fast as Python statements."""
    import re
    body = src.split("mrt_collide_fast(", 1)[1].split("{", 1)[1]
    body = body[: body.index("\n}\n")]
    body = re.sub(r"(-?0x[0-9a-f.]+p[+-]\d+)f", lambda m: repr(float.fromhex(m.group(1))), body)
    body = re.sub(r"\b(\d+\.\d+)f\b", r"\1", body)
    stmts = []
    for line in body.strip().splitlines():
        line = line.strip()
        if line.startswith("{"):
            line = line.strip("{} ")
        for stmt in filter(None, (s.strip() for s in line.split(";"))):
            stmt = re.sub(r"^(const )?V ", "", stmt)
            stmts.extend(_split_top(stmt))
    return "\n".join(stmts).replace("splat<V>(0.0)", "0.0")


def _collide_f64(gen, F, u, G, S):
    """MRT + Guo collision of the reference written from its definition, in float64."""
    E = np.array(gen.E, float)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    M = gen.M.astype(np.float64)
    eu, eG = u @ E.T, G @ E.T
    t = w * (eG - (u * G).sum(1)[:, None] + eu * eG)
    m, g = F @ M.T, t @ M.T
    ux, uy, uz = u.T
    meq = np.zeros_like(m)
    meq[:, 1] = ux * ux + uy * uy + uz * uz
    meq[:, 9] = 2 * ux * ux - uy * uy - uz * uz
    meq[:, 11] = uy * uy - uz * uz
    meq[:, 13], meq[:, 14], meq[:, 15] = ux * uy, uy * uz, ux * uz
    post = m - S * (m - meq) + (1 - 0.5 * S) * g
    for k in (0, 3, 5, 7):
        post[:, k] = m[:, k] + g[:, k]
    return post @ np.linalg.inv(M).T


def test_fast_collision_is_the_same_operator():
    gen = load_gen()
    code = _fast_as_python(gen.gen())
    rng = np.random.default_rng(3)
    n = 4000
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    F = w * rng.uniform(0.9, 1.1, (n, 1)) * (1 + rng.normal(0, 0.02, (n, 19)))
    u = rng.normal(0, 0.05, (n, 3))
    G = rng.normal(0, 1e-4, (n, 3))
    S = np.array([0, 1.2, 1.3, 0, 1.1, 0, 1.1, 0, 1.1, 1.6, 1.6, 1.6, 1.6, 1.6, 1.6, 1.6, 1.4,
                  1.4, 1.4])
    out = [None] * 19
    env = {"F": F.T, "rho": F.sum(1), "ux": u[:, 0], "uy": u[:, 1], "uz": u[:, 2],
           "gx": G[:, 0], "gy": G[:, 1], "gz": G[:, 2], "S": S, "out": out,
           "vfma": lambda a, b, c: a * b + c, "fmaf": lambda a, b, c: a * b + c,
           "vadd": lambda a, b: a + b, "vsub": lambda a, b: a - b, "vmul": lambda a, b: a * b,
           "vneg": lambda a: -a}
    exec(code, env)
    want = _collide_f64(gen, F, u, G, S)
    got = np.stack(out, axis=1)
    # The generated coefficients are float32 roundings of 1/3, 1/18, ... (relative 3e-8); an
    # algebra mistake in a moment or forcing term shows up at 1e-5 and above.
    np.testing.assert_allclose(got, want, rtol=1e-7, atol=0)


def _exact_as_python(src: str, name: str) -> str:
    """Body of the generated exact transform `name` as Python statements (arrays as lists)."""
    import re
    body = src.split(f"void {name}(", 1)[1].split("{", 1)[1]
    body = body[: body.index("\n}\n")]
    body = re.sub(r"(-?0x[0-9a-f.]+p[+-]\d+)f", lambda m: repr(float.fromhex(m.group(1))), body)
    stmts = []
    for stmt in filter(None, (s.strip() for s in body.replace("\n", " ").split(";"))):
        if re.fullmatch(r"V \w+\[\d+\]", stmt):
            continue  # array declaration
        stmts.append(re.sub(r"^(const )?V ", "", stmt))
    return "\n".join(stmts)


def _f32_env(**arrays):
    f32 = np.float32
    return {"vadd": lambda a, b: (a + b).astype(f32), "vsub": lambda a, b: (a - b).astype(f32),
            "vmul": lambda a, b: (a * f32(b) if isinstance(b, float) else a * b).astype(f32),
            "vneg": lambda a: -a, **arrays}


def test_generated_exact_transforms_run_bit_exact():
    """The emitted text of mrt_forward / mrt_inverse (shared and negated prefixes included),
    run statement by statement in float32, equals the literal sequential sums bit for bit."""
    gen = load_gen()
    src = gen.gen()
    rng = np.random.default_rng(11)
    n = 20_000
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, np.float32)
    F = (w * rng.uniform(0.8, 1.2, (n, 1)) * (1 + rng.normal(0, 0.05, (n, 19)))).astype(np.float32)

    def forward(x):
        env = _f32_env(X=list(x.T), m=[None] * 19, two=[None] * 19)
        exec(_exact_as_python(src, "mrt_forward"), env)
        return np.stack(env["m"], axis=1)

    mom = gen._seq_dense(gen.M, F)
    assert np.array_equal(forward(F).view(np.uint32), mom.view(np.uint32))
    # Guo-like source terms with exact zeros of both signs: equal as values (the sign of an
    # exact zero may differ, which the collision cannot carry to an output).
    t = (rng.normal(0, 1e-6, (n, 19)) * (rng.uniform(size=(n, 19)) < 0.7)).astype(np.float32)
    t[rng.uniform(size=(n, 19)) < 0.2] *= np.float32(-1.0)
    assert np.array_equal(forward(t), gen._seq_dense(gen.M, t))

    mom[:, 3:8] += rng.normal(0, 1e-4, (n, 5)).astype(np.float32)
    env = _f32_env(m=list(mom.T), f=[None] * 19)
    exec(_exact_as_python(src, "mrt_inverse"), env)
    got = np.stack(env["f"], axis=1)
    assert np.array_equal(got.view(np.uint32), gen._seq_dense(gen.INV, mom).view(np.uint32))


def _kernel_exact_collision(gen, src, F, G_prev, G, S):
    """numpy float32 restatement of the step kernel's exact form for rows of F (cells x 19):
    rho and u from rows 0, 3, 5, 7 of the emitted M F (macro_of_moments), then collide_cell
    (Guo terms with (e.u)(e.G) shared by q and opp(q), forcing weights 1 - S/2 rounded once,
    relaxation, emitted inverse), as csrc/lbm_core.cuh writes them."""
    f32 = np.float32

    def run(name, **arrays):
        env = _f32_env(**arrays)
        exec(_exact_as_python(src, name), env)
        return env

    mF = run("mrt_forward", X=list(F.T), m=[None] * 19, two=[None] * 19)["m"]
    r = mF[0]
    u = [mF[k] / r + (G_prev[:, a] * f32(0.5)) / r for a, k in enumerate((3, 5, 7))]
    g3 = [G[:, a] for a in range(3)]
    d = [[(f32(-1.0) - u[a]) * g3[a], (-u[a]) * g3[a], (f32(1.0) - u[a]) * g3[a]]
         for a in range(3)]
    E = gen.E
    w = [f32(1 / 3)] + [f32(1 / 18)] * 6 + [f32(1 / 36)] * 12

    def edot(q, v):
        s = None
        for a in range(3):
            if E[q][a] != 0:
                term = v[a] if E[q][a] > 0 else -v[a]
                s = term if s is None else s + term
        return s

    t, b = [None] * 19, [None] * 19
    for q in range(19):
        a = (d[0][E[q][0] + 1] + d[1][E[q][1] + 1]) + d[2][E[q][2] + 1]
        if q == 0:
            t[q] = w[q] * a
        else:
            b[q] = edot(q, u) * edot(q, g3) if q % 2 else b[q - 1]
            t[q] = w[q] * (a + b[q])
    g = run("mrt_forward", X=t, m=[None] * 19, two=[None] * 19)["m"]
    ux, uy, uz = u
    uxx, uyy, uzz = ux * ux, uy * uy, uz * uz
    meq = {1: (uxx + uyy) + uzz, 9: ((f32(2.0) * ux) * ux - uyy) - uzz, 11: uyy - uzz,
           13: ux * uy, 14: uy * uz, 15: ux * uz}
    SG = f32(1.0) - f32(0.5) * S
    m = list(mF)
    for k in range(19):
        if k in (0, 3, 5, 7):
            m[k] = m[k] + g[k]
        else:
            dk = m[k] - meq[k] if k in meq else m[k]
            m[k] = m[k] - S[k] * dk
            m[k] = m[k] + SG[k] * g[k]
    f = run("mrt_inverse", m=m, f=[None] * 19)["f"]
    return r, np.stack(u, axis=1), np.stack(f, axis=1)


def _stream_periodic(gen, f_post, solid):
    """The reference's stream (periodic wrap, half-way bounce-back at solid targets) of
    post-collision populations (nx, ny, nz, 19); entries of solid cells stay zero."""
    sol = solid.astype(bool)
    out = np.zeros_like(f_post)
    axes = (0, 1, 2)
    for q in range(19):
        e = tuple(gen.E[q])
        moved = np.roll(f_post[..., q], e, axis=axes)          # moved[y] = f*(y - e)
        from_fluid = (~sol) & np.roll(~sol, e, axis=axes)     # y fluid, y - e fluid
        out[..., q] = np.where(from_fluid, moved, out[..., q])
        bounce = (~sol) & np.roll(sol, tuple(-x for x in e), axis=axes)  # x fluid, x + e solid
        o = gen.OPP[q]
        out[..., o] = np.where(bounce, f_post[..., q], out[..., o])
    return out


@pytest.mark.parametrize("case", ["rest_unforced", "forced_uniform", "forced_with_solids",
                                  "moving_with_solids"])
def test_exact_collision_restatement_matches_the_oracle_bit_for_bit(case):
    """The kernel's exact-form arithmetic (shared Guo products, rho and j from M F, host-rounded
    forcing weights) restated in numpy float32 and streamed gives the oracle's next state and
    its rho, u bit for bit, exact zeros of the unforced rest state included."""
    from helpers import periodic_lbm
    from oracle import oracle as O

    gen = load_gen()
    src = gen.gen()
    force = (0.0, 0.0, 0.0) if case == "rest_unforced" else (2e-5, -1e-5, 5e-6)
    u0 = (0.02, -0.01, 0.005) if case in ("forced_uniform", "moving_with_solids") else (0, 0, 0)
    shape = (6, 5, 7)
    cfg = periodic_lbm(nx=shape[0], ny=shape[1], nz=shape[2], viscosity=0.05, force=force,
                       initial_velocity=u0)
    lbm = O.LBMSolver3D(cfg)
    solid = np.zeros(shape, np.int32)
    if case.endswith("with_solids"):
        solid[2, 1:3, 2:5] = 1
        solid[4, 3, 1] = 1
    lbm.initialize(solid)
    for _ in range(4):
        lbm.step()
    fluid = solid.reshape(-1) == 0
    F = lbm.F.reshape(-1, 19)[fluid].copy()
    G = lbm.force.reshape(-1, 3)[fluid].copy()
    rho_want = lbm.rho.reshape(-1)[fluid].copy()
    u_want = lbm.v.reshape(-1, 3)[fluid].copy()
    lbm.step()
    rho, u, f = _kernel_exact_collision(gen, src, F, G, G, lbm.S)
    assert np.array_equal(rho.view(np.uint32), rho_want.view(np.uint32))
    assert np.array_equal(u.view(np.uint32), u_want.view(np.uint32))
    f_post = np.zeros((*shape, 19), np.float32)
    f_post.reshape(-1, 19)[fluid] = f
    got = _stream_periodic(gen, f_post, solid).reshape(-1, 19)[fluid]
    want = lbm.F.reshape(-1, 19)[fluid]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
