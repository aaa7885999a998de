"""Generate ``lbm_formulas.cuh``: the D3Q19 MRT collision as straight-line register code.

The reference collides each fluid cell with two dense 19x19 products
(fsi/lbm3d.py:314-333): ``m = M F`` with sequential float32 sums over q, the
relaxation and Guo forcing in moment space, then ``f = inv(M) m`` with
sequential sums over the 19 moments. This script emits the same arithmetic as
explicit formulas, operation for operation, so the device result is
bit-identical to a literal evaluation of those sums in IEEE float32:

* ``M`` has entries in {0, +-1, +-2}; products with it are exact, so each moment
  is a chain of additions/subtractions of F_q or 2 F_q, in q order, with the
  zero terms dropped (adding an exact zero never changes a float sum).
* ``inv(M)`` is what ``np.linalg.inv`` returns for the float32 ``M`` (as in
  lbm3d.py:170). Its entries below 1e-10 are rounding residue of the exact
  zeros; a product with them is far below half an ulp of the running sum (the
  first term, inv(M)[q,0] * rho, is always >= rho/36), so they are dropped.
  Within a column the remaining magnitudes differ by powers of two, so one
  rounded product per (column, magnitude class) is reused with exact scaling.

Every claim above is checked numerically by ``self_check()`` (and by the test
suite) against a literal sequential float32 evaluation with the full tables.

The functions are templates over the value type V: ``float`` for one cell, or
``float2`` for two cells at once through the packed FP32 instructions of sm_100+
(``vadd``/``vsub``/``vmul``/``vfma`` of lbm_vec.cuh), whose per-lane results are
those of the scalar round-to-nearest operations, so both are bit-identical.

Run: python gen_lbm_formulas.py  (rewrites lbm_formulas.cuh next to this file)
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "lbm_formulas.cuh"
Q = 19
E = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
     (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0), (1, 0, 1), (-1, 0, -1), (1, 0, -1),
     (-1, 0, 1), (0, 1, 1), (0, -1, -1), (0, 1, -1), (0, -1, 1)]
OPP = [0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17]
NOISE = 1e-10


def mrt_matrix() -> np.ndarray:
    rows = [
        [1] * 19,
        [-1, 0, 0, 0, 0, 0, 0] + [1] * 12,
        [1, -2, -2, -2, -2, -2, -2] + [1] * 12,
        [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
        [0, -2, 2, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0],
        [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1],
        [0, 0, 0, -2, 2, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1],
        [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1],
        [0, 0, 0, 0, 0, -2, 2, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1],
        [0, 2, 2, -1, -1, -1, -1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
        [0, -2, -2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -2, -2, -2, -2],
        [0, 0, 0, 1, 1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
        [0, 0, 0, -1, -1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, 1, -1, 1, -1, -1, 1, -1, 1, 0, 0, 0, 0],
        [0, 0, 0, 0, 0, 0, 0, -1, 1, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1],
        [0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, -1, -1, 1, -1, 1, 1, -1],
    ]
    return np.array(rows, dtype=np.float32)


M = mrt_matrix()
INV = np.linalg.inv(M).astype(np.float32)


def forward_plan():
    """Rows of M as signed terms [(q, coefficient)] in q order (zeros dropped), and for each
    row b the earlier row a whose first L >= 2 terms are exactly the negatives of b's first L
    terms: {b: (a, L)}, longest L kept. Round-to-nearest is symmetric, so the partial sum of
    b after L terms is minus that of a (up to the sign of an exact zero) and b's chain can
    continue from it: (-p) + X = X - p exactly."""
    rows = [[(q, int(M[k, q])) for q in range(Q) if M[k, q] != 0] for k in range(Q)]
    reuse = {}
    for b in range(Q):
        best = None
        for a in range(b):
            n = 0
            while (n < min(len(rows[a]), len(rows[b])) and rows[a][n][0] == rows[b][n][0]
                   and rows[a][n][1] == -rows[b][n][1]):
                n += 1
            if n >= 2 and (best is None or n > best[1]):
                best = (a, n)
        if best is not None:
            reuse[b] = best
    for b, (a, n) in reuse.items():
        # the prefix of a must be one that a's own chain computes
        assert a not in reuse or reuse[a][1] <= n
    return rows, reuse


def inverse_plan():
    """Per column k: list of (class_id, base_magnitude); per entry (q,k): (sign, class, shift)."""
    classes = []        # (k, base) per product register
    entry = {}          # (q, k) -> (sign, class_index, power_of_two)
    for k in range(Q):
        bases: list[float] = []
        for q in range(Q):
            v = float(INV[q, k])
            if abs(v) < NOISE:
                continue
            mag = np.float32(abs(v))
            found = None
            for ci, b in enumerate(bases):
                ratio = float(mag) / b
                j = round(math.log2(ratio))
                if np.float32(math.ldexp(b, j)) == mag:
                    found = (ci, j)
                    break
            if found is None:
                bases.append(float(mag))
                found = (len(bases) - 1, 0)
            entry[(q, k)] = (1 if v > 0 else -1, (k, found[0]), found[1])
        for ci, b in enumerate(bases):
            classes.append(((k, ci), b))
    return classes, entry


def f32hex(x: float) -> str:
    return float(np.float32(x)).hex() + "f"


def _term(sign: int, expr: str, first: bool) -> str:
    if first:
        return expr if sign > 0 else f"-({expr})"
    return expr


def chain(var: str, terms: list[tuple[int, str]]) -> list[str]:
    """Sequential float sum of signed terms, in order, with explicit rounding per step."""
    lines = []
    if not terms:
        lines.append(f"{var} = splat<V>(0.0f);")
        return lines
    s0, e0 = terms[0]
    lines.append(f"{var} = {e0 if s0 > 0 else 'vneg(' + e0 + ')'};")
    for s, e in terms[1:]:
        op = "vadd" if s > 0 else "vsub"
        lines.append(f"{var} = {op}({var}, {e});")
    return lines


def gen() -> str:
    out = []
    w = out.append
    w("// GENERATED by gen_lbm_formulas.py -- do not edit by hand.")
    w("// D3Q19 MRT collision of the reference (fsi/lbm3d.py:269-333) as explicit")
    w("// register formulas with the reference's float32 operation order.")
    w("#pragma once")
    w("")
    w('#include "lbm_vec.cuh"')
    w("")
    w("namespace fsi {")
    w("")
    # forward transform on an input array X (F or Guo terms t)
    w("// m[k] = sum_q M[k][q] * X[q], sequential in q (lbm3d.py:269-274).")
    w("template <class V>")
    w("__device__ __forceinline__ void mrt_forward(const V (&X)[19], V (&m)[19]) {")
    w("  V two[19];")
    need_two = sorted({q for k in range(Q) for q in range(Q) if abs(M[k, q]) == 2})
    for q in need_two:
        w(f"  two[{q}] = vadd(X[{q}], X[{q}]);")
    rows, reuse = forward_plan()
    keep = {}  # row a -> prefix lengths that later rows continue from
    for a, n in reuse.values():
        keep.setdefault(a, set()).add(n)
    for k in range(Q):
        terms = [(1 if c > 0 else -1, f"X[{q}]" if abs(c) == 1 else f"two[{q}]")
                 for q, c in rows[k]]
        var = f"m[{k}]"
        if k in reuse:
            a, n = reuse[k]
            pre = f"pre{a}_{n}"
            if len(terms) == n:
                body = [f"{var} = vneg({pre});"]
            else:
                s, e = terms[n]
                body = [f"{var} = vsub({e}, {pre});" if s > 0
                        else f"{var} = vneg(vadd({pre}, {e}));"]
                for s, e in terms[n + 1:]:
                    body.append(f"{var} = {'vadd' if s > 0 else 'vsub'}({var}, {e});")
        else:
            body = chain(var, terms)
            for n in sorted(keep.get(k, ()), reverse=True):
                body.insert(n, f"const V pre{k}_{n} = {var};")
        w("  " + " ".join(body))
    w("}")
    w("")
    classes, entry = inverse_plan()
    w("// f[q] = sum_k inv(M)[q][k] * m[k], sequential in k (lbm3d.py:328-333).")
    w(f"// {len(classes)} rounded products; every other product is an exact power-of-two scaling.")
    w("template <class V>")
    w("__device__ __forceinline__ void mrt_inverse(const V (&m)[19], V (&f)[19]) {")
    names = {}
    for (k, ci), b in classes:
        nm = f"p{k}_{ci}"
        names[(k, ci)] = nm
        w(f"  const V {nm} = vmul(m[{k}], {f32hex(b)});")
    # Each scaled product once; rows that begin with the same terms (same products, signs and
    # order) continue from one named partial sum, which is the same value in both rows.
    rows = []
    scaled = {}
    for q in range(Q):
        terms = []
        for k in range(Q):
            if (q, k) not in entry:
                continue
            sign, cls, j = entry[(q, k)]
            base = names[cls]
            if j == 0:
                expr = base
            else:
                if (base, j) not in scaled:
                    scaled[(base, j)] = f"{base}_s{len(scaled)}"
                    w(f"  const V {scaled[(base, j)]} = vmul({base}, {f32hex(2.0 ** j)});")
                expr = scaled[(base, j)]
            terms.append((sign, expr))
        rows.append(terms)
    shared = {}  # prefix (tuple of terms, length >= 2) -> name, for prefixes a later row reuses
    for b in range(Q):
        for a in range(b):
            n = 0
            while n < min(len(rows[a]), len(rows[b])) and rows[a][n] == rows[b][n]:
                n += 1
            if n >= 2:
                shared.setdefault(tuple(rows[b][:n]), None)
    defined = set()
    for q, terms in enumerate(rows):
        var = f"f[{q}]"
        start = 0
        for n in range(len(terms), 1, -1):
            if tuple(terms[:n]) in defined:
                start = n
                break
        if start:
            body = [f"{var} = {shared[tuple(terms[:start])]};"]
        else:
            s0, e0 = terms[0]
            body = [f"{var} = {e0 if s0 > 0 else 'vneg(' + e0 + ')'};"]
            start = 1
        for i in range(start, len(terms)):
            s, e = terms[i]
            body.append(f"{var} = {'vadd' if s > 0 else 'vsub'}({var}, {e});")
            key = tuple(terms[:i + 1])
            if key in shared and key not in defined:
                shared[key] = f"r{len(defined)}"
                defined.add(key)
                body.append(f"const V {shared[key]} = {var};")
        w("  " + " ".join(body))
    w("}")
    w("")
    out.extend(gen_fast().splitlines())
    w("}  // namespace fsi")
    return "\n".join(out) + "\n"


# ------------------------------------------------- reduced-operation collision --

def _fmt(c: float) -> str:
    return float(np.float32(c)).hex() + "f"


def _lin(terms: list[tuple[float, str]]) -> str:
    """Sum of coefficient * symbol with fused multiply-adds (coefficients +-1 become adds)."""
    terms = [(c, s) for c, s in terms if c != 0.0]
    if not terms:
        return "splat<V>(0.0f)"
    c0, s0 = terms[0]
    expr = s0 if c0 == 1.0 else (f"vneg({s0})" if c0 == -1.0 else f"vmul({s0}, {_fmt(c0)})")
    for c, s in terms[1:]:
        if c == 1.0:
            expr = f"vadd({expr}, {s})"
        elif c == -1.0:
            expr = f"vsub({expr}, {s})"
        else:
            expr = f"vfma({_fmt(c)}, {s}, {expr})"
    return expr


def gen_fast() -> str:
    """The same MRT + Guo operator with far fewer operations (not bit-identical):
    M is block-diagonal in parity (even rows are symmetric under q <-> opp(q), odd rows
    antisymmetric), so moments come from the 9 pair sums P and differences D; the forcing
    moments M t have closed forms in u and G; inv(M) splits the same way."""
    Md = M.astype(np.float64)
    inv = np.linalg.inv(Md)
    inv[np.abs(inv) < NOISE] = 0.0
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    E = np.array(E_LIST, float)
    pairs = [(2 * p + 1, 2 * p + 2) for p in range(9)]
    even = [k for k in range(Q) if all(Md[k, q] == Md[k, OPP[q]] for q in range(Q))]
    odd = [k for k in range(Q) if k not in even]
    A = np.einsum("kq,q,qa->ka", Md, w, E)
    B = Md @ w
    C = np.einsum("kq,q,qa,qb->kab", Md, w, E, E)
    lines = []
    w_ = lines.append
    w_("")
    w_("// Reduced-operation MRT + Guo collision (same operator, not the reference's rounding):")
    w_("// parity-split moments from pair sums/differences, closed-form forcing moments")
    w_("// g_k = A_k.G - B_k (u.G) + u^T C_k G, parity-split inverse. Used by the FP16/BF16")
    w_("// storage forms and the FP32 fast form.")
    w_("template <class V>")
    w_("__device__ __forceinline__ void mrt_collide_fast(const V (&F)[19], V rho, V ux, V uy, V uz,")
    w_("    V gx, V gy, V gz, const float* __restrict__ S, V (&out)[19]) {")
    for p, (a, b) in enumerate(pairs):
        w_(f"  const V P{p} = vadd(F[{a}], F[{b}]), D{p} = vsub(F[{a}], F[{b}]);")
    for k in even:
        terms = [(Md[k, 0], "F[0]")] + [(Md[k, a], f"P{p}") for p, (a, b) in enumerate(pairs)]
        w_(f"  V m{k} = {_lin(terms)};")
    for k in odd:
        terms = [(Md[k, a], f"D{p}") for p, (a, b) in enumerate(pairs)]
        w_(f"  V m{k} = {_lin(terms)};")
    w_("  const V uG = vfma(ux, gx, vfma(uy, gy, vmul(uz, gz)));")
    w_("  const V pxx = vmul(ux, gx), pyy = vmul(uy, gy), pzz = vmul(uz, gz);")
    w_("  const V sxy = vfma(ux, gy, vmul(uy, gx)), syz = vfma(uy, gz, vmul(uz, gy)), "
       "sxz = vfma(ux, gz, vmul(uz, gx));")
    sym = {(0, 0): "pxx", (1, 1): "pyy", (2, 2): "pzz", (0, 1): "sxy", (1, 2): "syz", (0, 2): "sxz"}
    gnames = {}
    for k in range(Q):
        terms = [(A[k, 0], "gx"), (A[k, 1], "gy"), (A[k, 2], "gz"), (-B[k], "uG")]
        for (a, b), s in sym.items():
            coef = C[k, a, b] if a == b else C[k, a, b]  # C symmetric: C_ab u_a G_b + C_ba u_b G_a
            terms.append((coef, s))
        terms = [(float(c), s) for c, s in terms if abs(c) > 1e-14]
        if terms:
            w_(f"  const V g{k} = {_lin(terms)};")
            gnames[k] = f"g{k}"
    w_("  const V uu = vfma(ux, ux, vfma(uy, uy, vmul(uz, uz)));")
    meq = {0: "rho", 1: "uu", 3: "ux", 5: "uy", 7: "uz",
           9: "vfma(vadd(ux, ux), ux, vneg(vfma(uy, uy, vmul(uz, uz))))",
           11: "vfma(uy, uy, vneg(vmul(uz, uz)))",
           13: "vmul(ux, uy)", 14: "vmul(uy, uz)", 15: "vmul(ux, uz)"}
    for k in range(Q):
        g = gnames.get(k)
        if k in (0, 3, 5, 7):
            if g:
                w_(f"  m{k} = vadd(m{k}, {g});")
            continue
        d = f"vsub(m{k}, {meq[k]})" if k in meq else f"m{k}"
        rel = f"vfma(-S[{k}], {d}, m{k})"
        if g:
            w_(f"  m{k} = vfma(fmaf(-0.5f, S[{k}], 1.0f), {g}, {rel});")
        else:
            w_(f"  m{k} = {rel};")
    w_(f"  out[0] = {_lin([(inv[0, k], f'm{k}') for k in even])};")
    for p, (a, b) in enumerate(pairs):
        ev = _lin([(inv[a, k], f"m{k}") for k in even])
        od = _lin([(inv[a, k], f"m{k}") for k in odd])
        w_(f"  {{ const V e = {ev}, o = {od}; out[{a}] = vadd(e, o); out[{b}] = vsub(e, o); }}")
    w_("}")
    return "\n".join(lines)


E_LIST = E


# ---------------------------------------------------------------- checks --

def _seq_dense(mat: np.ndarray, x: np.ndarray) -> np.ndarray:
    """Literal sequential float32 evaluation: out = 0; out += mat[r, c] * x[c] for c in order."""
    n = x.shape[0]
    out = np.zeros((n, mat.shape[0]), np.float32)
    for r in range(mat.shape[0]):
        acc = np.zeros(n, np.float32)
        for c in range(mat.shape[1]):
            acc = (acc + (mat[r, c] * x[:, c]).astype(np.float32)).astype(np.float32)
        out[:, r] = acc
    return out


def _plan_inverse(m: np.ndarray) -> np.ndarray:
    classes, entry = inverse_plan()
    prod = {}
    for (k, ci), b in classes:
        prod[(k, ci)] = (np.float32(b) * m[:, k]).astype(np.float32)
    out = np.zeros_like(m)
    for q in range(Q):
        acc = None
        for k in range(Q):
            if (q, k) not in entry:
                continue
            sign, cls, j = entry[(q, k)]
            t = (prod[cls] * np.float32(2.0 ** j)).astype(np.float32)
            if acc is None:
                acc = t if sign > 0 else -t
            else:
                acc = (acc + t if sign > 0 else acc - t).astype(np.float32)
        out[:, q] = acc
    return out


def _plan_forward(x: np.ndarray) -> np.ndarray:
    """The generated forward transform in numpy: zero terms dropped, 2 X as X + X, rows in
    ``forward_plan()``'s reuse list continued from the negated prefix of an earlier row."""
    rows, reuse = forward_plan()
    out = np.zeros_like(x)
    prefix = {}
    for k in range(Q):
        terms = [(1 if c > 0 else -1, x[:, q] if abs(c) == 1 else (x[:, q] + x[:, q]))
                 for q, c in rows[k]]
        if k in reuse:
            a, used = reuse[k]
            acc = -prefix[(a, used)]
        else:
            s0, t0 = terms[0]
            acc, used = (t0 if s0 > 0 else -t0), 1
        for s, t in terms[used:]:
            acc = (acc + t if s > 0 else acc - t).astype(np.float32)
            used += 1
            prefix[(k, used)] = acc
        out[:, k] = acc
    return out


def self_check(n: int = 200_000, seed: int = 0) -> None:
    """Planned forward and inverse == literal dense products, bit for bit, on near-equilibrium
    populations and moments; the forward also on Guo-like source terms with signed zeros,
    where only the sign of an exact zero may differ (it is then added to a relaxed moment
    that is non-zero or +0, which such a zero cannot change)."""
    # Rows 0, 3, 5, 7 of the forward transform are update_macro's sums of f, e_x f, e_y f and
    # e_z f term for term (the step kernel reads rho and j from them).
    rows, reuse = forward_plan()
    for k, axis in ((0, None), (3, 0), (5, 1), (7, 2)):
        want = ([(q, 1) for q in range(Q)] if axis is None
                else [(q, E[q][axis]) for q in range(Q) if E[q][axis] != 0])
        if rows[k] != want or k in reuse:
            raise AssertionError(f"forward row {k} is not the macro sum it stands for")
    rng = np.random.default_rng(seed)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, np.float32)
    rho = rng.uniform(0.8, 1.2, n).astype(np.float32)
    F = (w[None, :] * rho[:, None] * (1 + rng.normal(0, 0.05, (n, Q)))).astype(np.float32)
    mom = _seq_dense(M, F)
    bad = np.count_nonzero(mom.view(np.uint32) != _plan_forward(F).view(np.uint32))
    if bad:
        raise AssertionError(f"planned forward differs from the literal sum in {bad} entries")
    t = (rng.normal(0, 1e-6, (n, Q)) * (rng.uniform(size=(n, Q)) < 0.7)).astype(np.float32)
    t[rng.uniform(size=(n, Q)) < 0.2] *= np.float32(-1.0)  # +-0 entries
    if not np.array_equal(_seq_dense(M, t), _plan_forward(t)):
        raise AssertionError("planned forward differs from the literal sum on source terms")
    mom[:, 3:8] += rng.normal(0, 1e-4, (n, 5)).astype(np.float32)
    full = _seq_dense(INV, mom)
    planned = _plan_inverse(mom)
    bad = np.count_nonzero(full.view(np.uint32) != planned.view(np.uint32))
    if bad:
        raise AssertionError(f"planned inverse differs from the literal sum in {bad} entries")


if __name__ == "__main__":
    self_check()
    OUT.write_text(gen())
    print("wrote", OUT)
