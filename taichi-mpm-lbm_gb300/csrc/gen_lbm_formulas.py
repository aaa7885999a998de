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
        lines.append(f"{var} = 0.0f;")
        return lines
    s0, e0 = terms[0]
    lines.append(f"{var} = {e0 if s0 > 0 else '-' + e0};")
    for s, e in terms[1:]:
        op = "__fadd_rn" if s > 0 else "__fsub_rn"
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
    w("namespace fsi {")
    w("")
    # forward transform on an input array X (F or Guo terms t)
    w("// m[k] = sum_q M[k][q] * X[q], sequential in q (lbm3d.py:269-274).")
    w("__device__ __forceinline__ void mrt_forward(const float (&X)[19], float (&m)[19]) {")
    w("  float two[19];")
    need_two = sorted({q for k in range(Q) for q in range(Q) if abs(M[k, q]) == 2})
    for q in need_two:
        w(f"  two[{q}] = __fadd_rn(X[{q}], X[{q}]);")
    for k in range(Q):
        terms = []
        for q in range(Q):
            c = int(M[k, q])
            if c == 0:
                continue
            terms.append((1 if c > 0 else -1, f"X[{q}]" if abs(c) == 1 else f"two[{q}]"))
        body = chain(f"m[{k}]", terms)
        w("  " + " ".join(body))
    w("}")
    w("")
    classes, entry = inverse_plan()
    w("// f[q] = sum_k inv(M)[q][k] * m[k], sequential in k (lbm3d.py:328-333).")
    w(f"// {len(classes)} rounded products; every other product is an exact power-of-two scaling.")
    w("__device__ __forceinline__ void mrt_inverse(const float (&m)[19], float (&f)[19]) {")
    names = {}
    for (k, ci), b in classes:
        nm = f"p{k}_{ci}"
        names[(k, ci)] = nm
        w(f"  const float {nm} = __fmul_rn({f32hex(b)}, m[{k}]);")
    for q in range(Q):
        terms = []
        for k in range(Q):
            if (q, k) not in entry:
                continue
            sign, cls, j = entry[(q, k)]
            base = names[cls]
            expr = base if j == 0 else f"__fmul_rn({base}, {f32hex(2.0 ** j)})"
            terms.append((sign, expr))
        w("  { float a; " + " ".join(chain("a", terms)) + f" f[{q}] = a; }}")
    w("}")
    w("")
    w("}  // namespace fsi")
    return "\n".join(out) + "\n"


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


def self_check(n: int = 200_000, seed: int = 0) -> None:
    """Planned inverse == literal dense inverse, bit for bit, on near-equilibrium moments."""
    rng = np.random.default_rng(seed)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12, np.float32)
    rho = rng.uniform(0.8, 1.2, n).astype(np.float32)
    F = (w[None, :] * rho[:, None] * (1 + rng.normal(0, 0.05, (n, Q)))).astype(np.float32)
    mom = _seq_dense(M, F)
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
