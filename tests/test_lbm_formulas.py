"""The generated MRT register formulas equal the literal float32 19x19 sums of the reference."""
from __future__ import annotations

import importlib.util
from pathlib import Path

import numpy as np

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
