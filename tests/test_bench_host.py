"""Host logic of bench.py (no GPU): the clock record, the roofline peak, and the reference
arm's JSON line (the oracle timed on a small sample of the same workload)."""
from __future__ import annotations

import functools
import json
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

import bench
from fsi import scenes

ROOT = Path(__file__).resolve().parents[1]


def _sampler(rows):
    s = bench.ClockSampler(0)
    s.rows = [[x.strip() for x in r.split(",")] for r in rows]
    return s


def test_clock_summary_median_and_throttle_reasons():
    s = _sampler(["2070, 2070, 300.1, Not Active, Not Active, Not Active, Not Active",
                  "1980, 2070, 520.4, Not Active, Not Active, Not Active, Active",
                  "2070, 2070, 410.0, Not Active, Not Active, Not Active, Not Active"])
    out = s.summary()
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"] and out["samples"] == 3
    assert out["power_w_max"] == pytest.approx(520.4)
    hot = _sampler(["1500, 2070, [N/A], Active, Not Active, Active, Not Active"]).summary()
    assert hot["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"] and hot["power_w_max"] == 0.0
    assert bench.ClockSampler(0).summary()["reasons"] == ["unsampled"]


def test_roofline_peak_is_the_measured_copy_bandwidth():
    peak, source = bench.load_peaks()
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        assert source == "measured"
        assert peak == float(json.loads(path.read_text())["hbm_gbs"])
    else:
        assert (peak, source) == (6800.0, "fallback")


@pytest.fixture
def small_sample(monkeypatch):
    """cpu_coupled_sample on a small channel of the headline kind: 64x24x24, two bodies."""
    for var in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(var, raising=False)
    real = bench.cpu_coupled_sample
    monkeypatch.setattr(bench, "cpu_coupled_sample", lambda steps, warmup, nthreads, **kw:
                        real(steps, warmup, nthreads, nx=64, ny=24, nz=24, bodies=2,
                             cube_edge=4, sphere_radius=2.0))


def test_reference_arm_prints_the_contract_line(small_sample):
    out = bench.run_reference(SimpleNamespace(steps=2, warmup=1))
    assert out["impl"] == "reference" and out["metric"] == bench.METRIC
    assert out["unit"] == "MLUPS" and out["value"] > 0 and out["higher_is_better"] is True
    assert out["n_gpus"] == 1 and (out["steps"], out["warmup"]) == (2, 1)
    assert out["ms_per_step"] > 0 and out["vs_baseline"] is None and out["scaling"] == "weak"
    assert out["config"]["workload"].startswith("coupled at scale")
    cb = out["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == out["value"] and cb["cores"] >= 1
    assert out["e2e"] == {"value": out["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                          "d2h_bytes_per_step": 0}
    assert out["particle_steps_per_s"] > 0
    json.dumps(out)  # one JSON line


def test_bounded_sample_for_long_reference_runs(small_sample):
    out = bench.run_reference(SimpleNamespace(steps=bench.FULL_REFERENCE_STEPS, warmup=1))
    assert "bounded sample" in out["config"]["sample"]


def test_roofline_bytes_basis():
    assert bench.lattice_bytes(10, 3) == 10 * 181 + 3 * 4
    base = np.array([[0, 0, 0], [0, 0, 0], [5, 5, 5], [-3, 0, 0]])
    # one cell at the corner: its 27 stencil nodes; one interior cell: 27 more; the last
    # particle's stencil lies outside the grid
    assert bench.touched_nodes(base, (16, 16, 16)) == 54
    assert bench.touched_nodes(np.array([[14, 14, 14]]), (16, 16, 16)) == 8


def test_reference_arm_runs_on_rank_zero_only(small_sample, monkeypatch):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    assert bench.run_reference(SimpleNamespace(steps=1, warmup=0)) is None
