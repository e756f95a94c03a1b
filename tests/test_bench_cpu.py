"""bench.py's figures that come from committed ncu summaries, checked on the CPU.

The bench line's `roofline.traffic`, its pipe percentages and its FP64-pipe roof read
profiles/*.md; a summary that lost a key would silently turn them into null.
"""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("oeb_bench_cpu", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    argv = sys.argv
    sys.argv = ["bench.py"]
    try:
        spec.loader.exec_module(mod)
    finally:
        sys.argv = argv
    return mod


NAMES = ["laplace", "hdiffsa", "hdiffsmag", "hadvuv", "hadvuv5th", "fastwavesuv", "uvbke", "nh_p_grad", "p_grad_c",
         "fvtp2d"]


def test_dominant_kernel_summary_keys(bench):
    traffic = bench._ncu_traffic("fvtp2d")
    # DRAM bytes per call: at least the algorithmic 80 B/pt (the q_i, q_j, fx2, fy2 round
    # trip between the two launches comes on top), at most a few times it
    assert traffic is not None and 80 * 128 * 128 * 80 <= traffic <= 4 * 80 * 128 * 128 * 80
    for key in ("fp64_pipe_active_pct", "alu_pipe_active_pct"):
        v = bench._ncu_summary("fvtp2d", key)
        assert v is not None and 0 < v <= 100


def test_fp64_pipe_counts_present(bench):
    for k in NAMES:
        v = bench._ncu_summary(bench.PIPE_MIX_PROFILE, "fp64_instr_per_point_" + k)
        assert v is not None and 1 <= v <= 200, k


def test_fp64_pipe_roofline_arithmetic(bench):
    # the measured FP64 addition rate, rescaled from the probe's SM clock to the timed region's
    per_kernel = {k: 0.1 for k in NAMES}
    add_rate = 3.2e11
    r = bench._fp64_pipe_roofline(NAMES, per_kernel, "fvtp2d", 1.0, {"sm_mhz": 1800.0}, 100, add_rate,
                                  {"sm_mhz": 2000.0})
    rate = add_rate * 1800.0 / 2000.0
    pts = bench.NX * bench.NY * bench.NZ
    want_k = r["kernel_instr_per_point"] * pts / rate * 1e3
    assert r["kernel_bound_ms"] == pytest.approx(want_k, rel=1e-4)
    assert r["kernel_frac"] == pytest.approx(want_k / 0.1, rel=1e-3)
    want_s = sum(bench._ncu_summary(bench.PIPE_MIX_PROFILE, "fp64_instr_per_point_" + k) for k in NAMES) * pts / rate * 1e3
    assert r["step_bound_ms"] == pytest.approx(want_s, rel=1e-4)
    assert r["step_frac"] == pytest.approx(want_s / 1.0, rel=1e-3)
    assert r["rate_per_clk_per_sm"] == pytest.approx(add_rate / (100 * 2000e6), rel=1e-3)
    # no measured rate: no roof
    assert bench._fp64_pipe_roofline(NAMES, per_kernel, "fvtp2d", 1.0, {"sm_mhz": 1800.0}, 100, None, {}) is None


def test_tuning_summary_counts_each_choice(bench):
    h = bench._tuning_summary([(4, 0, 0), (4, 2, 2), (1, 1, 0)])
    assert h == {"kb": {"4": 2, "1": 1}, "shape": {"32x32": 1, "64x16": 1, "32x8": 1},
                 "form": {"wave": 2, "per_member": 1}}


def test_chain_and_batch_roofs(bench):
    # the chained and batched legs' anchors read profiles/ncu_pipe_chain_128x128x80.md
    instr = bench._ncu_summary(bench.CHAIN_PROFILE, "fp64_instr_per_point_chain_f64")
    assert instr is not None and 100 <= instr <= 5000
    for p in ("f64", "f32"):
        b = bench._ncu_summary(bench.CHAIN_PROFILE, "dram_bytes_per_point_chain_" + p)
        assert b is not None and 100 <= b <= 10000, p
    chain = {"f64": {"ms_per_step": 2.0}, "f32": {"ms_per_step": 0.5}}
    batched = {"ms_per_run": 80.0, "fp64_points": 40_000_000}
    rate, peak = 5.0e11, 7000.0
    bench._chain_roofs(chain, batched, rate, peak)
    pts = bench.NX * bench.NY * bench.NZ
    assert chain["f64"]["fp64_pipe_roof"]["bound_ms"] == pytest.approx(instr * pts / rate * 1e3, rel=1e-3)
    assert chain["f64"]["fp64_pipe_roof"]["frac"] == pytest.approx(instr * pts / rate * 1e3 / 2.0, rel=1e-3)
    b32 = bench._ncu_summary(bench.CHAIN_PROFILE, "dram_bytes_per_point_chain_f32")
    assert chain["f32"]["dram"]["gbs"] == pytest.approx(b32 * pts / 0.5e-3 / 1e9, rel=1e-3)
    assert batched["fp64_pipe_roof"]["frac"] == pytest.approx(instr * 40e6 / rate * 1e3 / 80.0, rel=1e-3)
