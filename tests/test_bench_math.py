"""The bench's rate and roofline arithmetic (bench.kernel_table,
bench.roofline_of) on made-up kernel timings: the symmetric products are
rated by their own operation counts per unordered pair against the FMA-pipe
instruction rate (half the measured flop peak), the dominant kernel sets the
roofline, and the fraction is achieved over peak."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_symmetric_fp64_and_fp32_rates():
    n = 90000
    pairs_unordered = n * (n - 1) / 2
    # (launches, total ms, columns) for FP64, FP32, double-single
    kst = [(2, 460.0, 2), (14, 60.0, 14), (0, 0.0, 0)]
    peak64, peak32 = 1.2, 72.0  # TFLOP/s (FMA counted twice)
    t = bench.kernel_table(kst, n, peak64, peak32, ("symmetric", 1, 1))
    f64 = t["tmu_fp64"]
    assert f64["achieved_tops"] == pytest.approx(bench.FP64_SYM_OPS_PER_PAIR * pairs_unordered * 2 / 0.46 / 1e12)
    assert f64["frac"] == pytest.approx(f64["achieved_tops"] / (peak64 / 2))
    f32 = t["tmu_fp32"]
    assert f32["kernel"] == "symmetric"
    assert f32["achieved_tops"] == pytest.approx(bench.FP32_SYM_OPS_PER_PAIR * pairs_unordered * 14 / 0.06 / 1e12)
    assert f32["frac"] == pytest.approx(f32["achieved_tops"] / (peak32 / 2))
    assert f32["frac_nominal"] == pytest.approx(f32["achieved_tops"] / 40.3)
    assert "tmu_ds" not in t


def test_roofline_takes_the_dominant_kernel():
    n = 90000
    kst = [(2, 460.0, 2), (14, 60.0, 14), (0, 0.0, 0)]
    t = bench.kernel_table(kst, n, 1.2, 72.0, ("symmetric", 1, 1))
    r = bench.roofline_of(t, 520.0, n)
    assert r["bound"] == "fp64" and r["kernel"] == "tmu_fp64"
    assert r["frac"] == pytest.approx(t["tmu_fp64"]["frac"])
    assert r["share_of_timed"] == pytest.approx(460.0 / 520.0)
    assert r["traffic"] == pytest.approx(bench.TRAFFIC_30K["tmu_fp64"] * n / 30000)


def test_tiled_fp32_kernel_keeps_the_conventional_rate():
    n = 30000
    kst = [(0, 0.0, 0), (10, 10.0, 10), (0, 0.0, 0)]
    t = bench.kernel_table(kst, n, 1.2, 72.0, ("tiled", 1, 4))
    f32 = t["tmu_fp32"]
    assert f32["kernel"] == "tiled" and "achieved_tops" not in f32
    assert f32["achieved_tflops"] == pytest.approx(bench.FLOP_PER_PAIR * n * (n - 1) * 10 / 0.01 / 1e12)
