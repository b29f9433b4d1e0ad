"""The compute roofline's arithmetic (host code, no GPU): frozen per-pair
operation counts for every benchmark cutter, and T_roof / T_step formed from
the library's per-call counters as opencamlib_gb300.roofline documents."""
import pytest

from opencamlib_gb300 import cutters as cu
from opencamlib_gb300 import roofline as rf


def test_every_benchmark_cutter_has_frozen_counts():
    names = list(cu.standard_cutters())
    assert rf.measured(names)
    for n in names:
        assert 100 < rf.FP32_PER_SCREEN[n] < 10000
        assert 10 < rf.FP64_PER_REFINED[n] < 10000


def test_step_roofline_arithmetic():
    counts = {"cyl": (1_000_000, 10_000), "bull": (2_000_000, 50_000)}
    p32, p64 = 80e12, 1.25e12
    r = rf.step_roofline(counts, 0.01, p32, p64)
    f32 = 1e6 * rf.FP32_PER_SCREEN["cyl"] + 2e6 * rf.FP32_PER_SCREEN["bull"]
    f64 = 1e4 * rf.FP64_PER_REFINED["cyl"] + 5e4 * rf.FP64_PER_REFINED["bull"]
    assert r["fp32_ops"] == pytest.approx(f32)
    assert r["fp64_ops"] == pytest.approx(f64)
    assert r["t_roof_s"] == pytest.approx(f32 / p32 + f64 / p64)
    assert r["frac"] == pytest.approx(r["t_roof_s"] / 0.01)
    # one FP32-equivalent rate against the FP32 peak gives the same fraction
    assert r["achieved_flops_fp32_equiv"] / p32 == pytest.approx(r["frac"])


def test_every_benchmark_cutter_has_screen_traffic():
    """roofline.traffic: the screens' DRAM bytes per call on the full raster,
    from a one-pass ncu capture; at least the algorithmic bytes of a call
    (every triangle's FP64 vertices once, 24 B in and 36 B out per point)."""
    algorithmic = 1_048_576 * 72 + 1_000_000 * (24 + 36)
    for n in cu.standard_cutters():
        b = rf.SCREEN_DRAM_BYTES[n]
        assert b is not None and algorithmic <= b < 20 * algorithmic
