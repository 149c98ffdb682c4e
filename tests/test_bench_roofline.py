"""CPU: the roofline fractions of the bench line are reproducible from the
line's own fields (gram_blocks, tile_pairs_run, ms_gram) and the peak file,
with the definitions bench.gram_roofline documents."""
import argparse
import importlib.util
import os

import pytest

from conftest import ROOT

spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
bench = importlib.util.module_from_spec(spec)
spec.loader.exec_module(bench)

PEAKS = {"bf16_tflops": 1910.6, "bf16_tflops_sustained": 1703.5}


def run(prec, d, ms, tiles, blocks):
    stats = [{"ms_gram": ms, "tile_pairs_run": tiles, "gram_blocks": blocks}]
    args = argparse.Namespace(config="cX")
    return bench.gram_roofline(stats, d, prec, PEAKS, args, 8)


def test_bf16_split_c4_shape():
    r = run("bf16_split", 64, 13.2, 2_593_306, 1_413_573)
    flops = 2_593_306 * 2.0 * 128 * 128 * (3 * 64)
    assert r["flops_per_launch"] == pytest.approx(flops)
    assert r["frac"] == pytest.approx(flops / 13.2e-3 / 1e12 / 1910.6)
    executed = 1_413_573 * 2.0 * 128 * 256 * (3 * 64 + 16)
    assert r["frac_executed"] == pytest.approx(executed / 13.2e-3 / 1e12 / 1910.6)
    useful = 2_593_306 * 2.0 * 128 * 128 * 64
    assert r["frac_useful"] == pytest.approx(useful / 13.2e-3 / 1e12 / 1910.6)
    # per block: two 128-byte K-slab stages of 128 + 256 rows, and 32-byte aug rows
    assert r["l2_operand_bytes"] == 1_413_573 * (2 * 384 * 128 + 384 * 32)
    assert "burst" in r["peak_source"]


def test_long_launch_uses_sustained_peak():
    r = run("bf16_split", 256, 2400.0, 122_078_125, 61_000_000)
    assert r["peak"] == pytest.approx(1703.5)
    assert "sustained" in r["peak_source"]


def test_fp8_peak_is_twice_bf16():
    r = run("fp8_e4m3", 1024, 360.0, 30_525_391, 15_268_553)
    assert r["peak"] == pytest.approx(2 * 1910.6)
    flops = 30_525_391 * 2.0 * 128 * 128 * 1024
    assert r["frac"] == pytest.approx(flops / 0.36 / 1e12 / (2 * 1910.6))
