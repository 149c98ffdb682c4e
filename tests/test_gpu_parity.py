"""GPU: every precision mode returns per-point counts bit-identical to the
FP64 oracle (the reference's predicate), on golden and seeded inputs."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MODES = ["fp64_direct", "fp64_dmma", "bf16", "bf16_split", "fp16", "fp8_e4m3"]


def load_f64(name, d):
    return np.fromfile(os.path.join(GOLDEN, name), dtype="<f8").reshape(-1, d)


def eps_for_mean(x, mean, rng):
    """eps whose expected neighbour count is about `mean` (from sampled pairs)."""
    n = x.shape[0]
    i = rng.integers(0, n, 4000)
    j = rng.integers(0, n, 4000)
    d = np.sqrt(((x[i] - x[j]) ** 2).sum(1))
    q = min(0.999, max(mean / n, 1e-4))
    return float(np.quantile(d, q))


def clustered(n, d, rng, k=8, sigma=0.05, offset=0.0):
    c = rng.random((k, d))
    lab = rng.integers(0, k, n)
    return c[lab] + sigma * rng.standard_normal((n, d)) + offset


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", ["test100", "test128"])
def test_golden_sample_files(ej, mode, name):
    g = json.load(open(os.path.join(GOLDEN, "join_golden.json")))["files"][name]
    x = load_f64(name + ".f64", g["d"])
    for case in g["cases"]:
        counts, total, st = ej.self_join(x, case["eps"], precision=mode)
        assert total == case["total"], (mode, case["eps"], st)
        assert counts.tolist() == case["counts"]


@pytest.mark.parametrize("mode", MODES)
def test_golden_ties(ej, mode):
    g = json.load(open(os.path.join(GOLDEN, "ties.json")))
    x = load_f64("ties.f64", g["d"])
    for case in g["cases"]:
        counts, total, st = ej.self_join(x, case["eps"], precision=mode)
        assert counts.tolist() == case["counts"], (mode, case["eps"], st)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("name", ["contraction", "contraction_d64", "contraction_d128"])
def test_golden_contraction(ej, mode, name):
    """Pairs within ulps of the radius whose count depends on how the
    reference's accumulation is rounded: every mode counts what the
    reference's own compiled kernel counts (fma(t0, t0, fl(t1 * t1)), then
    the fma chain; kernel_join.cu:186-189)."""
    g = json.load(open(os.path.join(GOLDEN, name + ".json")))
    x = load_f64(name + ".f64", g["d"])
    counts, total, st = ej.self_join(x, g["eps"], precision=mode)
    assert total == g["first"]["total"], (mode, st)
    assert counts.tolist() == g["first"]["counts"], mode


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n,d", [(1, 3), (2, 1), (15, 18), (16, 3), (17, 64), (127, 128),
                                 (128, 18), (129, 64), (1000, 18), (3000, 128), (2500, 1)])
def test_random_sizes(ej, oracle_mod, mode, n, d):
    rng = np.random.default_rng(n * 1000 + d)
    x = clustered(n, d, rng) if n > 200 else rng.random((n, d))
    eps = eps_for_mean(x, 20, rng) if n > 20 else 0.5
    exp, tot = oracle_mod.self_join(x, eps)
    counts, total, st = ej.self_join(x, eps, precision=mode)
    assert total == tot, st
    assert np.array_equal(counts, exp)


@pytest.mark.parametrize("mode", MODES)
def test_offset_data_exercises_centring(ej, oracle_mod, mode):
    rng = np.random.default_rng(21)
    x = clustered(4000, 64, rng, k=16, sigma=0.03, offset=1000.0)
    eps = eps_for_mean(x, 40, rng)
    exp, tot = oracle_mod.self_join(x, eps)
    counts, total, st = ej.self_join(x, eps, precision=mode)
    assert np.array_equal(counts, exp), st


@pytest.mark.parametrize("mode", MODES)
def test_edge_cases(ej, oracle_mod, mode):
    rng = np.random.default_rng(5)
    x = rng.random((300, 9))
    x[10] = x[11] = x[12]          # duplicates
    x[50] = np.nan                  # NaN row: never a neighbour, not even of itself
    x[60, 3] = np.inf               # Inf coordinate
    x[70, 0] = -np.inf
    for eps in (0.0, 0.3, 0.8, 100.0, float("inf"), -1.0, float("nan")):
        exp, tot = oracle_mod.self_join(x, eps)
        counts, total, st = ej.self_join(x, eps, precision=mode)
        assert np.array_equal(counts, exp), (eps, st)
        assert total == tot
    # all-equal points
    y = np.full((257, 5), 0.25)
    for eps in (0.0, 1e-300, 1.0):
        counts, total, _ = ej.self_join(y, eps, precision=mode)
        assert total == 257 * 257 and np.all(counts == 257)


def test_empty_input(ej):
    counts, total, st = ej.self_join(np.zeros((0, 4)), 0.5)
    assert total == 0 and counts.shape == (0,)


@pytest.mark.parametrize("mode", ["bf16_split", "fp64_dmma"])
def test_device_resident_input_and_output(ej, oracle_mod, mode):
    import torch
    rng = np.random.default_rng(8)
    x = clustered(2000, 32, rng)
    eps = eps_for_mean(x, 25, rng)
    exp, tot = oracle_mod.self_join(x, eps)
    xd = torch.from_numpy(x).cuda()
    cd = torch.zeros(2000, dtype=torch.int32, device="cuda")
    _, total, _ = ej.self_join(xd, eps, precision=mode, counts=cd)
    assert total == tot
    assert np.array_equal(cd.cpu().numpy(), exp)


def test_determinism(ej):
    rng = np.random.default_rng(12)
    x = clustered(5000, 64, rng)
    eps = eps_for_mean(x, 30, rng)
    a, ta, sa = ej.self_join(x, eps, precision="bf16")
    b, tb, sb = ej.self_join(x, eps, precision="bf16")
    assert ta == tb and np.array_equal(a, b)
    assert sa["band_pairs"] == sb["band_pairs"]


def test_reference_compat_entry_point(ej, oracle_mod):
    """GPUJoinMainBruteForce on the padded layout main.cu:38-57 builds."""
    x = load_f64("test128.f64", 18)
    n, din, dcomp = 128, 18, 32
    padded = np.zeros((n + 15, dcomp))
    padded[:n, :din] = x
    for mode in (1, 2, 3, 4):
        assert ej.GPUJoinMainBruteForce(mode, 0, padded, n, 0.1, din, dcomp) == 11100
    with pytest.raises(ej.EjoinError):
        ej.GPUJoinMainBruteForce(9, 0, padded, n, 0.1, din, dcomp)


def test_query_counts(ej, oracle_mod):
    rng = np.random.default_rng(13)
    x = clustered(3000, 20, rng)
    eps = eps_for_mean(x, 30, rng)
    rows = rng.choice(3000, 100, replace=False)
    assert np.array_equal(ej.query_counts(x, eps, rows), oracle_mod.query_counts(x, eps, rows))


def test_cli_reference_argv_and_csv(ej, tmp_path):
    """ejoin_main takes the reference's argv (file, eps, searchMode, device)
    and appends the reference's CSV result line (main.cu:115-127)."""
    import subprocess
    x = load_f64("test128.f64", 18)
    data = tmp_path / "test128.txt"
    with open(data, "w") as f:
        for r in x:
            f.write(", ".join(f"{v:.6f}" for v in r) + " \n")
    exe = os.path.join(os.path.dirname(ej.LIB_PATH), "ejoin_main")
    for mode, eps, total in ((4, 0.1, 11100), (1, 0.05, 828), (5, 0.2, 16384)):
        out = subprocess.run([exe, str(data), str(eps), str(mode), "0"], cwd=tmp_path,
                             capture_output=True, text=True, check=True).stdout
        assert f"Total result set size: {total}" in out
    lines = open(tmp_path / "tensor_brute-force.txt").read().splitlines()
    assert lines[0].startswith("Dataset, epsilon, searchMode, executionTime, totalNeighbors")
    assert len(lines) == 4 and lines[1].split(", ")[4] == "11100"
    # inputDim, computeDim, blockSize, warpPerBlock, computePrec, accumPrec of
    # the kernel each mode ran: FP16 Gram screen (AUTO at d = 18), FP64 direct
    assert lines[1].split(", ")[5:] == ["18", "64", "608", "19", "16", "32"]
    assert lines[2].split(", ")[5:] == ["18", "18", "256", "8", "64", "64"]


@pytest.mark.parametrize("mode", ["bf16_split", "fp16", "fp8_e4m3", "fp64_dmma"])
def test_extreme_magnitudes(ej, oracle_mod, mode):
    """Coordinates near the FP64 range limits: tiny (1e-200) and huge (1e200,
    beyond FP32) data stay exact (huge data takes the FP64 screen)."""
    rng = np.random.default_rng(31)
    base = clustered(1500, 16, rng)
    for scale in (1e-200, 1e-30, 1e30, 1e200):
        x = base * scale
        eps = eps_for_mean(x, 15, rng)
        exp, tot = oracle_mod.self_join(x, eps)
        counts, total, st = ej.self_join(x, eps, precision=mode)
        assert np.array_equal(counts, exp), (scale, st)
