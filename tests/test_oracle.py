"""CPU: the oracle against the golden vectors and an independent restatement."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN


def load_f64(name, d):
    return np.fromfile(os.path.join(GOLDEN, name), dtype="<f8").reshape(-1, d)


@pytest.mark.parametrize("name", ["test100", "test128"])
def test_oracle_known_answers(oracle_mod, name):
    g = json.load(open(os.path.join(GOLDEN, "join_golden.json")))["files"][name]
    x = load_f64(name + ".f64", g["d"])
    assert x.shape == (g["n"], g["d"])
    for case in g["cases"]:
        counts, total = oracle_mod.self_join(x, case["eps"])
        assert total == case["total"], case["eps"]
        assert counts.tolist() == case["counts"]


def test_oracle_ties_against_rational_restatement(oracle_mod):
    g = json.load(open(os.path.join(GOLDEN, "ties.json")))
    x = load_f64("ties.f64", g["d"])
    for case in g["cases"]:
        counts, total = oracle_mod.self_join(x, case["eps"])
        assert total == case["total"], case["eps"]
        assert counts.tolist() == case["counts"]


@pytest.mark.parametrize("name", ["contraction", "contraction_d64", "contraction_d128"])
def test_oracle_follows_the_compiled_reference_reading(oracle_mod, name):
    """The contraction fixtures hold pairs within ulps of the radius whose
    count depends on how the reference's `acc += (p - c) * (p - c)`
    (kernel_join.cu:186-189) is rounded: the plain fma chain, the uncontracted
    sum, or fma(t0, t0, fl(t1 * t1)) followed by the fma chain -- the form
    nvcc compiles it to (pinned by running the reference's own kernel, see
    test_gpu_reference.py).  The oracle takes that form."""
    g = json.load(open(os.path.join(GOLDEN, name + ".json")))
    x = load_f64(name + ".f64", g["d"])
    counts, total = oracle_mod.self_join(x, g["eps"])
    totals = {g[r]["total"] for r in ("fma", "first", "mul_add")}
    assert len(totals) == 3
    assert total == g["first"]["total"]
    assert counts.tolist() == g["first"]["counts"]
    assert oracle_mod.threshold(g["eps"]) == g["threshold"]
    if g["d"] <= 18:
        c2, t2 = oracle_mod.py_self_join(x, g["eps"])
        assert t2 == total and c2.tolist() == g["first"]["counts"]


def test_oracle_matches_python_loops_random(oracle_mod):
    rng = np.random.default_rng(3)
    x = rng.random((40, 5))
    for eps in (0.2, 0.5, 0.8):
        c1, t1 = oracle_mod.self_join(x, eps)
        c2, t2 = oracle_mod.py_self_join(x, eps)
        assert t1 == t2 and c1.tolist() == c2.tolist()


def test_threshold_properties(oracle_mod):
    rng = np.random.default_rng(5)
    for eps in list(rng.random(200) * 10) + [1e-300, 1e-160, 1e150, 1.0, 0.1]:
        T = oracle_mod.threshold(eps)
        assert math.sqrt(T) <= eps
        assert not (math.sqrt(math.nextafter(T, math.inf)) <= eps)
        assert T == oracle_mod.py_threshold(eps)
    assert oracle_mod.threshold(0.0) == 0.0
    assert oracle_mod.threshold(-1.0) == -math.inf
    assert math.isnan(oracle_mod.threshold(float("nan")))
    assert oracle_mod.threshold(float("inf")) == math.inf


def test_oracle_nonfinite_rows(oracle_mod):
    x = np.array([[0.0, 0.0], [np.nan, 0.0], [np.inf, 1.0], [0.0, 0.1]])
    c, t = oracle_mod.self_join(x, 0.5)
    assert c.tolist() == [2, 0, 0, 2]
    c, t = oracle_mod.self_join(x, float("inf"))
    # inf row: d2 = inf with finite rows (counted at eps = inf), NaN with itself (inf - inf)
    assert c.tolist() == [3, 0, 2, 3]


def test_oracle_query_counts(oracle_mod):
    rng = np.random.default_rng(9)
    x = rng.random((300, 7))
    full, _ = oracle_mod.self_join(x, 0.6)
    rows = np.array([0, 5, 299, 17])
    assert oracle_mod.query_counts(x, 0.6, rows).tolist() == full[rows].tolist()


def test_oracle_neighbor_lists_golden(oracle_mod):
    """The oracle's lists have the golden counts as lengths and hold exactly
    the pairs a direct restatement of the predicate selects."""
    g = json.load(open(os.path.join(GOLDEN, "join_golden.json")))["files"]["test100"]
    x = np.fromfile(os.path.join(GOLDEN, "test100.f64"), dtype="<f8").reshape(-1, g["d"])
    case = g["cases"][len(g["cases"]) // 2]
    off, nb = oracle_mod.neighbor_lists(x, case["eps"])
    assert np.diff(off.astype(np.int64)).tolist() == case["counts"]
    T = oracle_mod.threshold(case["eps"])
    for i in range(0, x.shape[0], 7):
        ref = [j for j in range(x.shape[0]) if oracle_mod.pair_d2(x[i], x[j]) <= T]
        assert nb[off[i]:off[i + 1]].tolist() == ref
