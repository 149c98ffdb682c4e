"""GPU: neighbour lists (CSR) of the exact self-join are identical to the
oracle's -- every list, in ascending order, self included -- in every
precision mode and with learned pruning; plus the sizing-only call and the
too-small-buffer error."""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

MODES = ["fp64_direct", "fp64_dmma", "bf16", "bf16_split", "fp16", "fp8_e4m3"]


def clustered(n, d, rng, k=8, sigma=0.05):
    c = rng.random((k, d))
    return c[rng.integers(0, k, n)] + sigma * rng.standard_normal((n, d))


def eps_for_mean(x, mean, rng):
    n = x.shape[0]
    i, j = rng.integers(0, n, 4000), rng.integers(0, n, 4000)
    return float(np.quantile(np.sqrt(((x[i] - x[j]) ** 2).sum(1)), min(0.999, mean / n)))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n,d", [(2500, 18), (3000, 64), (700, 3)])
def test_lists_match_oracle(ej, oracle_mod, mode, n, d):
    rng = np.random.default_rng(n + d)
    x = clustered(n, d, rng)
    x[7] = x[3]  # a duplicate
    x[11, 2 % d] = np.nan  # a non-finite row: no neighbours, not even itself
    eps = eps_for_mean(x[np.isfinite(x).all(1)], 30, rng)
    off_ref, nb_ref = oracle_mod.neighbor_lists(x, eps)
    off, nb, st = ej.neighbor_lists(x, eps, precision=mode)
    assert np.array_equal(off, off_ref), (mode, st)
    assert np.array_equal(nb, nb_ref), (mode, st)


@pytest.mark.parametrize("mode", ["bf16_split", "fp16"])
def test_lists_with_learned_pruning(ej, oracle_mod, mode):
    rng = np.random.default_rng(5)
    lat = rng.random((20000, 4))
    E = np.linalg.qr(rng.standard_normal((64, 4)))[0]
    x = lat @ E.T + 0.002 * rng.standard_normal((20000, 64))
    eps = eps_for_mean(x, 40, rng)
    off_ref, nb_ref = oracle_mod.neighbor_lists(x, eps)
    off, nb, st = ej.neighbor_lists(x, eps, precision=mode, proj_k=8)
    assert st["tile_pairs_run"] < st["tile_pairs_total"]  # pruning was active
    assert np.array_equal(off, off_ref) and np.array_equal(nb, nb_ref)


def test_lists_golden_file(ej, oracle_mod):
    g = json.load(open(os.path.join(GOLDEN, "join_golden.json")))["files"]["test128"]
    x = np.fromfile(os.path.join(GOLDEN, "test128.f64"), dtype="<f8").reshape(-1, g["d"])
    for case in g["cases"]:
        off, nb, _ = ej.neighbor_lists(x, case["eps"], precision="bf16_split")
        assert np.diff(off.astype(np.int64)).tolist() == case["counts"]
        off_ref, nb_ref = oracle_mod.neighbor_lists(x, case["eps"])
        assert np.array_equal(nb, nb_ref)


def test_sizing_call_and_small_buffer(ej):
    rng = np.random.default_rng(9)
    x = clustered(1000, 16, rng)
    eps = eps_for_mean(x, 20, rng)
    counts, total, _ = ej.self_join(x, eps, precision="bf16_split")
    L = ej.load_library()
    o = ej._options(precision="bf16_split")
    xs = np.ascontiguousarray(x)
    off = np.zeros(1001, dtype=np.uint64)
    tot = ctypes.c_uint64(0)
    # neighbors = NULL: offsets and the total only
    assert L.ejoin_neighbor_lists(xs.ctypes.data, 1000, 16, eps, ctypes.byref(o), off.ctypes.data,
                                  None, 0, ctypes.byref(tot), None) == 0
    assert tot.value == total and np.diff(off.astype(np.int64)).tolist() == counts.tolist()
    # a buffer one entry short: ENOMEM, offsets still filled
    nb = np.zeros(total - 1, dtype=np.uint32)
    off2 = np.zeros(1001, dtype=np.uint64)
    rc = L.ejoin_neighbor_lists(xs.ctypes.data, 1000, 16, eps, ctypes.byref(o), off2.ctypes.data,
                                nb.ctypes.data, total - 1, ctypes.byref(tot), None)
    assert rc == -3 and np.array_equal(off, off2)
