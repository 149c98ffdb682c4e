"""GPU: exact joins at the benchmark sizes.

The oracle cannot run the full O(N^2 d) join on the host, so each case checks
(i) the per-point counts of seeded query rows against the oracle (rows x all
N) and against the GPU FP64 direct kernel (more rows), and (ii) properties
that hold at any size: counts sum to the total; the predicate is symmetric,
so total - (finite rows counting themselves) is even; every finite row counts
itself (eps >= 0); pruned and unpruned joins agree exactly.
"""
import numpy as np
import pytest

from tensor_bf_main_gb300 import datagen

pytestmark = pytest.mark.gpu


def check(ej, oracle_mod, x, eps, counts, total, nrows_oracle=16, nrows_gpu=256, seed=0):
    n = x.shape[0]
    assert counts.shape == (n,)
    assert int(counts.astype(np.int64).sum()) == total
    finite = np.isfinite(x).all(1)
    assert np.all(counts[finite] >= 1)
    assert (total - int(finite.sum())) % 2 == 0
    rng = np.random.default_rng(seed)
    rows = rng.choice(n, nrows_oracle, replace=False)
    assert np.array_equal(counts[rows], oracle_mod.query_counts(x, eps, rows))
    rows = rng.choice(n, nrows_gpu, replace=False)
    assert np.array_equal(counts[rows], ej.query_counts(x, eps, rows))


def test_c4_full_learned(ej, oracle_mod):
    x = datagen.generate("c4")
    eps = datagen.EPS["c4"]
    counts, total, st = ej.self_join(x, eps, precision="bf16_split", proj_k=8)
    check(ej, oracle_mod, x, eps, counts, total)
    assert st["tile_pairs_run"] < 0.02 * st["tile_pairs_total"]
    c2, t2, _ = ej.self_join(x, eps, precision="fp16", proj_k=8, order=1)
    assert t2 == total and np.array_equal(c2, counts)


def test_c2_full_fp16(ej, oracle_mod):
    x = datagen.generate("c2")
    eps = datagen.EPS["c2"]
    counts, total, st = ej.self_join(x, eps, precision="fp16")
    check(ej, oracle_mod, x, eps, counts, total)


def test_c3_shape_centring_and_sweep(ej, oracle_mod):
    """c3 distribution (offset +10, rotated power-law spectrum) at N = 500,000."""
    x = datagen.generate("c3", n=500_000)
    for target in (16, 1024):
        eps = datagen.calibrate_eps(x, target, nq=64)
        counts, total, st = ej.self_join(x, eps, precision="bf16_split")
        check(ej, oracle_mod, x, eps, counts, total, nrows_oracle=8)
        c16, t16, _ = ej.self_join(x, eps, precision="bf16")
        assert t16 == total and np.array_equal(c16, counts)


def test_c5_shape_fp8(ej, oracle_mod):
    """c5 distribution (unit sphere, d = 1024) at N = 100,000 with FP8 operands."""
    x = datagen.generate("c5", n=100_000)
    eps = datagen.EPS["c5"]
    counts, total, st = ej.self_join(x, eps, precision="fp8_e4m3")
    check(ej, oracle_mod, x, eps, counts, total, nrows_oracle=8, nrows_gpu=128)
    cb, tb, _ = ej.self_join(x, eps, precision="bf16", proj_k=16, train_steps=20)
    assert tb == total and np.array_equal(cb, counts)


def test_pinned_host_input_streams_copy(ej, oracle_mod):
    """Pinned host rows (>= 64 MB) are copied in chunks by the centring pass;
    counts and lists equal those of pageable and device-resident input."""
    torch = pytest.importorskip("torch")
    x = datagen.generate("c4", n=500_000)
    eps = datagen.EPS["c4"]
    xp = torch.from_numpy(x).pin_memory()
    c_pin, t_pin, _ = ej.self_join(xp, eps, precision="bf16_split", proj_k=8)
    c_np, t_np, _ = ej.self_join(x, eps, precision="bf16_split", proj_k=8)
    c_dev, t_dev, _ = ej.self_join(torch.from_numpy(x).cuda(), eps, precision="bf16_split",
                                   proj_k=8)
    assert t_pin == t_np == t_dev
    assert np.array_equal(c_pin, c_np) and np.array_equal(c_pin, c_dev)
    check(ej, oracle_mod, x, eps, c_pin, t_pin, nrows_oracle=8)
    c16, t16, _ = ej.self_join(xp, eps, precision="fp16")
    assert t16 == t_pin and np.array_equal(c16, c_pin)
    off_p, nb_p, _ = ej.neighbor_lists(xp, eps, precision="bf16_split", proj_k=8)
    off_n, nb_n, _ = ej.neighbor_lists(x, eps, precision="bf16_split", proj_k=8)
    assert np.array_equal(off_p, off_n) and np.array_equal(nb_p, nb_n)
    assert int(off_p[-1]) == t_pin
