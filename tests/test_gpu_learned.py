"""GPU: the learned contractive projection -- training kernels against the
CPU restatement, the certified spectral norm, and pruned joins whose counts
equal the plain join's exactly; plus what training gains over no training."""
import ctypes

import numpy as np
import pytest

from oracle import learned

pytestmark = pytest.mark.gpu


def latent_data(n, seed, d=64, k=32, m=8, sigma=0.02, noise=0.01):
    """c4-shaped data: clusters on an m-dim latent embedded in R^d."""
    rng = np.random.default_rng(seed)
    c = rng.random((k, m))
    E, _ = np.linalg.qr(rng.standard_normal((d, m)))
    z = c[rng.integers(0, k, n)] + sigma * rng.standard_normal((n, m))
    return z @ E.T + noise * rng.standard_normal((n, d))


def eps_for_mean(x, mean, seed=0):
    rng = np.random.default_rng(seed)
    n = x.shape[0]
    i, j = rng.integers(0, n, 20000), rng.integers(0, n, 20000)
    return float(np.quantile(np.sqrt(((x[i] - x[j]) ** 2).sum(1)), mean / n))


@pytest.mark.parametrize("k,d", [(8, 64), (16, 1024), (3, 17)])
def test_training_gradient_matches_cpu(ej, k, d):
    lib = ej.load_library()
    rng = np.random.default_rng(k + d)
    M = 3000
    V = rng.standard_normal((M, d)).astype(np.float32)
    P = (rng.standard_normal((k, d)) / np.sqrt(d)).astype(np.float32)
    r = np.sqrt(((V.astype(np.float64) @ P.T.astype(np.float64)) ** 2).sum(1))
    tgt = np.where(rng.random(M) < 0.8, r * rng.uniform(0.5, 2.0, M), 0.0).astype(np.float32)
    G = np.zeros((k, d), dtype=np.float32)
    loss = ctypes.c_float(0)
    rc = lib.ejoin_testing_projection_grad(V.ctypes.data, tgt.ctypes.data, M, P.ctypes.data, k, d,
                                           G.ctypes.data, ctypes.byref(loss))
    assert rc == 0
    ref_loss, ref_G = learned.loss_and_grad(V, tgt, P)
    assert abs(loss.value - ref_loss) <= 1e-4 * max(1.0, ref_loss)
    scale = np.abs(ref_G).max()
    assert np.allclose(G, ref_G, rtol=2e-3, atol=2e-4 * scale)


def test_renormalisation_bounds_spectral_norm(ej):
    lib = ej.load_library()
    rng = np.random.default_rng(3)
    P = (rng.standard_normal((8, 64)) * 0.5).astype(np.float32)
    s0 = learned.spectral_norm(P)
    est = ctypes.c_float(0)
    assert lib.ejoin_testing_renormalise(P.ctypes.data, 8, 64, ctypes.byref(est)) == 0
    assert est.value >= s0  # inflated power-iteration estimate
    assert learned.spectral_norm(P) <= 1.0


def test_trained_projection_is_certified_contractive(ej):
    x = latent_data(60000, 1)
    eps = eps_for_mean(x, 30)
    P, sigma, st = ej.train_projection(x, eps, k=8, train_steps=120)
    exact = learned.spectral_norm(P)
    assert sigma >= exact
    assert sigma <= exact * (1 + 2e-3)
    assert sigma <= 1.05
    assert st["loss_last"] < st["loss_first"]  # the hinge loss decreased


@pytest.mark.parametrize("mode", ["bf16_split", "bf16", "fp16"])
def test_pruned_counts_equal_plain_join(ej, oracle_mod, mode):
    x = latent_data(80000, 2)
    eps = eps_for_mean(x, 40)
    plain, tp, sp = ej.self_join(x, eps, precision=mode)
    pruned, tq, sq = ej.self_join(x, eps, precision=mode, proj_k=8, train_steps=100)
    assert tp == tq
    assert np.array_equal(plain, pruned)
    assert sq["tile_pairs_run"] < sp["tile_pairs_run"]
    rows = np.random.default_rng(0).choice(x.shape[0], 24, replace=False)
    assert np.array_equal(pruned[rows], oracle_mod.query_counts(x, eps, rows))


def test_lead_order_and_reused_projection(ej):
    x = latent_data(50000, 3)
    eps = eps_for_mean(x, 30)
    plain, tp, _ = ej.self_join(x, eps, precision="bf16_split")
    lead, tl, _ = ej.self_join(x, eps, precision="bf16_split", proj_k=8, order=1, train_steps=60)
    assert np.array_equal(plain, lead)
    P, sigma, _ = ej.train_projection(x, eps, k=8, train_steps=60)
    c1, t1, s1 = ej.self_join(x, eps, precision="bf16_split", proj_k=8, projection=P)
    c2, t2, s2 = ej.self_join(x, eps, precision="bf16_split", proj_k=8, projection=P)
    assert np.array_equal(c1, plain) and np.array_equal(c2, plain)
    assert s1["tile_pairs_run"] == s2["tile_pairs_run"]
    assert abs(s1["sigma_cert"] - sigma) <= 1e-12 * sigma


def test_saved_projection_reused_from_file(ej, tmp_path):
    """A trained P saved to a projection file and loaded back prunes exactly
    the same tile pairs and gives the same exact counts."""
    x = latent_data(50000, 7)
    eps = eps_for_mean(x, 30)
    P, sigma, _ = ej.train_projection(x, eps, k=8, train_steps=40)
    path = str(tmp_path / "c.ejp")
    ej.save_projection(path, P, sigma)
    Q, sig2 = ej.load_projection(path)
    assert sig2 == sigma and np.array_equal(P, Q)
    c1, t1, s1 = ej.self_join(x, eps, precision="fp16", proj_k=8, projection=P)
    c2, t2, s2 = ej.self_join(x, eps, precision="fp16", proj_k=8, projection=Q)
    plain, tp, _ = ej.self_join(x, eps, precision="fp64_dmma")
    assert t1 == t2 == tp and np.array_equal(c1, c2) and np.array_equal(c1, plain)
    assert s1["tile_pairs_run"] == s2["tile_pairs_run"] < s1["tile_pairs_total"]


def test_training_gains_over_untrained_projection(ej):
    """What the trained network buys: tile pairs reaching the GEMM and time,
    trained P vs an untrained random contractive P vs no projection."""
    x = latent_data(200000, 4)
    eps = eps_for_mean(x, 40)
    rng = np.random.default_rng(5)
    R = rng.standard_normal((8, 64)).astype(np.float32)
    R /= np.float32(np.linalg.svd(R.astype(np.float64), compute_uv=False)[0] * 1.001)
    c0, t0, s0 = ej.self_join(x, eps, precision="bf16_split")
    cr, tr, sr = ej.self_join(x, eps, precision="bf16_split", proj_k=8, projection=R)
    ct, tt, st = ej.self_join(x, eps, precision="bf16_split", proj_k=8)
    assert t0 == tr == tt and np.array_equal(c0, ct) and np.array_equal(c0, cr)
    frac = lambda s: s["tile_pairs_run"] / s["tile_pairs_total"]
    print(f"tile pairs run: none {frac(s0):.4f}  untrained {frac(sr):.4f}  trained {frac(st):.4f}; "
          f"ms: none {s0['ms_total']:.1f} untrained {sr['ms_total']:.1f} trained {st['ms_total']:.1f} "
          f"(train {st['ms_train']:.1f})")
    assert frac(st) < frac(sr) < frac(s0) == 1.0


def test_learned_pipeline_is_reproducible(ej):
    """Fixed-point gradient accumulation makes training bit-reproducible: two
    runs prune exactly the same tile pairs and queue the same band."""
    x = latent_data(60000, 6)
    eps = eps_for_mean(x, 30)
    a, ta, sa = ej.self_join(x, eps, precision="bf16_split", proj_k=8, train_steps=80)
    b, tb, sb = ej.self_join(x, eps, precision="bf16_split", proj_k=8, train_steps=80)
    assert ta == tb and np.array_equal(a, b)
    assert sa["tile_pairs_run"] == sb["tile_pairs_run"]
    assert sa["band_pairs"] == sb["band_pairs"]
    assert sa["sigma_cert"] == sb["sigma_cert"]
