"""CPU: the learned projection's loss/gradient restatement is itself right
(analytic gradient vs central finite differences)."""
import numpy as np

from oracle import learned


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    M, k, d = 400, 4, 10
    V = rng.standard_normal((M, d))
    P = rng.standard_normal((k, d)) * 0.2
    tgt = np.where(rng.random(M) < 0.8, np.abs(rng.standard_normal(M)) * 3 + 0.5, 0.0)
    loss, G = learned.loss_and_grad(V, tgt, P)
    assert loss > 0
    h = 1e-6
    num = np.zeros_like(P)
    for a in range(k):
        for c in range(d):
            Pp, Pm = P.copy(), P.copy()
            Pp[a, c] += h
            Pm[a, c] -= h
            num[a, c] = (learned.loss_only(V, tgt, Pp) - learned.loss_only(V, tgt, Pm)) / (2 * h)
    assert np.allclose(num, G, rtol=1e-5, atol=1e-8)
