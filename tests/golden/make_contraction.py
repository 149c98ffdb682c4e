"""Generate tests/golden/contraction.f64 / contraction.json.

The reference's FP64 kernel (kernel_join.cu:186-189) accumulates
`acc += (p - c) * (p - c)` per coordinate.  Compiled by nvcc with its default
floating-point contraction, that is acc = fma(t, t, acc); without contraction
it is acc = acc + fl(t * t).  The two readings give different d2 in the last
bits, so they can disagree on `sqrt(d2) <= eps` for pairs that lie within a
few ulps of the radius.  Every other fixture here is built on exactly
representable sums, where both readings agree; this one is built from such
disagreeing pairs, so it tells the readings apart.

Construction (seeded, pure Python, no reference code): 64 pairs (a, b) in 18
dimensions, pair k at a = B_k + U[0,1)^18 with B_k = 8 x (the 7 low bits of k)
on the first 7 coordinates, and b = a + r u for a random unit vector u and r
within a few ulps of eps = 1 (threshold T = the largest double whose square
root is <= 1).  For each candidate both readings are evaluated exactly
(rational arithmetic, rounded once per operation as the hardware does); a
candidate is kept when its readings fall on different sides of T: the first
40 pairs are counted by the fma reading only, the other 24 by the mul-add
reading only.  Points of different pairs differ by more than 5 in some
coordinate, so no point has a neighbour besides its partner.  The JSON holds the per-point counts and
totals of both readings.

    python tests/golden/make_contraction.py
"""
import json
import math
import os
import sys
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
D = 18
EPS = 1.0
N_FMA_ONLY, N_MUL_ONLY = 40, 24


def threshold(eps):
    t = eps * eps
    while t > 0 and math.sqrt(t) > eps:
        t = math.nextafter(t, 0.0)
    while math.sqrt(math.nextafter(t, math.inf)) <= eps:
        t = math.nextafter(t, math.inf)
    return t


def fma_reading(a, b):
    acc = 0.0
    for x, y in zip(a, b):
        t = x - y
        acc = float(Fraction(t) * Fraction(t) + Fraction(acc))
    return acc


def mul_add_reading(a, b):
    acc = 0.0
    for x, y in zip(a, b):
        t = x - y
        acc = acc + t * t
    return acc


def main():
    T = threshold(EPS)
    rng = np.random.default_rng(20260101)
    fma_only, mul_only = [], []
    tries = 0
    for k in range(N_FMA_ONLY + N_MUL_ONLY):
        want_fma = k < N_FMA_ONLY
        base = np.zeros(D)
        base[:7] = 8.0 * ((k >> np.arange(7)) & 1)
        while True:
            tries += 1
            if tries > 5_000_000:
                sys.exit("not enough discriminating pairs found")
            a = base + rng.random(D)
            u = rng.standard_normal(D)
            u /= np.linalg.norm(u)
            r = 1.0 + rng.uniform(-4, 4) * 2.0 ** -53
            b = a + r * u
            af, bf = [float(v) for v in a], [float(v) for v in b]
            f, m = fma_reading(af, bf) <= T, mul_add_reading(af, bf) <= T
            if want_fma and f and not m:
                fma_only.append((af, bf))
                break
            if not want_fma and m and not f:
                mul_only.append((af, bf))
                break
    pairs = fma_only + mul_only
    x = np.array([p for pair in pairs for p in pair], dtype="<f8")
    n = x.shape[0]
    x.tofile(os.path.join(HERE, "contraction.f64"))
    out = {"n": n, "d": D, "eps": EPS, "threshold": T}
    for name, fn in (("fma", fma_reading), ("mul_add", mul_add_reading)):
        counts = [1] * n
        for i in range(0, n, 2):
            if fn(list(x[i]), list(x[i + 1])) <= T:
                counts[i] += 1
                counts[i + 1] += 1
        out[name] = {"total": sum(counts), "counts": counts}
    with open(os.path.join(HERE, "contraction.json"), "w") as f:
        json.dump(out, f)
    print(f"{n} points, totals: fma {out['fma']['total']}, mul_add {out['mul_add']['total']} "
          f"({tries} candidate pairs)")


if __name__ == "__main__":
    main()
