"""Generate the contraction fixtures: tests/golden/contraction[_d<D>].f64/.json.

The reference's FP64 kernel (kernel_join.cu:186-189) accumulates
`acc += (p - c) * (p - c)` per coordinate, from acc = 0.  The compiler decides
how the products are rounded, and three readings are plausible:

  fma      acc = fma(t_j, t_j, acc) for every j (contraction of every step)
  first    acc = fma(t_0, t_0, fl(t_1 * t_1)), then fma(t_j, t_j, acc) for
           j >= 2 (`0 + t_0 * t_0` folded into the bare product, which is then
           fused into the second step instead of the second product)
  mul_add  acc = acc + fl(t_j * t_j) (no contraction)

They give different d2 in the last bits, so they can disagree on
`sqrt(d2) <= eps` for pairs that lie within a few ulps of the radius.  Every
other fixture here is built on exactly representable sums, where all readings
agree; these are built from disagreeing pairs, so they tell the readings
apart (the GPU tests run the reference's own compiled kernel on them).

Construction (seeded, pure Python, no reference code), for each dimension D:
pairs (a, b) in D dimensions, pair k at a = B_k + U[0,1)^D with
B_k = 8 x (the 7 low bits of k) on the first 7 coordinates, and b = a + r u
for a random unit vector u and r within a few ulps of eps = 1 (threshold
T = the largest double whose square root is <= 1).  Each candidate is
evaluated exactly in every reading (rational arithmetic, rounded once per
operation as the hardware does) and kept when its readings do not all agree:
for each ordered pair of readings (X, Y), WANT[(X, Y)] pairs that X counts and
Y does not -- unequal numbers, so that the three readings also give three
different totals (the reference's kernel reports only a total).  Points of
different pairs differ by more than 5 in some coordinate, so no point has a
neighbour besides its partner.  The JSON holds the per-point counts and totals
of every reading.

    python tests/golden/make_contraction.py
"""
import json
import math
import os
import sys
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
EPS = 1.0
WANT = {("fma", "first"): 12, ("first", "fma"): 3, ("fma", "mul_add"): 9, ("mul_add", "fma"): 2,
        ("first", "mul_add"): 6, ("mul_add", "first"): 1}


def threshold(eps):
    t = eps * eps
    while t > 0 and math.sqrt(t) > eps:
        t = math.nextafter(t, 0.0)
    while math.sqrt(math.nextafter(t, math.inf)) <= eps:
        t = math.nextafter(t, math.inf)
    return t


def _fma(x, y, z):
    return float(Fraction(x) * Fraction(y) + Fraction(z))


def fma_reading(a, b):
    acc = 0.0
    for x, y in zip(a, b):
        t = x - y
        acc = _fma(t, t, acc)
    return acc


def first_reading(a, b):
    t = [x - y for x, y in zip(a, b)]
    if len(t) == 1:
        return t[0] * t[0]
    acc = _fma(t[0], t[0], t[1] * t[1])
    for v in t[2:]:
        acc = _fma(v, v, acc)
    return acc


def mul_add_reading(a, b):
    acc = 0.0
    for x, y in zip(a, b):
        t = x - y
        acc = acc + t * t
    return acc


READINGS = {"fma": fma_reading, "first": first_reading, "mul_add": mul_add_reading}


def make(d, name, seed):
    T = threshold(EPS)
    rng = np.random.default_rng(seed)
    want = dict(WANT)
    pairs = []
    tries = 0
    while any(want.values()):
        tries += 1
        if tries > 20_000_000:
            sys.exit(f"d={d}: not enough discriminating pairs ({want})")
        k = len(pairs)
        base = np.zeros(d)
        base[:7] = 8.0 * ((k >> np.arange(7)) & 1)
        a = base + rng.random(d)
        u = rng.standard_normal(d)
        u /= np.linalg.norm(u)
        b = a + (1.0 + rng.uniform(-4, 4) * 2.0 ** -53) * u
        af, bf = [float(v) for v in a], [float(v) for v in b]
        if abs(mul_add_reading(af, bf) - T) > 2.0 ** -46:
            continue  # farther than 64 ulps from T: every reading agrees
        inside = {r: fn(af, bf) <= T for r, fn in READINGS.items()}
        for (x, y), left in want.items():
            if left and inside[x] and not inside[y]:
                want[(x, y)] -= 1
                pairs.append((af, bf))
                break
    x = np.array([p for pair in pairs for p in pair], dtype="<f8")
    n = x.shape[0]
    totals = set()
    x.tofile(os.path.join(HERE, name + ".f64"))
    out = {"n": n, "d": d, "eps": EPS, "threshold": T}
    for r, fn in READINGS.items():
        counts = [1] * n
        for i in range(0, n, 2):
            if fn(list(x[i]), list(x[i + 1])) <= T:
                counts[i] += 1
                counts[i + 1] += 1
        out[r] = {"total": sum(counts), "counts": counts}
        totals.add(sum(counts))
    if len(totals) != len(READINGS):
        sys.exit(f"{name}: totals do not tell the readings apart; change the seed")
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(out, f)
    print(f"{name}: {n} points, totals " +
          ", ".join(f"{r} {out[r]['total']}" for r in READINGS) + f" ({tries} candidates)")


def main():
    make(18, "contraction", 20260101)
    make(64, "contraction_d64", 20260164)
    make(128, "contraction_d128", 20260228)


if __name__ == "__main__":
    main()
