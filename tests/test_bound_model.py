"""CPU: the bookkeeping of the tensor-core accumulation bound of the 16-bit
screens (api.cu: screen_params, ejoin_internal.cuh: acc_margin2).

The Gram kernel issues its MMAs in order of magnitude: per K-slab the hi*lo
and lo*hi products first, then hi*hi, and the aug step (-alpha_i - alpha_j)
last.  The screen charges each MMA instruction of K_t products with
K_t 2^-22 times everything accumulated up to its end, plus 16 2^-22 of the
total, which for the BF16 hi+lo split gives

    |err| <= 2^-22 [128 L_ij + c_h a_i a_j + 32 (|alpha_i| + |alpha_j|)],
    c_h = 96 + 192 (slabs - 1),

split per row with a_i a_j <= (a_i^2 + a_j^2) / 2 and
L_ij <= 2^-9 (a_i^2 + a_j^2) / 2 + 2^9 (l_i^2 + l_j^2) / 2.

Here the accumulation is emulated in that order with every single product
added by a truncating FP32 addition (round toward zero, 24-bit significand):
a model whose error is at most half of what the bound charges per
instruction.  The test checks that the emulated error stays within the bound
on random and adversarial rows, and that the per-row split never undercuts the
pair bound.  (The GPU probes in test_gpu_probe.py measure the hardware against
the same model.)"""
import math
from fractions import Fraction

import numpy as np

U22 = 2.0 ** -22


def bf16(x):
    """Round float64 values to BF16 (nearest even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    out = (((b + r) >> 16) << 16).astype(np.uint32).view(np.float32)
    return out.astype(np.float64)


def trunc24(v):
    """FP32 rounding toward zero of an exact rational value (24-bit
    significand)."""
    if v == 0:
        return Fraction(0)
    a = abs(v)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    while Fraction(2) ** e > a:
        e -= 1
    while Fraction(2) ** (e + 1) <= a:
        e += 1
    ulp = Fraction(2) ** (e - 23)
    q = (a / ulp).numerator // (a / ulp).denominator
    return q * ulp if v > 0 else -q * ulp


def split_row(z):
    hi = bf16(z)
    lo = bf16(z - hi)
    return hi, lo


def alpha_pieces(alpha):
    a0 = float(bf16(alpha))
    a1 = float(bf16(alpha - a0))
    a2 = float(bf16(alpha - a0 - a1))
    return [a0, a1, a2]


def emulate(hi_i, lo_i, hi_j, lo_j, al_i, al_j):
    """Accumulate in the kernel's order, one truncating addition per product;
    returns (computed, exact)."""
    dp = hi_i.size
    prods = []
    for s in range(dp // 64):
        for kk in range(4):
            k = slice(64 * s + 16 * kk, 64 * s + 16 * kk + 16)
            prods.append(hi_i[k] * lo_j[k])   # hi*lo
            prods.append(lo_i[k] * hi_j[k])   # lo*hi
        for kk in range(4):
            k = slice(64 * s + 16 * kk, 64 * s + 16 * kk + 16)
            prods.append(hi_i[k] * hi_j[k])   # hi*hi
    prods.append(np.array([-p for p in al_i] + [-p for p in al_j]))  # aug step
    S = Fraction(0)
    exact = Fraction(0)
    for group in prods:
        for p in group:
            fp = Fraction(float(p))  # a product of two BF16 values is exact in FP64
            S = trunc24(S + fp)
            exact += fp
    return S, exact


def pair_bound(hi_i, lo_i, hi_j, lo_j, al_i, al_j):
    slabs = hi_i.size // 64
    c_h = 96 + 192 * (slabs - 1)
    L = float(np.abs(hi_i) @ np.abs(lo_j) + np.abs(lo_i) @ np.abs(hi_j))
    a_i = math.sqrt(float(((np.abs(hi_i) + np.abs(lo_i)) ** 2).sum()))
    a_j = math.sqrt(float(((np.abs(hi_j) + np.abs(lo_j)) ** 2).sum()))
    al = sum(abs(p) for p in al_i) + sum(abs(p) for p in al_j)
    return U22 * (128 * L + c_h * a_i * a_j + 32 * al), a_i, a_j


def row_share(hi, lo, al, slabs):
    """e_i of the per-row split (half of acc_margin2 plus the alpha term)."""
    c_h = 96 + 192 * (slabs - 1)
    a2 = float(((np.abs(hi) + np.abs(lo)) ** 2).sum())
    l2 = float((lo ** 2).sum())
    m2 = c_h * U22 * a2 + 128 * U22 * (a2 / 512.0 + 512.0 * l2)
    return 0.5 * m2 + 32 * U22 * sum(abs(p) for p in al)


def check(z_i, z_j):
    hi_i, lo_i = split_row(z_i)
    hi_j, lo_j = split_row(z_j)
    n_i = float(((hi_i + lo_i) ** 2).sum())
    n_j = float(((hi_j + lo_j) ** 2).sum())
    al_i, al_j = alpha_pieces(n_i / 2), alpha_pieces(n_j / 2)
    S, exact = emulate(hi_i, lo_i, hi_j, lo_j, al_i, al_j)
    bound, _, _ = pair_bound(hi_i, lo_i, hi_j, lo_j, al_i, al_j)
    err = float(abs(S - exact))
    assert err <= bound / 2, (err, bound)
    slabs = hi_i.size // 64
    split = row_share(hi_i, lo_i, al_i, slabs) + row_share(hi_j, lo_j, al_j, slabs)
    assert split >= bound * (1 - 1e-12), (split, bound)
    return err / bound


def test_bound_random_rows():
    rng = np.random.default_rng(3)
    worst = 0.0
    for d in (64, 128):
        for _ in range(40):
            z = rng.uniform(-1, 1, size=(2, d))
            worst = max(worst, check(z[0], z[1]))
    assert worst < 0.5


def test_bound_adversarial_rows():
    """Same-sign rows (every product adds), near neighbours (the aug step
    cancels the data part: the pairs the band is about), one dominant
    coordinate, and magnitudes spread over many binades."""
    rng = np.random.default_rng(5)
    for d in (64, 128):
        a = np.abs(rng.uniform(0.5, 1.0, size=d))
        check(a, a * (1 + 1e-3 * rng.standard_normal(d)))
        b = np.full(d, 1e-3)
        b[0] = 1.0
        check(b, b[::-1].copy())
        c = np.abs(rng.standard_normal(d)) * 2.0 ** rng.integers(-20, 0, size=d)
        check(c, c * 0.999)
