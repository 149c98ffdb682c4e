"""CPU: the decision rule of the FP16 first pass of the band recheck (after
the FP8 screen), emulated and checked against exact distances.

Each row carries FP32 coordinates zf within `rad` of the exact point z (the
centring bound) and an FP16 copy zh = fp16(zf) with its own radius
radh = rad + |zh - zf| (the packer's sum of squares rounded up, then an FP32
square root rounded up).  The kernel forms S = sum (zh_i - zh_j)^2 in FP32 and
decides

    in   if  S + abs <= (sqrt(T_lo) - radh_i - radh_j)^2 (1 - c32)
    out  if  S - abs >  (sqrt(T_hi) + radh_i + radh_j)^2 (1 + c32)

with c32 = (d + 8) 2^-24 1.01.  Here z is drawn exactly (rationals), zf
within rad of it, and every decision the rule makes is compared with the
exact |z_i - z_j|^2 against T (T_lo = T_hi = T: no oracle rounding band)."""
import math
from fractions import Fraction

import numpy as np


def f32(x):
    return np.float32(x)


def sum_sq_f32(a, b):
    """Sequential FP32 sum of squared differences (the kernel's per-lane
    chains and tree are another order within the same (d + 8) bound)."""
    s = np.float32(0.0)
    for x, y in zip(a, b):
        t = np.float32(x) - np.float32(y)
        s = np.float32(s + np.float32(t * t))
    return s


def radius_up(err32):
    """sqrt of an FP32 sum of squares, both rounded up (in FP64, then one
    ulp up in FP32: an upper bound)."""
    e = math.fsum(float(v) * float(v) for v in err32)
    r = np.float32(math.sqrt(e) * (1 + 1e-6))
    return np.nextafter(r, np.float32(np.inf))


def decide(S, radh_i, radh_j, T, d):
    c32 = (d + 8) * 2.0 ** -24 * 1.01
    absd = (d + 8) * 2.0 ** -148
    rr = float(radh_i) + float(radh_j)
    lo = math.sqrt(T) - rr
    if lo >= 0 and float(S) + absd <= lo * lo * (1 - c32):
        return 1
    hi = math.sqrt(T) + rr
    if float(S) - absd > hi * hi * (1 + c32):
        return 0
    return -1


def test_fp16_first_pass_never_contradicts_exact_distance():
    rng = np.random.default_rng(17)
    decided = far = 0
    for d in (96, 256):
        for trial in range(60):
            # two exact points near the sphere, some pairs near the threshold
            zi = rng.uniform(-1, 1, d) / math.sqrt(d)
            zj = zi + rng.normal(0, 1, d) * rng.choice([0.02, 0.05, 0.1]) / math.sqrt(d)
            exact_i = [Fraction(float(v)) for v in zi]
            exact_j = [Fraction(float(v)) for v in zj]
            D = sum((a - b) ** 2 for a, b in zip(exact_i, exact_j))
            factor = float(rng.choice([0.8, 0.98, 0.995, 1.0, 1.005, 1.02, 1.25]))
            T = float(D) * factor
            # FP32 copies within rad of the exact points (the centring bound)
            zf_i = (zi + rng.normal(0, 1e-8, d)).astype(np.float32)
            zf_j = (zj + rng.normal(0, 1e-8, d)).astype(np.float32)
            rad_i = radius_up([Fraction(float(a)) - b for a, b in zip(zf_i, exact_i)])
            rad_j = radius_up([Fraction(float(a)) - b for a, b in zip(zf_j, exact_j)])
            # FP16 copies and their radii
            zh_i, zh_j = zf_i.astype(np.float16), zf_j.astype(np.float16)
            eh_i = np.float32(radius_up(zf_i.astype(np.float64) - zh_i.astype(np.float64)))
            eh_j = np.float32(radius_up(zf_j.astype(np.float64) - zh_j.astype(np.float64)))
            radh_i = np.nextafter(np.float32(rad_i + eh_i), np.float32(np.inf))
            radh_j = np.nextafter(np.float32(rad_j + eh_j), np.float32(np.inf))
            S = sum_sq_f32(zh_i.astype(np.float32), zh_j.astype(np.float32))
            dec = decide(S, radh_i, radh_j, T, d)
            if dec == 1:
                assert D <= Fraction(T), (d, trial)
            elif dec == 0:
                assert D > Fraction(T), (d, trial)
            if factor in (0.8, 1.25):
                far += 1
                decided += dec >= 0
    assert decided == far > 0  # pairs 20% off the threshold are always decided
