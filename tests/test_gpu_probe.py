"""GPU: the tcgen05 building blocks (descriptors, TMA swizzle, tensor-memory
layout, FP32 accumulation) through a one-tile probe, against numpy."""
import ctypes
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

PROBE = os.path.join(ROOT, "tests", "csrc", "libumma_probe.so")


def f32_to_bf16_bits(x):
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) >> 16).astype(np.uint16)


def bf16_bits_to_f64(b):
    return (b.astype(np.uint32) << 16).view(np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def probe(ej):
    lib = ctypes.CDLL(PROBE)
    lib.umma_probe_gram.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint)]
    lib.umma_probe_gram.restype = ctypes.c_int

    def run(A, B, nslab, fmt, mode):
        D = np.zeros((128, 128), dtype=np.float32)
        to = ctypes.c_uint(0)
        rc = lib.umma_probe_gram(A.ctypes.data, B.ctypes.data, nslab, fmt, mode, D.ctypes.data,
                                 ctypes.byref(to))
        assert rc == 0, (rc, to.value)
        return D.astype(np.float64)

    return run


@pytest.mark.parametrize("nslab", [1, 2, 4])
@pytest.mark.parametrize("fmt", [0, 1])
def test_probe_gram_tile(probe, nslab, fmt):
    rng = np.random.default_rng(nslab * 10 + fmt)
    K = 64 * nslab
    a = rng.standard_normal((128, K)).astype(np.float32)
    b = rng.standard_normal((128, K)).astype(np.float32)
    if fmt == 1:
        A, B = f32_to_bf16_bits(a), f32_to_bf16_bits(b)
        af, bf = bf16_bits_to_f64(A), bf16_bits_to_f64(B)
    else:
        A, B = a.astype(np.float16).view(np.uint16), b.astype(np.float16).view(np.uint16)
        af, bf = a.astype(np.float16).astype(np.float64), b.astype(np.float16).astype(np.float64)
    D = probe(np.ascontiguousarray(A), np.ascontiguousarray(B), nslab, fmt, 0)
    ref = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    err = np.abs(D - ref)
    assert np.all(err <= 2.0 ** -20 * scale + 1e-30), float((err / scale).max())


def test_probe_aug_offset(probe):
    """A at byte 0, B at byte 32 of the same swizzled slab (the aug MMA)."""
    rng = np.random.default_rng(7)
    a = rng.standard_normal((128, 64)).astype(np.float32)
    b = rng.standard_normal((128, 64)).astype(np.float32)
    A, B = f32_to_bf16_bits(a), f32_to_bf16_bits(b)
    af, bf = bf16_bits_to_f64(A), bf16_bits_to_f64(B)
    D = probe(A, B, 1, 1, 1)
    ref = af[:, :16] @ bf[:, 16:32].T
    assert np.allclose(D, ref, rtol=1e-5, atol=1e-5)


def test_probe_accumulation_error_within_bound(probe):
    """Adversarial sums (one large product, many small ones of mixed sign):
    the observed FP32 accumulation error stays a factor >= 4 inside the bound
    the screen uses, c_acc = (K + 16) 2^-22 relative to sum |products|."""
    rng = np.random.default_rng(11)
    K = 256
    a = rng.standard_normal((128, K)).astype(np.float32)
    b = rng.standard_normal((128, K)).astype(np.float32)
    a[:, 0] *= 2.0 ** 12
    b[:, 0] *= 2.0 ** 12
    a[:, 1::2] *= 2.0 ** -6
    A, B = f32_to_bf16_bits(a), f32_to_bf16_bits(b)
    af, bf = bf16_bits_to_f64(A), bf16_bits_to_f64(B)
    D = probe(A, B, 4, 1, 0)
    ref = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    rel = (np.abs(D - ref) / scale).max()
    bound = (K + 16) * 2.0 ** -22
    print(f"max accumulation error / sum|p| = {rel:.3e} (bound {bound:.3e})")
    assert rel * 4 <= bound


def prefix_model_bound(af, bf, kstep):
    """The screen's per-instruction accumulation model: instruction t (kstep
    products, issued in K order) errs by at most kstep 2^-22 times the sum of
    |products| accumulated up to its end, plus 16 2^-22 of the total."""
    K = af.shape[1]
    prefix = np.zeros((af.shape[0], bf.shape[0]))
    total = np.zeros_like(prefix)
    for t in range(K // kstep):
        sl = slice(t * kstep, (t + 1) * kstep)
        prefix += np.abs(af[:, sl]) @ np.abs(bf[:, sl]).T
        total += kstep * prefix
    return (total + 16 * prefix) * 2.0 ** -22


def magnitude_pattern(rng, pattern, K):
    """Per-coordinate exponent offsets for the prefix-model probes."""
    s = np.zeros(K)
    if pattern == "small_then_large":    # the split screen's order: lo products first
        s[: K // 2] = -9
    elif pattern == "large_last":        # one big instruction at the end (the aug step)
        s[: K - 16] = -10
    elif pattern == "ramp":              # magnitudes growing along K
        s = np.floor(np.linspace(-14, 0, K))
    elif pattern == "large_first":
        s[16:] = -8
    return 2.0 ** s


@pytest.mark.parametrize("pattern", ["small_then_large", "large_last", "ramp", "large_first"])
@pytest.mark.parametrize("fmt", [0, 1])
def test_probe_accumulation_prefix_model(probe, fmt, pattern):
    """The bound the screen's margins use (api.cu screen_params): every
    observed error, with small products issued before large ones and with
    signs that cancel, stays a factor >= 4 inside the per-instruction model."""
    rng = np.random.default_rng(100 + fmt * 10 + len(pattern))
    K = 256
    m = magnitude_pattern(rng, pattern, K)
    a = (rng.standard_normal((128, K)) * m).astype(np.float32)
    b = (rng.standard_normal((128, K)) * m).astype(np.float32)
    # rows 64..: b_j = -a_j on the last 16 coordinates, so the last
    # instruction of pair (j, j) only subtracts
    b[64:, K - 16:] = -a[64:, K - 16:]
    if fmt == 1:
        A, B = f32_to_bf16_bits(a), f32_to_bf16_bits(b)
        af, bf = bf16_bits_to_f64(A), bf16_bits_to_f64(B)
    else:
        # the screen stores no subnormal operand (the packer flushes them)
        a16, b16 = a.astype(np.float16), b.astype(np.float16)
        a16[np.abs(a16) < 2.0 ** -14] = 0
        b16[np.abs(b16) < 2.0 ** -14] = 0
        A, B = a16.view(np.uint16), b16.view(np.uint16)
        af, bf = a16.astype(np.float64), b16.astype(np.float64)
    D = probe(np.ascontiguousarray(A), np.ascontiguousarray(B), K // 64, fmt, 0)
    err = np.abs(D - af @ bf.T)
    bound = prefix_model_bound(af, bf, 16)
    worst = float((err / bound).max())
    print(f"{pattern} fmt {fmt}: max error / model bound = {worst:.3e}")
    assert worst * 4 <= 1.0


@pytest.mark.parametrize("pattern", ["small_then_large", "large_last", "ramp"])
def test_probe_fp8_accumulation_prefix_model(probe, pattern):
    rng = np.random.default_rng(200 + len(pattern))
    K = 256
    lo_hi = {"small_then_large": [(-6, -4)] * 4 + [(2, 5)] * 4,
             "large_last": [(-6, -5)] * 7 + [(5, 7)],
             "ramp": [(-6 + i, -5 + i) for i in range(8)]}[pattern]
    A = np.concatenate([random_e4m3(rng, (128, 32), l, h) for l, h in lo_hi], axis=1)
    B = np.concatenate([random_e4m3(rng, (128, 32), l, h) for l, h in lo_hi], axis=1)
    af, bf = e4m3_decode(A), e4m3_decode(B)
    D = probe(np.ascontiguousarray(A), np.ascontiguousarray(B), K // 128, 2, 0)
    err = np.abs(D - af @ bf.T)
    bound = prefix_model_bound(af, bf, 32)
    worst = float((err / bound).max())
    print(f"FP8 {pattern}: max error / model bound = {worst:.3e}")
    assert worst * 4 <= 1.0


@pytest.mark.parametrize("fmt", [0, 1])
def test_probe_sw32_aug_tiles(probe, fmt):
    """The aug operands: [rows][32] 16-bit arrays, A = columns 0..15 and
    B = columns 16..31, loaded as 32-byte-swizzled boxes (one K = 16 step)."""
    rng = np.random.default_rng(40 + fmt)
    a = rng.standard_normal((128, 64)).astype(np.float32)
    b = rng.standard_normal((128, 64)).astype(np.float32)
    if fmt == 1:
        A, B = f32_to_bf16_bits(a), f32_to_bf16_bits(b)
        af, bf = bf16_bits_to_f64(A), bf16_bits_to_f64(B)
    else:
        A, B = a.astype(np.float16).view(np.uint16), b.astype(np.float16).view(np.uint16)
        af, bf = a.astype(np.float16).astype(np.float64), b.astype(np.float16).astype(np.float64)
    # the probe reads the first 128 x 32 elements of each buffer as [128][32]
    A32 = np.ascontiguousarray(A[:, :32])
    B32 = np.ascontiguousarray(B[:, :32])
    Ap = np.zeros((128, 64), dtype=np.uint16)
    Bp = np.zeros((128, 64), dtype=np.uint16)
    Ap.reshape(-1)[: 128 * 32] = A32.reshape(-1)
    Bp.reshape(-1)[: 128 * 32] = B32.reshape(-1)
    D = probe(Ap, Bp, 1, fmt, 2)
    ref = af[:, :16] @ bf[:, 16:32].T
    assert np.allclose(D, ref, rtol=1e-5, atol=1e-5)


def e4m3_decode(b):
    b = b.astype(np.int64)
    s = np.where(b & 0x80, -1.0, 1.0)
    e = (b >> 3) & 0xF
    m = b & 0x7
    val = np.where(e == 0, m / 8.0 * 2.0 ** -6, (1 + m / 8.0) * 2.0 ** (e - 7))
    return s * val


def random_e4m3(rng, shape, lo_exp=-6, hi_exp=6):
    """Random finite, normal E4M3 codes with exponents in [lo_exp, hi_exp]
    (hi_exp <= 7: exponent code 15 with mantissa 7 is NaN)."""
    assert hi_exp <= 7
    e = rng.integers(lo_exp + 7, hi_exp + 8, shape)
    m = rng.integers(0, 8, shape)
    s = rng.integers(0, 2, shape)
    return ((s << 7) | (e << 3) | m).astype(np.uint8)


@pytest.mark.parametrize("nslab", [1, 2])
def test_probe_fp8_gram_tile(probe, nslab):
    rng = np.random.default_rng(70 + nslab)
    K = 128 * nslab
    A = random_e4m3(rng, (128, K))
    B = random_e4m3(rng, (128, K))
    af, bf = e4m3_decode(A), e4m3_decode(B)
    D = probe(A, B, nslab, 2, 0)
    ref = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    rel = (np.abs(D - ref) / scale).max()
    bound = (K + 16) * 2.0 ** -22
    print(f"FP8: max accumulation error / sum|p| = {rel:.3e} (bound {bound:.3e})")
    assert rel * 4 <= bound


def test_probe_fp8_accumulation_adversarial(probe):
    """One large product followed by many small ones of mixed sign: the FP8
    kind keeps FP32-class accumulation precision (the screen's bound holds)."""
    rng = np.random.default_rng(77)
    K = 256
    A = random_e4m3(rng, (128, K), -6, -3)
    B = random_e4m3(rng, (128, K), -6, -3)
    A[:, 0] = random_e4m3(rng, (128,), 6, 7)
    B[:, 0] = random_e4m3(rng, (128,), 6, 7)
    af, bf = e4m3_decode(A), e4m3_decode(B)
    D = probe(A, B, 2, 2, 0)
    ref = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    rel = (np.abs(D - ref) / scale).max()
    bound = (K + 16) * 2.0 ** -22
    print(f"FP8 adversarial: max error / sum|p| = {rel:.3e} (bound {bound:.3e})")
    assert rel * 4 <= bound
