"""CPU oracle for the epsilon self-join -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
(``cpu_baseline`` and ``--impl reference``) may import this package.  It is
the oracle the CUDA path is compared with, never part of the product.

``oracle.c`` restates the reference's FP64 CUDA-core join
(kernel_join.cu:168-200) and its loader (dataset.cu:10-39); see the header of
that file for the exact arithmetic.  The small pure-Python/numpy functions
below restate the same predicate independently so the C oracle itself can be
cross-checked on small inputs.
"""
from __future__ import annotations

import ctypes
import math
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LOADER = os.path.join(HERE, "_ref", "ref_loader")


def build(force: bool = False) -> str:
    """Compile oracle.c (gcc, OpenMP, -ffp-contract=off) into liboracle.so."""
    src = os.path.join(HERE, "oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    flags = ["-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11"]
    if platform.machine() in ("x86_64", "AMD64"):
        # hardware fma only changes speed: fma() is correctly rounded either way
        flags.append("-mfma")
    tmp = LIB_PATH + ".tmp"
    subprocess.check_call(["gcc", *flags, src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_threshold.restype = ctypes.c_double
        L.oracle_threshold.argtypes = [ctypes.c_double]
        L.oracle_pair_d2.restype = ctypes.c_double
        L.oracle_pair_d2.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32]
        L.oracle_query_counts.restype = ctypes.c_int
        L.oracle_query_counts.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p,
                                          ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int]
        L.oracle_self_join.restype = ctypes.c_int
        L.oracle_self_join.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                       ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int]
        L.oracle_cross_counts.restype = ctypes.c_int
        L.oracle_cross_counts.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                          ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint64,
                                          ctypes.c_double, ctypes.c_void_p, ctypes.c_int]
        L.oracle_neighbor_lists.restype = ctypes.c_int
        L.oracle_neighbor_lists.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32,
                                            ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_int]
        L.oracle_import_dataset.restype = ctypes.c_int
        L.oracle_import_dataset.argtypes = [ctypes.c_char_p, ctypes.c_uint32,
                                            ctypes.POINTER(ctypes.c_void_p),
                                            ctypes.POINTER(ctypes.c_uint64)]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        L.oracle_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def threshold(eps: float) -> float:
    """Largest double T with sqrt(T) <= eps (the reference predicate as d2 <= T)."""
    return lib().oracle_threshold(float(eps))


def num_threads() -> int:
    return lib().oracle_num_threads()


def _as_rows(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    if x.ndim != 2:
        raise ValueError("points must be a 2-D array")
    return x


def self_join(x, eps: float, nthreads: int = 0):
    """Per-point neighbour counts (self included) and their total."""
    x = _as_rows(x)
    n, d = x.shape
    counts = np.zeros(n, dtype=np.int32)
    total = ctypes.c_uint64(0)
    rc = lib().oracle_self_join(x.ctypes.data, n, d, d, float(eps), counts.ctypes.data,
                                ctypes.addressof(total), nthreads)
    if rc:
        raise RuntimeError(f"oracle_self_join failed: {rc}")
    return counts, int(total.value)


def cross_counts(q, x, eps: float, nthreads: int = 0):
    """For every query row, the number of points within eps."""
    q, x = _as_rows(q), _as_rows(x)
    if q.shape[1] != x.shape[1]:
        raise ValueError("queries and points differ in dimension")
    counts = np.zeros(q.shape[0], dtype=np.int32)
    rc = lib().oracle_cross_counts(q.ctypes.data, q.shape[0], x.ctypes.data, x.shape[0], x.shape[1],
                                   x.shape[1], float(eps), counts.ctypes.data, nthreads)
    if rc:
        raise RuntimeError(f"oracle_cross_counts failed: {rc}")
    return counts


def neighbor_lists(x, eps: float, nthreads: int = 0):
    """CSR neighbour lists (ascending, self included): (offsets uint64[n+1],
    neighbors uint32[total])."""
    x = _as_rows(x)
    n, d = x.shape
    counts, total = self_join(x, eps, nthreads)
    offsets = np.zeros(n + 1, dtype=np.uint64)
    offsets[1:] = np.cumsum(counts.astype(np.uint64))
    nb = np.zeros(max(total, 1), dtype=np.uint32)
    rc = lib().oracle_neighbor_lists(x.ctypes.data, n, d, d, float(eps), offsets.ctypes.data,
                                     nb.ctypes.data, nthreads)
    if rc:
        raise RuntimeError(f"oracle_neighbor_lists failed: {rc}")
    return offsets, nb[:total]


def query_counts(x, eps: float, rows, nthreads: int = 0):
    """Counts of the selected query rows against all points."""
    x = _as_rows(x)
    n, d = x.shape
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    counts = np.zeros(rows.shape[0], dtype=np.int32)
    rc = lib().oracle_query_counts(x.ctypes.data, n, d, d, float(eps), rows.ctypes.data,
                                   rows.shape[0], counts.ctypes.data, nthreads)
    if rc:
        raise RuntimeError(f"oracle_query_counts failed: {rc}")
    return counts


def pair_d2(a, b) -> float:
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().oracle_pair_d2(a.ctypes.data, b.ctypes.data, a.shape[0])


def import_dataset(filename: str, dim: int) -> np.ndarray:
    """Restatement of dataset.cu:10-39 (fscanf loop), returns an (n, dim) array."""
    ptr = ctypes.c_void_p()
    n = ctypes.c_uint64()
    rc = lib().oracle_import_dataset(filename.encode(), dim, ctypes.byref(ptr), ctypes.byref(n))
    if rc:
        raise OSError(f"oracle_import_dataset({filename!r}) failed: {rc}")
    try:
        count = n.value * dim
        if count == 0:
            return np.zeros((0, dim), dtype=np.float64)
        buf = (ctypes.c_double * count).from_address(ptr.value)
        return np.array(buf, dtype=np.float64).reshape(n.value, dim)
    finally:
        lib().oracle_free(ptr)


def reference_loader_available() -> bool:
    return os.path.exists(REF_LOADER)


def reference_import_dataset(filename: str, out_path: str) -> np.ndarray:
    """Run the reference's own compiled importDataset (dim fixed at its
    compile-time INPUT_DATA_DIM = 90, params.h:4)."""
    subprocess.check_call([REF_LOADER, filename, out_path])
    with open(out_path, "rb") as f:
        header = f.readline().split()
        n, dim = int(header[0]), int(header[1])
        data = np.frombuffer(f.read(), dtype=np.float64)
    return data.reshape(n, dim) if n else np.zeros((0, 90))


# --- independent pure-Python restatement (small inputs only) -----------------

def py_threshold(eps: float) -> float:
    if math.isnan(eps):
        return math.nan
    if eps < 0:
        return -math.inf
    if math.isinf(eps):
        return math.inf
    t = eps * eps
    if math.isinf(t):
        t = 1.7976931348623157e308
    while t > 0 and math.sqrt(t) > eps:
        t = math.nextafter(t, 0.0)
    while True:
        up = math.nextafter(t, math.inf)
        if math.isinf(up) or not (math.sqrt(up) <= eps):
            return t
        t = up


def py_fma(a: float, b: float, c: float) -> float:
    """Correctly rounded a*b+c via exact rational arithmetic (CPython's
    int/int true division rounds correctly)."""
    if not (math.isfinite(a) and math.isfinite(b) and math.isfinite(c)):
        return a * b + c
    from fractions import Fraction
    r = Fraction(a) * Fraction(b) + Fraction(c)
    if r == 0:
        return 0.0 if not (c == 0 and math.copysign(1, c) < 0 and a * b == 0) else c
    return r.numerator / r.denominator


def py_pair_d2(a, b) -> float:
    """The reference's compiled arithmetic (oracle.c pair_d2): with t_j the
    rounded differences, fma(t0, t0, fl(t1 * t1)), then fma(t_j, t_j, acc)."""
    t = [float(ak) - float(bk) for ak, bk in zip(a, b)]
    t1 = t[1] if len(t) > 1 else 0.0
    acc = py_fma(t[0], t[0], t1 * t1)
    for v in t[2:]:
        acc = py_fma(v, v, acc)
    return acc


def py_self_join(x, eps: float):
    """O(n^2 d) pure-Python loops with sqrt(d2) <= eps literally (tiny n only)."""
    x = [list(map(float, r)) for r in np.asarray(x, dtype=np.float64)]
    counts = []
    for a in x:
        c = 0
        for b in x:
            d2 = py_pair_d2(a, b)
            if math.sqrt(d2) <= eps if not math.isnan(d2) else False:
                c += 1
        counts.append(c)
    return np.array(counts, dtype=np.int32), int(sum(counts))
