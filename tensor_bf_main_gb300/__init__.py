"""GB300-native exact epsilon self-join (Python host side of libejoin.so).

The product is the C ABI in ``include/ejoin.h`` (``libejoin.so``, hand-written
sm_103a CUDA kernels).  This module binds it with ctypes and mirrors the
reference's host interface:

* :func:`importDataset` -- the reference's loader (dataset.cu:10-39)
* :func:`GPUJoinMainBruteForce` -- the reference's driver (gpu_join.cu:210-216),
  returning the total number of ordered neighbour pairs
* :func:`self_join` -- the full interface: per-point counts, total, statistics

Inputs may be numpy arrays (host memory) or CUDA tensors / objects exposing
``data_ptr()`` (device memory, used in place).  There is no CPU fallback: if
the library or an sm_103 GPU is missing, calls raise :class:`EjoinError`.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

__all__ = [
    "EjoinError", "Precision", "Order", "self_join", "query_counts", "train_projection",
    "certify_spectral_norm", "threshold", "importDataset", "import_binary",
    "GPUJoinMainBruteForce", "load_library", "LIB_PATH",
]

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libejoin.so")

# searchMode ids of the reference (params.h:166-171)
SM_GPU, SM_CUDA_ALT, SM_TENSOR, SM_TENSOR_MQ, SM_LEARNED = 1, 2, 3, 4, 5


class Precision:
    FP64_DIRECT = 0
    FP64_DMMA = 1
    FP16 = 2
    BF16 = 3
    BF16_SPLIT = 4
    FP8_E4M3 = 5
    AUTO = 6
    NAMES = {0: "fp64_direct", 1: "fp64_dmma", 2: "fp16", 3: "bf16", 4: "bf16_split",
             5: "fp8_e4m3", 6: "auto"}

    @classmethod
    def parse(cls, p) -> int:
        if isinstance(p, str):
            inv = {v: k for k, v in cls.NAMES.items()}
            if p.lower() not in inv:
                raise ValueError(f"unknown precision {p!r}")
            return inv[p.lower()]
        return int(p)


class Order:
    MORTON = 0
    LEAD = 1


class EjoinError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"ejoin status {status}: {message}")
        self.status = status


class Options(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32), ("device", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("proj_k", ctypes.c_uint32), ("ld", ctypes.c_uint64),
        ("projection", ctypes.c_void_p), ("train_pairs", ctypes.c_uint64),
        ("train_steps", ctypes.c_uint32), ("order", ctypes.c_uint32), ("seed", ctypes.c_uint64),
        ("stream", ctypes.c_void_p), ("band_capacity", ctypes.c_uint64),
        ("acc_bound_scale", ctypes.c_double), ("flags", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32 * 7),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_uint64), ("d", ctypes.c_uint32), ("precision", ctypes.c_int32),
        ("band_pairs", ctypes.c_uint64), ("band_hits", ctypes.c_uint64),
        ("tile_pairs_total", ctypes.c_uint64), ("tile_pairs_run", ctypes.c_uint64),
        ("band_overflows", ctypes.c_uint64), ("band_fraction", ctypes.c_double),
        ("sigma_cert", ctypes.c_double), ("ms_total", ctypes.c_double),
        ("ms_prep", ctypes.c_double), ("ms_train", ctypes.c_double),
        ("ms_order", ctypes.c_double), ("ms_gram", ctypes.c_double),
        ("ms_recheck", ctypes.c_double), ("gram_flops", ctypes.c_double),
        ("kernel_launches", ctypes.c_uint64), ("reserved", ctypes.c_double * 5),
    ]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}
        d["precision"] = Precision.NAMES.get(d["precision"], d["precision"])
        d["exact_rechecks"] = int(self.reserved[0])
        d["gram_blocks"] = int(self.reserved[1])
        d["scratch_peak_bytes"] = int(self.reserved[2])
        d["band_records"] = int(self.reserved[3])
        return d


# Every symbol include/ejoin.h declares (checked by the CPU test-suite).
EXPORTED = [
    "ejoin_default_options", "ejoin_self_join", "ejoin_query_counts", "ejoin_train_projection",
    "ejoin_certify_spectral_norm", "ejoin_threshold", "ejoin_import_dataset",
    "ejoin_import_binary", "ejoin_free", "ejoin_last_error", "ejoin_version",
    "ejoin_gpu_join_main_brute_force", "ejoin_self_join_noalloc", "ejoin_neighbor_lists",
    "ejoin_join_counts", "ejoin_release_scratch", "ejoin_save_projection",
    "ejoin_load_projection",
]

# Test hooks declared in include/ejoin_testing.h.
TESTING = ["ejoin_testing_projection_grad", "ejoin_testing_renormalise", "ejoin_testing_inject"]

# option flags (include/ejoin.h)
FLAG_KEEP_SCRATCH = 0x2
# failure injection (include/ejoin_testing.h)
TESTING_FAIL_ALLOC = 1
TESTING_GRAM_TIMEOUT = 2

_lib = None


def load_library(path: str = LIB_PATH):
    """Load libejoin.so (building it first if it is missing and nvcc exists)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(path)
    vp, u64, u32, i32, dbl = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int32, ctypes.c_double
    L.ejoin_default_options.argtypes = [ctypes.POINTER(Options)]
    L.ejoin_self_join.argtypes = [vp, u64, u32, dbl, ctypes.POINTER(Options), vp, ctypes.POINTER(u64),
                                  ctypes.POINTER(Stats)]
    L.ejoin_query_counts.argtypes = [vp, u64, u32, dbl, vp, u64, ctypes.POINTER(Options), vp]
    L.ejoin_neighbor_lists.argtypes = [vp, u64, u32, dbl, ctypes.POINTER(Options), vp, vp, u64,
                                       ctypes.POINTER(u64), ctypes.POINTER(Stats)]
    L.ejoin_join_counts.argtypes = [vp, u64, vp, u64, u32, dbl, ctypes.POINTER(Options), vp,
                                    ctypes.POINTER(u64), ctypes.POINTER(Stats)]
    L.ejoin_train_projection.argtypes = [vp, u64, u32, dbl, ctypes.POINTER(Options), vp,
                                         ctypes.POINTER(dbl), ctypes.POINTER(Stats)]
    L.ejoin_certify_spectral_norm.argtypes = [vp, u32, u32, ctypes.POINTER(dbl)]
    L.ejoin_threshold.argtypes = [dbl]
    L.ejoin_threshold.restype = dbl
    L.ejoin_import_dataset.argtypes = [ctypes.c_char_p, u32, ctypes.POINTER(vp), ctypes.POINTER(u64)]
    L.ejoin_import_binary.argtypes = [ctypes.c_char_p, u32, ctypes.POINTER(vp), ctypes.POINTER(u64)]
    L.ejoin_free.argtypes = [vp]
    L.ejoin_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    L.ejoin_gpu_join_main_brute_force.argtypes = [u32, u32, vp, ctypes.POINTER(u32),
                                                  ctypes.POINTER(dbl), ctypes.POINTER(u64), u32, u32]
    L.ejoin_testing_projection_grad.argtypes = [vp, vp, u64, vp, u32, u32, vp, vp]
    L.ejoin_testing_projection_grad.restype = ctypes.c_int
    L.ejoin_testing_renormalise.argtypes = [vp, u32, u32, vp]
    L.ejoin_testing_renormalise.restype = ctypes.c_int
    L.ejoin_self_join_noalloc.argtypes = [vp, u64, u32, dbl, ctypes.c_int, vp, vp, ctypes.POINTER(u64)]
    L.ejoin_release_scratch.argtypes = [ctypes.c_int]
    L.ejoin_save_projection.argtypes = [ctypes.c_char_p, vp, u32, u32, dbl]
    L.ejoin_load_projection.argtypes = [ctypes.c_char_p, vp, u64, ctypes.POINTER(u32),
                                        ctypes.POINTER(u32), ctypes.POINTER(dbl)]
    L.ejoin_testing_inject.argtypes = [ctypes.c_int, u64]
    L.ejoin_testing_inject.restype = ctypes.c_int
    for name in EXPORTED:
        if name not in ("ejoin_threshold", "ejoin_free"):
            getattr(L, name).restype = ctypes.c_int
    L.ejoin_free.restype = None
    _lib = L
    return L


def _check(rc: int):
    if rc != 0:
        buf = ctypes.create_string_buffer(2048)
        load_library().ejoin_last_error(buf, len(buf))
        raise EjoinError(rc, buf.value.decode(errors="replace"))


def _options(device=0, precision=Precision.AUTO, proj_k=0, ld=0, projection=None,
             train_pairs=1 << 19, train_steps=50, order=Order.MORTON, seed=0x5EED5EED,
             stream=None, band_capacity=0, acc_bound_scale=1.0, keep_scratch=False):
    o = Options()
    _check(load_library().ejoin_default_options(ctypes.byref(o)))
    o.device = int(device)
    o.precision = Precision.parse(precision)
    o.proj_k = int(proj_k)
    o.ld = int(ld)
    o.train_pairs = int(train_pairs)
    o.train_steps = int(train_steps)
    o.order = int(order)
    o.seed = int(seed)
    o.band_capacity = int(band_capacity)
    o.acc_bound_scale = float(acc_bound_scale)
    if keep_scratch:
        o.flags |= FLAG_KEEP_SCRATCH
    if projection is not None:
        p = np.ascontiguousarray(projection, dtype=np.float32)
        o._proj_keepalive = p
        o.projection = p.ctypes.data
    if stream is not None:
        o.stream = int(getattr(stream, "cuda_stream", stream))
    return o


def _points_arg(points):
    """(pointer, n, d, keepalive) for a numpy array or a CUDA tensor."""
    if hasattr(points, "data_ptr") and hasattr(points, "is_cuda"):
        if points.dtype.__str__() not in ("torch.float64",):
            raise TypeError("device points must be float64")
        if points.dim() != 2 or points.stride(1) != 1:
            raise ValueError("device points must be a row-major 2-D tensor")
        return points.data_ptr(), points.shape[0], points.shape[1], points.stride(0), points
    a = np.asarray(points)
    if a.ndim != 2:
        raise ValueError("points must be 2-D (n, d)")
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a.ctypes.data, a.shape[0], a.shape[1], a.shape[1], a


def self_join(points, eps: float, precision="auto", proj_k: int = 0, device: int = 0,
              counts=True, stats: bool = True, **kw):
    """Exact epsilon self-join.  Returns (counts, total, stats_dict).

    counts: per-point int32 numpy array (host) -- or pass a preallocated
    int32 CUDA tensor to receive them on the device -- or False for none.
    """
    L = load_library()
    ptr, n, d, ld, keep = _points_arg(points)
    o = _options(device=device, precision=precision, proj_k=proj_k, ld=ld if ld != d else 0, **kw)
    out = None
    out_ptr = None
    if counts is True:
        out = np.zeros(n, dtype=np.int32)
        out_ptr = out.ctypes.data
    elif counts is not False and counts is not None:
        out = counts
        out_ptr = counts.data_ptr() if hasattr(counts, "data_ptr") else counts.ctypes.data
    total = ctypes.c_uint64(0)
    st = Stats()
    _check(L.ejoin_self_join(ptr, n, d, float(eps), ctypes.byref(o), out_ptr, ctypes.byref(total),
                             ctypes.byref(st)))
    del keep
    return out, int(total.value), (st.as_dict() if stats else None)


def neighbor_lists(points, eps: float, precision="auto", proj_k: int = 0, device: int = 0, **kw):
    """Neighbour lists of the exact self-join (CSR, input order, ascending,
    self included).  Returns (offsets uint64[n+1], neighbors uint32[total],
    stats_dict).  Two library calls: the first sizes the lists."""
    L = load_library()
    ptr, n, d, ld, keep = _points_arg(points)
    o = _options(device=device, precision=precision, proj_k=proj_k, ld=ld if ld != d else 0, **kw)
    offsets = np.zeros(n + 1, dtype=np.uint64)
    total = ctypes.c_uint64(0)
    st = Stats()
    _check(L.ejoin_neighbor_lists(ptr, n, d, float(eps), ctypes.byref(o), offsets.ctypes.data,
                                  None, 0, ctypes.byref(total), ctypes.byref(st)))
    nb = np.zeros(max(int(total.value), 1), dtype=np.uint32)
    _check(L.ejoin_neighbor_lists(ptr, n, d, float(eps), ctypes.byref(o), offsets.ctypes.data,
                                  nb.ctypes.data, nb.shape[0], ctypes.byref(total),
                                  ctypes.byref(st)))
    del keep
    return offsets, nb[: int(total.value)], st.as_dict()


def join_counts(queries, points, eps: float, precision="auto", device: int = 0, **kw):
    """Join of two point sets: for every query row, the number of points within
    eps (exact).  Returns (counts int32[nq], total, stats_dict)."""
    L = load_library()
    qptr, nq, dq, ldq, keepq = _points_arg(queries)
    ptr, n, d, ld, keep = _points_arg(points)
    if dq != d or ldq != ld:
        raise ValueError("queries and points need the same dimension and row stride")
    o = _options(device=device, precision=precision, ld=ld if ld != d else 0, **kw)
    out = np.zeros(nq, dtype=np.int32)
    total = ctypes.c_uint64(0)
    st = Stats()
    _check(L.ejoin_join_counts(qptr, nq, ptr, n, d, float(eps), ctypes.byref(o), out.ctypes.data,
                               ctypes.byref(total), ctypes.byref(st)))
    del keep, keepq
    return out, int(total.value), st.as_dict()


def query_counts(points, eps: float, rows, device: int = 0):
    L = load_library()
    ptr, n, d, ld, keep = _points_arg(points)
    rows = np.ascontiguousarray(rows, dtype=np.uint64)
    out = np.zeros(rows.shape[0], dtype=np.int32)
    o = _options(device=device, ld=ld if ld != d else 0)
    _check(L.ejoin_query_counts(ptr, n, d, float(eps), rows.ctypes.data, rows.shape[0],
                                ctypes.byref(o), out.ctypes.data))
    del keep
    return out


def train_projection(points, eps: float, k: int = 8, device: int = 0, **kw):
    """Train the contractive projection; returns (P (k x d float32), sigma_cert, stats)."""
    L = load_library()
    ptr, n, d, ld, keep = _points_arg(points)
    o = _options(device=device, proj_k=k, ld=ld if ld != d else 0, **kw)
    P = np.zeros((k, d), dtype=np.float32)
    sig = ctypes.c_double(0)
    st = Stats()
    _check(L.ejoin_train_projection(ptr, n, d, float(eps), ctypes.byref(o), P.ctypes.data,
                                    ctypes.byref(sig), ctypes.byref(st)))
    del keep
    info = st.as_dict()
    info["loss_first"], info["loss_last"] = st.reserved[0], st.reserved[1]
    return P, sig.value, info


def save_projection(filename: str, P, sigma_cert: float) -> None:
    """Write a learned projection (k x d) and its certified bound to a file."""
    P = np.ascontiguousarray(P, dtype=np.float32)
    if P.ndim != 2:
        raise ValueError("P must be k x d")
    _check(load_library().ejoin_save_projection(filename.encode(), P.ctypes.data, P.shape[0],
                                                P.shape[1], float(sigma_cert)))


def load_projection(filename: str):
    """Read a projection file: returns (P (k x d float32), sigma_cert)."""
    L = load_library()
    k, d, sig = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_double()
    _check(L.ejoin_load_projection(filename.encode(), None, 0, ctypes.byref(k), ctypes.byref(d),
                                   ctypes.byref(sig)))
    P = np.zeros((k.value, d.value), dtype=np.float32)
    _check(L.ejoin_load_projection(filename.encode(), P.ctypes.data, P.size, ctypes.byref(k),
                                   ctypes.byref(d), ctypes.byref(sig)))
    return P, sig.value


def release_scratch(device: int = 0) -> None:
    """Return the scratch cached by keep_scratch=True calls to the device."""
    _check(load_library().ejoin_release_scratch(int(device)))


def testing_inject(what: int, value: int) -> None:
    """Failure injection for the error-path tests (include/ejoin_testing.h)."""
    _check(load_library().ejoin_testing_inject(int(what), int(value)))


def certify_spectral_norm(P) -> float:
    P = np.ascontiguousarray(P, dtype=np.float32)
    b = ctypes.c_double(0)
    _check(load_library().ejoin_certify_spectral_norm(P.ctypes.data, P.shape[0], P.shape[1],
                                                      ctypes.byref(b)))
    return b.value


def threshold(eps: float) -> float:
    return load_library().ejoin_threshold(float(eps))


def _import(fn, filename: str, dim: int) -> np.ndarray:
    L = load_library()
    p = ctypes.c_void_p()
    n = ctypes.c_uint64()
    _check(fn(filename.encode(), dim, ctypes.byref(p), ctypes.byref(n)))
    try:
        cnt = n.value * dim
        if cnt == 0:
            return np.zeros((0, dim), dtype=np.float64)
        buf = (ctypes.c_double * cnt).from_address(p.value)
        return np.array(buf, dtype=np.float64).reshape(n.value, dim)
    finally:
        L.ejoin_free(p)


def importDataset(filename: str, dim: int) -> np.ndarray:
    """The reference's text loader (dataset.cu:10-39) with a run-time dimension."""
    return _import(load_library().ejoin_import_dataset, filename, dim)


def import_binary(filename: str, dim: int) -> np.ndarray:
    return _import(load_library().ejoin_import_binary, filename, dim)


def GPUJoinMainBruteForce(searchMode: int, device: int, dataset, nbQueryPoints: int,
                          epsilon: float, input_dim: int | None = None,
                          compute_dim: int | None = None) -> int:
    """Mirror of the reference driver (gpu_join.cu:210-216).

    ``dataset`` is the padded host array main.cu:38-57 builds (row stride
    compute_dim, input_dim columns used, 15 trailing zero rows ignored) or a
    plain (n, d) array.  Returns totalNeighbors (ordered pairs, self included).
    """
    L = load_library()
    a = np.ascontiguousarray(dataset, dtype=np.float64)
    if a.ndim == 2:
        compute_dim = compute_dim or a.shape[1]
        input_dim = input_dim or a.shape[1]
    if input_dim is None or compute_dim is None:
        raise ValueError("input_dim and compute_dim are required for a flat dataset")
    nq = ctypes.c_uint32(int(nbQueryPoints))
    eps = ctypes.c_double(float(epsilon))
    total = ctypes.c_uint64(0)
    _check(L.ejoin_gpu_join_main_brute_force(int(searchMode), int(device), a.ctypes.data,
                                             ctypes.byref(nq), ctypes.byref(eps),
                                             ctypes.byref(total), int(input_dim), int(compute_dim)))
    return int(total.value)
