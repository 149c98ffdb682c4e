"""GPU: the allocation-free entry point.

ejoin_self_join_noalloc serves callers that cannot call cudaMalloc while they
run the join -- engines that own all device memory through their own pool,
serving paths that forbid allocation and the synchronisation it implies,
processes under a hard memory cap.  It keeps all scratch in one static device
array.  This test calls it through the C ABI on device buffers the test
allocates itself, twice in a row on different inputs (the shared array keeps
the previous call's contents, so each call must clear what starts at zero),
and checks its per-point counts and total against the allocating entry point
ejoin_self_join in the same exact mode (integer counts: equality).  It also
covers the special radii (inf, negative, NaN), rows with NaN / inf
coordinates, a boundary band larger than the array's queue (EJOIN_ENOMEM with
the counts left at zero), and that sizes beyond the array's limit are
rejected with a clear error.
Collected last (file name) so a stop-at-first-failure run has run the rest.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N, MAX_D = 16384, 128


def clustered(n, d, rng, k=6, sigma=0.04):
    c = rng.random((k, d))
    return c[rng.integers(0, k, n)] + sigma * rng.standard_normal((n, d))


def call(lib, xd, n, d, eps, cd):
    total = ctypes.c_uint64(0)
    rc = lib.ejoin_self_join_noalloc(xd.data_ptr() if xd is not None else None, n, d, eps, 0,
                                     None, cd.data_ptr() if cd is not None else None,
                                     ctypes.byref(total))
    return rc, total.value


def test_no_alloc_matches_allocating_entry_point(ej):
    import torch

    lib = ej.load_library()
    rng = np.random.default_rng(2024)
    for n, d, mean in ((6000, 48, 25), (MAX_N, MAX_D, 40)):
        x = clustered(n, d, rng)
        i, j = rng.integers(0, n, 3000), rng.integers(0, n, 3000)
        eps = float(np.quantile(np.sqrt(((x[i] - x[j]) ** 2).sum(1)), mean / n))
        xd = torch.from_numpy(x).cuda()
        cd = torch.full((n,), -5, dtype=torch.int32, device="cuda")  # stale contents
        rc, total = call(lib, xd, n, d, eps, cd)
        assert rc == 0, ej.EjoinError(rc, "")
        exp, exp_total, _ = ej.self_join(x, eps, precision="fp64_dmma")
        assert total == exp_total
        assert np.array_equal(cd.cpu().numpy(), exp)


def test_no_alloc_special_radii_and_non_finite_rows(ej):
    import torch

    lib = ej.load_library()
    rng = np.random.default_rng(7)
    n, d = 3000, 24
    x = clustered(n, d, rng)
    x[5, 3] = np.nan
    x[17, 0] = np.inf
    x[2999, 23] = -np.inf
    xd = torch.from_numpy(x).cuda()
    for eps in (0.3, float("inf"), -1.0, float("nan"), 0.0):
        cd = torch.full((n,), 7, dtype=torch.int32, device="cuda")
        rc, total = call(lib, xd, n, d, eps, cd)
        assert rc == 0, (eps, rc)
        exp, exp_total, _ = ej.self_join(x, eps, precision="fp64_direct")
        assert total == exp_total, eps
        assert np.array_equal(cd.cpu().numpy(), exp), eps


def test_no_alloc_band_beyond_queue_is_enomem_with_zero_counts(ej):
    """Two groups of 2,100 identical points exactly eps apart: all 4.41 M
    cross pairs lie on the boundary, more than the array's queue holds."""
    import torch

    lib = ej.load_library()
    n, d, half = 4200, 4, 2100
    x = np.zeros((n, d))
    x[half:, 0] = 0.75
    eps = 0.75
    xd = torch.from_numpy(x).cuda()
    cd = torch.full((n,), 9, dtype=torch.int32, device="cuda")
    rc, _ = call(lib, xd, n, d, eps, cd)
    assert rc == -3
    buf = ctypes.create_string_buffer(512)
    lib.ejoin_last_error(buf, 512)
    assert b"exceeds" in buf.value
    assert int(cd.abs().sum().item()) == 0
    # the allocating entry point grows its queue and answers exactly
    exp, exp_total, _ = ej.self_join(x, eps, precision="fp64_dmma")
    assert exp_total == n * n


def test_no_alloc_rejects_sizes_beyond_its_limit(ej):
    import torch

    lib = ej.load_library()
    xd = torch.zeros((4, 4), dtype=torch.float64, device="cuda")
    cd = torch.zeros(4, dtype=torch.int32, device="cuda")
    buf = ctypes.create_string_buffer(512)
    rc, _ = call(lib, xd, MAX_N + 1, 4, 0.5, cd)
    assert rc == -1
    lib.ejoin_last_error(buf, 512)
    assert b"exceeds the limit" in buf.value
    rc, _ = call(lib, xd, 4, MAX_D + 1, 0.5, cd)
    assert rc == -1
    # host buffers are refused: the entry point never stages (that would allocate)
    xh = np.zeros((4, 4))
    total = ctypes.c_uint64(0)
    rc = lib.ejoin_self_join_noalloc(xh.ctypes.data, 4, 4, 0.5, 0, None, cd.data_ptr(),
                                     ctypes.byref(total))
    assert rc == -1
