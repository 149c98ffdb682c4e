"""GPU: the failure paths of the library, made to happen on purpose.

The reference printed CUDA errors and carried on (utils.cu:7-13) or exited
(gpu_join.cu:313-314, dataset.cu:16-20).  Here every failure is a status
code, and these tests force each one through the library's own hooks
(include/ejoin_testing.h) -- never by faulting the GPU:

* a band queue far too small for the boundary band: the screen re-runs with
  the exact size and the counts stay exact;
* a bounded device wait that expires (the tensor-core screen with a 1 ms
  deadline and a producer that never issues its first stage): the call
  returns EJOIN_ETIMEOUT, the kernel drains and frees its tensor memory, and
  the next call succeeds;
* the k-th device allocation failing, for every k a join makes: EJOIN_ENOMEM,
  every buffer released, the next call exact;
* the library's scratch goes back to the device after each call (the default
  memory pool of the process is never touched), or stays cached with
  keep_scratch until release_scratch.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ENOMEM, ETIMEOUT = -3, -6


def clustered(n, d, rng, k=8, sigma=0.05):
    c = rng.random((k, d))
    return c[rng.integers(0, k, n)] + sigma * rng.standard_normal((n, d))


@pytest.fixture(scope="module")
def case(oracle_mod):
    """Clusters plus two far-off groups of 40 identical points exactly eps
    apart: 1,600 pairs on the boundary itself, which every screen (the FP64
    one included) must send to the exact recheck."""
    rng = np.random.default_rng(99)
    x = clustered(4000, 32, rng)
    i, j = rng.integers(0, 4000, 4000), rng.integers(0, 4000, 4000)
    eps = float(np.quantile(np.sqrt(((x[i] - x[j]) ** 2).sum(1)), 60 / 4000))
    g = np.full((80, 32), 50.0)
    g[40:, 0] += eps
    x = np.concatenate([x, g])
    exp, tot = oracle_mod.self_join(x, eps)
    return x, eps, exp, tot


@pytest.mark.parametrize("mode", ["bf16_split", "fp16", "fp8_e4m3", "fp64_dmma"])
def test_band_overflow_reruns_with_exact_counts(ej, case, mode):
    x, eps, exp, tot = case
    counts, total, st = ej.self_join(x, eps, precision=mode, band_capacity=1024)
    assert st["band_overflows"] >= 1, st
    assert total == tot and np.array_equal(counts, exp)


def test_expired_wait_returns_etimeout_and_next_call_succeeds(ej, case):
    x, eps, exp, tot = case
    ej.testing_inject(ej.TESTING_GRAM_TIMEOUT, 1_000_000)  # 1 ms deadline
    with pytest.raises(ej.EjoinError) as e:
        ej.self_join(x, eps, precision="bf16_split")
    assert e.value.status == ETIMEOUT
    assert "bounded device wait" in str(e.value)
    for mode in ("bf16_split", "fp8_e4m3"):
        counts, total, _ = ej.self_join(x, eps, precision=mode)
        assert total == tot and np.array_equal(counts, exp)


def free_bytes():
    import torch

    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


@pytest.mark.parametrize("mode,k", [("bf16_split", 8), ("fp64_dmma", 0)])
def test_every_allocation_failure_is_enomem_and_releases(ej, case, mode, k):
    x, eps, exp, tot = case
    free0 = free_bytes()
    failed = 0
    for nth in range(1, 200):
        ej.testing_inject(ej.TESTING_FAIL_ALLOC, nth)
        try:
            counts, total, _ = ej.self_join(x, eps, precision=mode, proj_k=k)
        except ej.EjoinError as e:
            assert e.status == ENOMEM, nth
            assert "allocation" in str(e)
            failed += 1
        else:
            # nth is beyond the allocations of one call: the join ran in full
            ej.testing_inject(ej.TESTING_FAIL_ALLOC, 0)
            assert total == tot and np.array_equal(counts, exp)
            break
        counts, total, _ = ej.self_join(x, eps, precision=mode, proj_k=k)
        assert total == tot and np.array_equal(counts, exp), nth
    else:
        pytest.fail("the join never completed with a late injected failure")
    assert failed >= 5
    assert abs(free_bytes() - free0) < (64 << 20)


def test_scratch_returns_to_the_device_unless_kept(ej, oracle_mod):
    from tensor_bf_main_gb300 import datagen

    x = datagen.generate("c4", n=1_000_000)
    eps = datagen.EPS["c4"]
    free0 = free_bytes()
    _, t0, st = ej.self_join(x, eps, precision="bf16_split", proj_k=8)
    assert st["scratch_peak_bytes"] > (256 << 20)
    assert abs(free_bytes() - free0) < (64 << 20)
    _, t1, st = ej.self_join(x, eps, precision="bf16_split", proj_k=8, keep_scratch=True)
    assert t1 == t0
    assert free0 - free_bytes() > (128 << 20)
    ej.release_scratch(0)
    assert abs(free_bytes() - free0) < (64 << 20)
