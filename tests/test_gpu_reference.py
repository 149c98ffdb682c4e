"""GPU: the reference's own compiled FP64 kernel pins the oracle's arithmetic.

The counts are defined by the reference's FP64 CUDA-core kernel
distanceCalculationBruteForceCuda (kernel_join.cu:168-200).  How its loop
`acc += (p - c) * (p - c)` is rounded is up to the compiler: a plain fma
chain, acc + fl(t * t) throughout, or -- what nvcc produces for sm_103a --
fma(t0, t0, fl(t1 * t1)) followed by the fma chain (`0 + t0 * t0` folded into
the bare product, which is then fused into the second step).  These tests run
that kernel itself -- compiled from the reference's sources for sm_103a by
oracle/build_ref.sh, launched as gpu_join.cu:273-282 does -- on the golden
fixtures:

* the contraction fixtures (d = 18, 64, 128), whose pairs lie within ulps of
  the radius and which the three readings count differently: the reference's
  kernel counts what the third reading, the oracle and the library count; the
  same source compiled with -fmad=false counts what the uncontracted sum
  counts;
* the reference's sample inputs test100 / test128 at the eps of its run log,
  and the tie grid: its totals equal the oracle's.

Skipped where the reference kernels were not built (no reference checkout
where build() ran).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refgpu():
    from oracle import refgpu as r

    r.build()
    if not r.available("fp64_d18", "fp64_d18_nofma", "fp64_d3"):
        pytest.skip("reference kernels not built (no reference checkout where build() ran)")
    return r


def load(name, d):
    return np.fromfile(os.path.join(GOLDEN, name), dtype="<f8").reshape(-1, d)


@pytest.mark.parametrize("variant,name,cdim", [("fp64_d18", "contraction", 20),
                                               ("fp64_d64", "contraction_d64", 64),
                                               ("fp64_d128", "contraction_d128", 128)])
def test_reference_fp64_kernel_pins_the_oracle_reading(refgpu, oracle_mod, variant, name, cdim):
    if not refgpu.available(variant):
        pytest.skip(f"{variant} not built")
    g = json.load(open(os.path.join(GOLDEN, name + ".json")))
    x = load(name + ".f64", g["d"])
    r = refgpu.run(variant, "cuda", x, g["eps"], cdim)
    assert r["total"] == g["first"]["total"] == oracle_mod.self_join(x, g["eps"])[1]
    assert len({g[k]["total"] for k in ("fma", "first", "mul_add")}) == 3


def test_reference_fp64_kernel_without_contraction(refgpu):
    g = json.load(open(os.path.join(GOLDEN, "contraction.json")))
    x = load("contraction.f64", g["d"])
    r = refgpu.run("fp64_d18_nofma", "cuda", x, g["eps"], 20)
    assert r["total"] == g["mul_add"]["total"]


@pytest.mark.parametrize("name", ["test100", "test128"])
def test_reference_fp64_kernel_on_its_sample_inputs(refgpu, name):
    g = json.load(open(os.path.join(GOLDEN, "join_golden.json")))["files"][name]
    x = load(name + ".f64", g["d"])
    for case in g["cases"]:
        r = refgpu.run("fp64_d18", "cuda", x, case["eps"], 20)
        assert r["total"] == case["total"], case["eps"]


def test_reference_fp64_kernel_on_the_tie_grid(refgpu):
    g = json.load(open(os.path.join(GOLDEN, "ties.json")))
    x = load("ties.f64", g["d"])
    for case in g["cases"]:
        r = refgpu.run("fp64_d3", "cuda", x, case["eps"], 4)
        assert r["total"] == case["total"], case["eps"]
