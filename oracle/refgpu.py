"""The reference's own GPU join kernels -- TEST AND MEASUREMENT INFRASTRUCTURE.

``oracle/build_ref.sh`` compiles the reference's kernel_join.cu (unmodified
but for its params.h configuration and, in FP64 builds, the guard around the
two FP16-only kernels) into ``oracle/_ref/ref_<variant>.cubin``;
``oracle/ref_gpu.cu`` (built by :func:`build`) loads a cubin and launches its
kernels as the reference driver GPUJoinMainBruteForce does
(gpu_join.cu:210-322).  Used by the GPU tests to pin the oracle's arithmetic
to the reference's compiled FP64 kernel (kernel_join.cu:168-200), and by
bench.py to time the reference's tensor-core kernels
(kernel_join.cu:328-524 FP16, kernel_join.cu:530-677 FP64) on the same GPU.
Never part of the product path.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
LAUNCHER = os.path.join(HERE, "ref_gpu_launch")
SRC = os.path.join(HERE, "ref_gpu.cu")


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return None


def build() -> str | None:
    """Compile the launcher (host code, CUDA driver API) if nvcc is present."""
    nv = _nvcc()
    if nv is None:
        return None
    if os.path.exists(LAUNCHER) and os.path.getmtime(LAUNCHER) >= os.path.getmtime(SRC):
        return LAUNCHER
    stubs = os.path.join(os.path.dirname(os.path.dirname(nv)), "lib64", "stubs")
    tmp = LAUNCHER + ".tmp"
    subprocess.check_call([nv, "-O2", "-std=c++17", SRC, "-o", tmp, "-L", stubs, "-lcuda"])
    os.replace(tmp, LAUNCHER)
    return LAUNCHER


def cubin(variant: str) -> str:
    return os.path.join(REF, f"ref_{variant}.cubin")


def available(*variants: str) -> bool:
    return os.path.exists(LAUNCHER) and all(os.path.exists(cubin(v)) for v in variants)


def run(variant: str, kind: str, x, eps: float, compute_dim: int, reps: int = 1,
        timeout: float = 900.0) -> dict:
    """Run kernel `kind` ('cuda' = searchMode 1, 'mq16' / 'mq64' = searchMode 4)
    of the cubin `variant` on the points x (n x input_dim, float64) with radius
    eps.  Returns the launcher's JSON record (total, kernel and driver ms)."""
    x = np.ascontiguousarray(x, dtype="<f8")
    n, d = x.shape
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "points.f64")
        x.tofile(path)
        out = subprocess.run([LAUNCHER, cubin(variant), kind, path, str(n), str(d),
                              str(compute_dim), repr(float(eps)), str(reps)],
                             capture_output=True, text=True, timeout=timeout)
    if out.returncode != 0:
        raise RuntimeError(f"ref_gpu_launch failed ({out.returncode}): {out.stderr.strip()}")
    return json.loads(out.stdout.strip().splitlines()[-1])
