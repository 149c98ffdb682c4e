"""Build recipe for libejoin.so (sm_103a) and its GPU self-test probe.

    python -m tensor_bf_main_gb300.build

Each translation unit is compiled by nvcc in parallel into ``_build/`` and
linked into ``tensor_bf_main_gb300/libejoin.so`` (CUDA runtime linked
statically, driver entry points resolved at run time, so the library loads on
a machine without a GPU).  No cmake, one ``-gencode``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libejoin.so")
CLI = os.path.join(PKG, "ejoin_main")
PROBE_SRC = os.path.join(ROOT, "tests", "csrc", "umma_probe.cu")
PROBE_LIB = os.path.join(ROOT, "tests", "csrc", "libumma_probe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-I", INCLUDE, "-I", CSRC, "-diag-suppress", "177"]

CU_SOURCES = ["api.cu", "k_direct.cu", "k_prep.cu", "k_dmma.cu", "k_umma.cu", "k_misc.cu",
              "k_learn.cu", "k_noalloc.cu", "k_lists.cu"]
CPP_SOURCES = ["host.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return hs


def _compile(src: str, obj: str, deps) -> str:
    if _newer(obj, [src, *deps]):
        return obj
    if src.endswith(".cpp"):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-I", INCLUDE, "-c", src, "-o", obj]
    else:
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, probe: bool = True) -> str:
    os.makedirs(BUILD, exist_ok=True)
    deps = _headers()
    jobs = []
    for f in CU_SOURCES + CPP_SOURCES:
        src = os.path.join(CSRC, f)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, os.path.splitext(f)[0] + ".o")
        jobs.append((src, obj))
    probe_obj = os.path.join(BUILD, "umma_probe.o")
    if probe and os.path.exists(PROBE_SRC):
        jobs.append((PROBE_SRC, probe_obj))
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    with ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda j: _compile(j[0], j[1], deps), jobs))
    lib_objs = [o for o in objs if o != probe_obj]
    if not _newer(LIB, lib_objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *lib_objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if probe and probe_obj in objs and not _newer(PROBE_LIB, [probe_obj, LIB]):
        tmp = PROBE_LIB + ".tmp"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, probe_obj, "-L", PKG, "-lejoin",
               "-Xlinker", "-rpath=" + PKG]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"probe link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, PROBE_LIB)
    cli_src = os.path.join(CSRC, "cli_main.cpp")
    if os.path.exists(cli_src) and not _newer(CLI, [cli_src, LIB, *deps]):
        cmd = ["g++", "-O2", "-std=c++17", "-I", INCLUDE, cli_src, "-o", CLI + ".tmp", "-L", PKG,
               "-lejoin", "-Wl,-rpath," + PKG]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(CLI + ".tmp", CLI)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
