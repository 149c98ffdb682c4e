#!/usr/bin/env python3
"""Benchmark of the exact epsilon self-join on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--config c4] [--precision auto] [--proj-k K] [--n N]

A step is one exact self-join of the whole synthetic workload (default: c4,
N = 4,000,000 points, d = 64, eps for ~50 neighbours; see
tensor_bf_main_gb300/datagen.py), inputs resident in device memory.  The JSON
line reports pair-distances/s (N^2 ordered pairs per second, the reference's
count semantics), the Gram kernel's tensor-pipe roofline fraction, the
end-to-end rate through the public API from pinned host memory, the plain
FP64 DMMA join rate (speedup denominator, measured on a row subset and
extrapolated as N^2 / rate) and the CPU baseline (the oracle restatement of
the reference's FP64 kernel on all host cores, bounded sample).

--impl reference times the reference's CPU algorithm (the oracle port; the
reference has no CPU join of its own) on the same workload, one bounded
sample of query rows per step.  The reference's own GPU kernels, built from
its sources where the reference checkout is present (oracle/build_ref.sh),
are timed on the same GPU by the default arm and reported in its line under
"reference_gpu".

With --gpus N under torchrun every rank runs an independent replica
(replicas only: the join runs on one GPU) and rank 0 reports the
whole-job rate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "gram_kernel_traffic.json")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", default="c4")
    p.add_argument("--precision", default="config", help="'config': the config's own arithmetic")
    p.add_argument("--proj-k", type=int, default=-1, help="-1: config default")
    p.add_argument("--n", type=int, default=0, help="override N (smaller runs)")
    p.add_argument("--eps", type=float, default=0.0)
    p.add_argument("--eps-index", type=int, default=0, help="c3: which of its three radii")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true")
    p.add_argument("--fp64-rows", type=int, default=65536)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-ref-gpu", action="store_true",
                   help="skip timing the reference's own GPU kernels")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def replica_rate(ms, n, world, dist=None, device=None):
    """Whole-job rate of `world` independent replicas, each joining n points:
    the step time is the maximum over ranks (all_reduce MAX on the process
    group), the rate counts every replica's n^2 ordered pairs.  Returns
    (step ms, pairs/s)."""
    if dist is not None and world > 1:
        import torch

        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * float(n) * float(n) / (ms / 1e3)


def workload(args):
    from tensor_bf_main_gb300 import datagen

    cfg = datagen.CONFIGS[args.config]
    n = args.n or cfg["n"]
    x = datagen.generate(args.config, n=n)
    eps = args.eps or datagen.frozen_eps(args.config, x, args.eps_index)
    return x, float(eps), cfg


def cpu_rate(x, eps, seconds, seed=0):
    """Oracle (reference FP64 arithmetic) on a bounded sample of query rows
    against all points, all host threads: returns (pairs/s, rows, seconds)."""
    import oracle

    oracle.build()
    rng = np.random.default_rng(seed)
    n = x.shape[0]
    rows = rng.choice(n, size=min(n, 16), replace=False)
    t0 = time.perf_counter()
    oracle.query_counts(x, eps, rows)
    t1 = time.perf_counter()
    per_row = max((t1 - t0) / len(rows), 1e-9)
    nq = int(max(1, min(n, seconds / per_row)))
    rows = rng.choice(n, size=nq, replace=False)
    t0 = time.perf_counter()
    oracle.query_counts(x, eps, rows)
    dt = time.perf_counter() - t0
    return nq * n / dt, nq, dt, oracle.num_threads()


class Clocks:
    """nvidia-smi sampling (every 50 ms) from the warm-up steps through the
    timed region: the timed region alone is often shorter than one sample
    period, and the warm-up steps run the same workload."""

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self, gpu_index):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index),
                 "--query-gpu=timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")][1:]  # drop the timestamp
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), float(parts[2]), parts[4:8]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i, v in enumerate(r[3]) if v == "Active"})
        loaded = [r for r in rows if r[2] > 200.0] or rows
        return {"sm_mhz": statistics.median(r[0] for r in loaded),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(r[2] for r in rows)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def gram_roofline(stats, d, prec, pk, args, proj_k):
    """Roofline of the dominant kernel, the tcgen05 Gram screen.

    achieved = MMA flops of the data products over the 128 x 128 tile pairs
    that the screen actually needs (the active halves, `tile_pairs_run`: upper
    triangle, not pruned), x3 with the hi+lo split (hi*hi, hi*lo, lo*hi), the
    16-wide aug product excluded; divided by the kernel's CUDA-event time
    (`ms_gram`, event pair on the launching stream around the one launch).
    peak = the dense BF16 rate of MEASURED_PEAKS.json: the burst figure for a
    launch shorter than half a second (the c4 screen runs for milliseconds
    under the burst clock), the sustained one (a seconds-long loop under the
    power cap) for longer launches; FP8 operands run kind::f8f6f4 at twice the
    BF16 rate, so their peak is 2x that figure.  Two more fractions against
    the same peak:
      frac_executed  every MMA the kernel issued: all 128 x 256 blocks
                     (`gram_blocks`, both halves, inactive ones included),
                     aug products included;
      frac_useful    the hi*hi products of the active halves only (the part
                     of the split that decides the answer alone).
    l2_operand_bytes: bytes the TMA engine moves from L2 into shared memory
    per launch (per block: the A slab of 128 rows and the B slab of 256 rows
    of every K step, plus the 128 + 256 aug rows of 32 bytes).
    """
    gram_ms = statistics.mean(s["ms_gram"] for s in stats)
    t = gram_ms / 1e3
    fp8 = prec == "fp8_e4m3"
    split = prec == "bf16_split"
    dp = -(-d // (128 if fp8 else 64)) * (128 if fp8 else 64)
    tiles = statistics.mean(s["tile_pairs_run"] for s in stats)
    blocks = statistics.mean(s["gram_blocks"] for s in stats)
    kdata = (3 if split else 1) * dp
    f_needed = tiles * 2.0 * 128 * 128 * kdata
    f_useful = tiles * 2.0 * 128 * 128 * dp
    f_exec = blocks * 2.0 * 128 * 256 * (kdata + 16)
    long_launch = gram_ms >= 500.0
    key = "bf16_tflops_sustained" if long_launch else "bf16_tflops"
    measured = (pk or {}).get(key)
    fallback = 1700.0 if long_launch else 1900.0
    peak = (measured or fallback) * (2.0 if fp8 else 1.0)
    src = (f"MEASURED_PEAKS.json {key} ({'sustained' if long_launch else 'burst'})" if measured
           else f"fallback {fallback / 1000:.1f} PFLOP/s") + (" x2 (FP8 kind::f8f6f4)" if fp8 else "")
    achieved = f_needed / t / 1e12
    elem = 1 if fp8 else 2
    steps = (dp * elem // 128) * (2 if split else 1)  # K slabs of 128-byte rows
    l2_bytes = blocks * (steps * (128 + 256) * 128 + (128 + 256) * 32)
    traffic = None
    try:
        prof = json.load(open(PROFILE_SUMMARY))
        key = f"{args.config}:{prec}:k{proj_k}"
        if key in prof:
            traffic = prof[key]["traffic_bytes_per_launch"]
    except (OSError, ValueError, KeyError):
        pass
    return {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": traffic, "peak_source": src,
            "kernel": "gram_kernel (tcgen05)",
            "flops_per_launch": f_needed, "ms_per_launch": gram_ms,
            "frac_executed": f_exec / t / 1e12 / peak, "flops_executed_per_launch": f_exec,
            "frac_useful": f_useful / t / 1e12 / peak,
            "active_tile_pairs": tiles, "blocks": blocks,
            "l2_operand_bytes": l2_bytes, "l2_operand_gbs": l2_bytes / t / 1e9}


def reference_gpu(ej, x, eps, stream, dev, n16=262144, n64=32768):
    """The reference's own tensor-core join kernels on this GPU, built from its
    kernel_join.cu by oracle/build_ref.sh and launched as its driver does
    (oracle/ref_gpu.cu): distanceCalculationBruteForceTensorHalf (FP16 MQ,
    kernel_join.cu:328-524) on the first n16 rows and ...TensorDouble (FP64
    MQ, kernel_join.cu:530-677) on the first n64 rows of the workload.  Both
    visit all N^2 ordered pairs, so their pairs/s does not depend on N.
    Their totals are not exact (FP16 rounding; races in the reference's
    shared-memory use); the exact total of the same rows is given beside
    them.  None if the kernels were not built (no reference checkout where
    build() ran) or d has no built variant."""
    try:
        from oracle import refgpu
    except ImportError:
        return None
    n, d = x.shape
    if d not in (64, 128) or not refgpu.available(f"fp16_d{d}", f"fp64_d{d}"):
        return None
    out = {}
    for key, variant, kind, rows in (("fp16_mq", f"fp16_d{d}", "mq16", n16),
                                     ("fp64_mq", f"fp64_d{d}", "mq64", n64)):
        m = min(n, rows)
        xs = np.ascontiguousarray(x[:m])
        r = refgpu.run(variant, kind, xs, eps, d, reps=1)
        _, exact, _ = ej.self_join(xs, eps, precision="bf16_split", stream=stream,
                                   device=dev.index)
        out[key] = {"kernel": ("distanceCalculationBruteForceTensorHalf" if kind == "mq16"
                               else "distanceCalculationBruteForceTensorDouble"),
                    "rows": m, "pairs_per_s": m * m / (r["kernel_ms_best"] / 1e3),
                    "kernel_ms": r["kernel_ms_best"], "driver_ms": r["driver_ms_best"],
                    "driver_pairs_per_s": m * m / (r["driver_ms_best"] / 1e3),
                    "total": r["total"], "exact_total": exact,
                    "sample": f"first {m} rows of the workload"}
    return out


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    x, eps, cfg = workload(args)
    n = x.shape[0]
    import oracle

    oracle.build()
    rates = []
    nq = None
    for i in range(args.warmup + args.steps):
        rate, nq, dt, cores = cpu_rate(x, eps, max(1.0, args.cpu_seconds / 3), seed=i)
        if i >= args.warmup:
            rates.append(rate)
    value = statistics.mean(rates)
    line = {
        "impl": "reference", "metric": "pair-distances/s at FP64-exact counts", "value": value,
        "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": n * n / value * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.config}: N={n}, d={x.shape[1]}, eps={eps:.6g}",
                   "n": n, "d": x.shape[1], "eps": eps},
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": oracle.num_threads(),
                         "kind": "port",
                         "sample": f"{nq} seeded query rows x all {n} points per step "
                                   "(reference FP64 predicate, OpenMP over query rows); "
                                   "ms_per_step extrapolates to the full N^2"},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch

    import tensor_bf_main_gb300 as ej

    world, rank, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    x, eps, cfg = workload(args)
    n, d = x.shape
    proj_k = args.proj_k if args.proj_k >= 0 else cfg.get("proj_k", 0)
    if args.precision == "config":
        args.precision = cfg.get("precision", "auto")
    stream = torch.cuda.current_stream(dev)
    xd = torch.from_numpy(x).to(dev)
    cd = torch.empty(n, dtype=torch.int32, device=dev)
    # repeated joins keep the library's scratch cached between calls (what a
    # caller that joins again and again does); the first warm-up call maps it
    kw = dict(precision=args.precision, proj_k=proj_k, counts=cd, stream=stream, device=dev.index,
              keep_scratch=True)

    def barrier():
        if dist:
            dist.barrier()

    clocks = Clocks()
    clocks.start(dev.index)
    for _ in range(args.warmup):
        ej.self_join(xd, eps, **kw)
    barrier()
    torch.cuda.synchronize(dev)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    stats = []
    e0.record(stream)
    for _ in range(args.steps):
        _, total, st = ej.self_join(xd, eps, **kw)
        stats.append(st)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    barrier()
    ck = clocks.stop()
    ms, value = replica_rate(e0.elapsed_time(e1) / args.steps, n, world, dist, dev)

    pk = peaks()
    prec = stats[0]["precision"]
    roof = None if prec in ("fp64_dmma", "fp64_direct") else gram_roofline(stats, d, prec, pk,
                                                                         args, proj_k)

    line = {
        "metric": "pair-distances/s at FP64-exact counts", "value": value, "unit": "pairs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": prec,
        "data": "synthetic (seeded generator with the config's shape and distribution)",
        "config": {"workload": f"{args.config}: N={n}, d={d}, eps={eps:.6g}", "n": n, "d": d,
                   "eps": eps, "precision": prec, "proj_k": proj_k,
                   "l2": "inputs larger than L2 (N*d*8 bytes)", "parallelism": f"replicas x{world}"},
        "total_pairs": int(total),
        "band_fraction": stats[-1]["band_fraction"], "band_pairs": stats[-1]["band_pairs"],
        "tile_pairs_run": stats[-1]["tile_pairs_run"],
        "gram_blocks": stats[-1].get("gram_blocks", 0),
        "exact_rechecks": stats[-1].get("exact_rechecks", 0),
        "band_records": stats[-1].get("band_records", 0),
        "scratch_peak_bytes": stats[-1].get("scratch_peak_bytes", 0),
        "tile_pairs_total": stats[-1]["tile_pairs_total"],
        "phase_ms": {k: stats[-1][k] for k in ("ms_prep", "ms_train", "ms_order", "ms_gram",
                                                "ms_recheck", "ms_total")},
        "algorithmic_tflops": 2.0 * d * n * (n + 1) / 2 / (ms / 1e3) / 1e12,
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "clocks": ck,
    }
    if roof:
        line["roofline"] = roof
        line["tensor_pipe_frac"] = roof["frac"]

    if rank == 0 and not args.no_fp64:
        sub = min(n, args.fp64_rows)
        xs = xd[:sub].contiguous()
        cs = torch.empty(sub, dtype=torch.int32, device=dev)
        ej.self_join(xs, eps, precision="fp64_dmma", counts=cs, stream=stream, device=dev.index)
        torch.cuda.synchronize(dev)
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        ej.self_join(xs, eps, precision="fp64_dmma", counts=cs, stream=stream, device=dev.index)
        f1.record(stream)
        torch.cuda.synchronize(dev)
        fms = f0.elapsed_time(f1)
        rate = sub * sub / (fms / 1e3)
        line["fp64_dmma_join"] = {"value": rate, "unit": "pairs/s",
                                  "sample": f"first {sub} rows, extrapolated as N^2/rate",
                                  "extrapolated_ms_full": n * n / rate * 1e3,
                                  "speedup": value / world / rate}

    if rank == 0 and not args.no_ref_gpu:
        rg = reference_gpu(ej, x, eps, stream, dev)
        if rg:
            line["reference_gpu"] = rg

    if rank == 0 and not args.no_e2e:
        xh = torch.from_numpy(x).pin_memory()
        ch = np.empty(n, dtype=np.int32)
        ej.self_join(xh, eps, precision=args.precision, proj_k=proj_k, counts=ch, stream=stream,
                     keep_scratch=True)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ej.self_join(xh, eps, precision=args.precision, proj_k=proj_k, counts=ch,
                         stream=stream, keep_scratch=True)
        torch.cuda.synchronize(dev)
        e2e_s = (time.perf_counter() - t0) / args.steps
        # the host link on its own: a plain copy of the same pinned rows (the
        # staged join cannot beat it; it varies between boxes with where the
        # pinned pages sit)
        xd2 = torch.empty_like(xd)
        xd2.copy_(xh, non_blocking=True)
        torch.cuda.synchronize(dev)
        c0 = time.perf_counter()
        xd2.copy_(xh, non_blocking=True)
        torch.cuda.synchronize(dev)
        copy_ms = (time.perf_counter() - c0) * 1e3
        del xd2
        line["e2e"] = {"value": float(n) * n / e2e_s, "unit": "pairs/s",
                       "h2d_bytes_per_step": int(n * d * 8), "d2h_bytes_per_step": int(n * 4 + 8),
                       "ms_per_step": e2e_s * 1e3, "plain_h2d_copy_ms": copy_ms,
                       "plain_h2d_gbs": n * d * 8 / copy_ms / 1e6}

    ej.release_scratch(dev.index)

    if rank == 0 and not args.no_cpu_baseline:
        rate, nq, dt, cores = cpu_rate(x, eps, args.cpu_seconds)
        line["cpu_baseline"] = {"value": rate, "unit": "pairs/s", "cores": cores, "kind": "port",
                                "sample": f"{nq} seeded query rows x all {n} points "
                                          f"({dt:.1f} s, oracle restatement of the reference "
                                          "FP64 kernel, OpenMP over query rows)"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
