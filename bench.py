"""Benchmark of the GB300 skeleton library on the plain single-call workload.

One step = one pass of the four full-size single-call skeletons:
  scanl1 (+)  Int64,   2^28 elements uniform in [-2^20, 2^20]
  fold (+) 0  Float32, 2^28 elements ~ N(0,1)       (compensated FP32)
  permute (+) histogram of 2^28 Int32 Zipf(s=1.1) bin indices into 2^16 bins
  stencil 3x3 Float32 (weights 1/9) on 8192 x 8192 ~ U(0,1), clamp boundary
Metric: HBM GB/s = algorithmic bytes / device time (scan 16 B/elem, fold
4 B/elem, permute 4 B/elem + 2 x 4 B per bin, stencil 8 B/elem).  Inputs are
seeded synthetic data of the workload's shapes and distributions, generated
on the device; every input is larger than L2, so no flush is needed.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --only scan|fold|permute|stencil|foldseg|batched|dotp|scanzip|stencil3d|rowscan [--scale S]   (one kernel, small case)

`--impl reference` times the CPU restatement of accelerate-llvm-native (the
reference's own CPU backend cannot be built here) on all host cores over a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_SCAN = 1 << 28
N_FOLD = 1 << 28
N_PERM, M_PERM = 1 << 28, 1 << 16
H_ST = W_ST = 8192
SEED = 0xACCE1 + 1

BYTES = {
    "scan": 16 * N_SCAN,
    "fold": 4 * N_FOLD,
    "permute": 4 * N_PERM + 2 * 4 * M_PERM,
    "stencil": 8 * H_ST * W_ST,
}
# DRAM bytes per full-size launch of each skeleton's kernel:
# dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of the
# `bench.py --only <skeleton> --scale <s>` small case, scaled by the units
# processed to the full launch (traffic grows in proportion; the stencil case
# is already full size).  Summaries with the commands sit in profiles/.
NCU_TRAFFIC = {
    "scan": int((270.588416e6 + 207.724288e6) * 8),   # 2^25 Int64 -> 2^28 (scan_l2_kernel)
    "fold": int((268.478208e6 + 2.757376e6) * 4),     # 2^26 Float32 -> 2^28
    "permute": int((268.722688e6 + 2.906368e6) * 4),  # 2^26 indices -> 2^28
    "stencil": int(292.122624e6 + 222.595328e6),      # 8192^2, full size
}

# foldSeg workload: 2^26 Float32 values ~ N(0,1) in 2^20 segments with
# lognormal lengths (median 48, sigma 1.5, capped at 2^16, 2 % empty),
# rescaled by largest remainder so that the lengths sum to 2^26; plus Int32
# `max` over the same segmentation.  Bytes: values + offsets + results.
N_SEG_VALUES, N_SEGS = 1 << 26, 1 << 20
BYTES_FOLDSEG = 4 * N_SEG_VALUES + 4 * (N_SEGS + 1) + 4 * N_SEGS


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------- clocks
class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- inputs
def make_inputs(torch, dev, scale=1):
    g = torch.Generator(device=dev)
    g.manual_seed(SEED)
    n_scan, n_fold, n_perm = N_SCAN // scale, N_FOLD // scale, N_PERM // scale
    h = H_ST // int(np.sqrt(scale))
    x_scan = torch.randint(-(1 << 20), (1 << 20) + 1, (n_scan,), dtype=torch.int64, device=dev, generator=g)
    x_fold = torch.randn(n_fold, dtype=torch.float32, device=dev, generator=g)
    ranks = torch.arange(1, M_PERM + 1, dtype=torch.float64, device=dev)
    p = ranks.pow(-1.1)
    cdf = torch.cumsum(p / p.sum(), 0)
    perm = torch.randperm(M_PERM, device=dev, generator=g).to(torch.int32)
    idx = torch.empty(n_perm, dtype=torch.int32, device=dev)
    chunk = 1 << 26
    for s in range(0, n_perm, chunk):
        u = torch.rand(min(chunk, n_perm - s), dtype=torch.float64, device=dev, generator=g)
        r = torch.searchsorted(cdf, u).clamp_(max=M_PERM - 1)
        idx[s:s + u.numel()] = perm[r]
        del u, r
    grid = torch.rand((h, h), dtype=torch.float32, device=dev, generator=g)
    return {"scan": x_scan, "fold": x_fold, "idx": idx, "grid": grid}


def make_segments(torch, dev, n_values=N_SEG_VALUES, nseg=N_SEGS):
    """Lognormal(median 48, sigma 1.5) lengths capped at 2^16 with 2 % empty,
    rescaled by largest remainder to sum to n_values; returns Int32 offsets."""
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 3)
    lens = torch.empty(nseg, dtype=torch.float64, device=dev).log_normal_(float(np.log(48.0)), 1.5, generator=g)
    lens.clamp_(max=float(1 << 16))
    lens[torch.rand(nseg, device=dev, generator=g) < 0.02] = 0.0
    lens *= n_values / lens.sum()
    fl = torch.floor(lens)
    rem = int(n_values - int(fl.sum().item()))
    order = torch.argsort(lens - fl, descending=True)
    fl[order[:rem]] += 1.0
    off = torch.zeros(nseg + 1, dtype=torch.int64, device=dev)
    off[1:] = torch.cumsum(fl.to(torch.int64), 0)
    vals = torch.randn(n_values, dtype=torch.float32, device=dev, generator=g)
    ivals = torch.randint(-(1 << 31), (1 << 31) - 1, (n_values,), dtype=torch.int32, device=dev, generator=g)
    return off.to(torch.int32), vals, ivals


W9 = [[1.0 / 9] * 3] * 3


# ----------------------------------------------------------------- our arm
def run_ours(args, rank, world):
    import torch
    import __graft_entry__ as ge

    dev = torch.device("cuda", rank % max(1, torch.cuda.device_count()))
    torch.cuda.set_device(dev)
    acc = ge.load_package()
    acc.load()
    inp = make_inputs(torch, dev)
    zeros = torch.zeros(M_PERM, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    names = ["scan", "fold", "permute", "stencil"]
    launches_per_step = 4  # one kernel per skeleton (the permute clone is a copy, not a kernel)

    def step(ev=None):
        outs = {}
        for i, nm in enumerate(names):
            if ev is not None:
                ev[nm][0].record(stream)
            if nm == "scan":
                outs[nm] = acc.scanl1("+", inp["scan"])
            elif nm == "fold":
                outs[nm] = acc.fold("+", 0.0, inp["fold"])
            elif nm == "permute":
                outs[nm] = acc.permute("+", zeros, inp["idx"], 1)
            else:
                outs[nm] = acc.stencil(W9, inp["grid"], "clamp")
            if ev is not None:
                ev[nm][1].record(stream)
        return outs

    for _ in range(args.warmup):
        step()
    acc.sync()
    dist_barrier(world)
    torch.cuda.synchronize()

    ev = [{nm: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for nm in names}
          for _ in range(args.steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    with Clocks(dev.index) as clk:
        t0.record(stream)
        for k in range(args.steps):
            step(ev[k])
        t1.record(stream)
        torch.cuda.synchronize()
    acc.sync()
    dist_barrier(world)
    total_ms = t0.elapsed_time(t1)
    per = {nm: [e[nm][0].elapsed_time(e[nm][1]) for e in ev] for nm in names}
    total_ms = dist_max(world, total_ms)

    # ---- correctness spot check of the timed outputs (cheap, device-side)
    outs = step()
    torch.cuda.synchronize()
    assert int(outs["permute"].sum().item()) == N_PERM
    assert int(outs["scan"][-1].item()) == int(inp["scan"].sum().item())

    # ---- end to end through the public API with host buffers (measured first,
    # before the other workloads allocate host and device memory)
    e2e = run_e2e(torch, acc, inp, zeros, args, dev)

    # ---- foldSeg and batched workloads (reported beside the metric, not part of `value`)
    extra = {"foldseg": run_foldseg(torch, acc, args, dev), "dotp": run_dotp(torch, acc, inp, args, dev),
             "precision": run_precision(torch, acc, inp, dev)}
    if not args.no_batch:
        extra["batched"] = run_batched(torch, acc, args, dev)
    if args.serve_seconds > 0:
        extra["serving"] = run_serving(torch, acc, args, dev)

    peak, peak_kind = peaks()
    step_bytes = sum(BYTES.values())
    ms_per_step = total_ms / args.steps
    value = whole_job_gbs(world, step_bytes, ms_per_step)
    scan_ms = statistics.mean(per["scan"])
    achieved = BYTES["scan"] / (scan_ms * 1e-3) / 1e9
    per_sk = {}
    for nm in names:
        ms = statistics.mean(per[nm])
        gbs = BYTES[nm] / (ms * 1e-3) / 1e9
        per_sk[nm] = {"ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / peak, 3),
                      "traffic": NCU_TRAFFIC[nm]}
    clocks = clk.summary()
    line = {
        "metric": "HBM GB/s per skeleton vs peak (plain single-call kernels at full size)",
        "value": round(value, 1),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int64+f32+i32",
        "data": "synthetic (seeded, on device): Int64 U[-2^20,2^20], Float32 N(0,1), Int32 Zipf(1.1) bins, Float32 U(0,1)",
        "config": workload_config(world),
        "per_skeleton": per_sk,
        "extra": extra,
        "roofline": {"bound": "hbm", "kernel": "scan_l2_kernel (scanl1 + Int64)", "achieved": round(achieved, 1),
                     "peak": peak, "peak_kind": f"{peak_kind} hbm_gbs (copy)", "unit": "GB/s",
                     "frac": round(achieved / peak, 3),
                     "traffic": NCU_TRAFFIC["scan"]},
        "e2e": e2e,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
    }
    # The CPU baseline is timed once, on rank 0 of a single-GPU run: with more
    # replicas the other GPUs would sit idle while the host cores are busy.
    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.cpu_scale)
    return line


def run_foldseg(torch, acc, args, dev):
    """foldSeg (+) Float32 compensated, plain and FP64-accumulated, and foldSeg max Int32, on the lognormal
    segmentation; device time per call and HBM GB/s (values + offsets + results)."""
    off, vals, ivals = make_segments(torch, dev)
    peak, _ = peaks()
    stream = torch.cuda.current_stream()
    res = {}
    runs = {"f32_add_compensated": lambda: acc.fold_seg("+", 0.0, vals, off),
            "f32_add_plain": lambda: acc.fold_seg("+", 0.0, vals, off, prec="plain"),
            "f32_add_fp64acc": lambda: acc.fold_seg("+", 0.0, vals, off, prec="fp64"),
            "i32_max": lambda: acc.fold_seg("max", -(1 << 31), ivals, off)}
    for name, fn in runs.items():
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        gbs = BYTES_FOLDSEG / (ms * 1e-3) / 1e9
        res[name] = {"ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / peak, 3)}
    acc.sync()
    res["workload"] = "foldSeg over 2^26 values in 2^20 lognormal segments (median 48, sigma 1.5, 2% empty)"
    return res


def run_dotp(torch, acc, inp, args, dev):
    """dotp xs ys = fold (+) 0 (zipWith (*) xs ys) on Float32 2^28 with the
    zipWith fused into the fold (compensated accumulation): 8 B/element."""
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 9)
    xs = inp["fold"]
    ys = torch.randn(xs.numel(), dtype=torch.float32, device=dev, generator=g)
    stream = torch.cuda.current_stream()
    for _ in range(max(1, args.warmup)):
        acc.dotp(xs, ys)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        acc.dotp(xs, ys)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    got = float(acc.dotp(xs, ys).item())
    ref = float((xs.double() * ys.double()).sum().item())
    acc.sync()
    gbs = 8 * xs.numel() / (ms * 1e-3) / 1e9
    peak, _ = peaks()
    return {"ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / peak, 3),
            "rel_err_vs_fp64": abs(got - ref) / abs(ref),
            "workload": "dotp Float32 2^28 x 2 (fused zipWith (*) -> fold (+) 0, compensated)"}


def run_precision(torch, acc, inp, dev):
    """Float32 (+) accuracy of the three accumulation modes against an FP64
    reference on the device: fold over the 2^28 bench input, scanl1 over its
    first 2^26 elements, foldSeg over the lognormal segmentation.  Errors are
    relative to the FP64 result and to the sum of magnitudes (the condition of
    the sum); for scan and foldSeg the maximum over prefixes / segments."""
    x = inp["fold"]
    ref = x.double().sum()
    mag = x.double().abs().sum()
    res = {}
    for mode in ("compensated", "plain", "fp64"):
        got = acc.fold("+", 0.0, x, prec=mode).double().reshape(())
        res.setdefault("fold_2^28", {})[mode] = {
            "rel_err": float(abs(got - ref) / abs(ref)), "err_over_sum_abs": float(abs(got - ref) / mag)}
    xs = x[: 1 << 26]
    ref_s = torch.cumsum(xs.double(), 0)
    mag_s = torch.cumsum(xs.double().abs(), 0)
    for mode in ("compensated", "plain", "fp64"):
        got = acc.scanl1("+", xs, prec=mode).double()
        err = (got - ref_s).abs()
        res.setdefault("scanl1_2^26", {})[mode] = {
            "max_err_over_prefix_sum_abs": float((err / mag_s).max()),
            "last_rel_err": float(err[-1] / ref_s[-1].abs())}
        del got, err
    del ref_s, mag_s
    off, vals, _ = make_segments(torch, dev)
    o = off.long()
    cs = torch.zeros(vals.numel() + 1, dtype=torch.float64, device=dev)
    cs[1:] = torch.cumsum(vals.double(), 0)
    ca = torch.zeros_like(cs)
    ca[1:] = torch.cumsum(vals.double().abs(), 0)
    ref_g = cs[o[1:]] - cs[o[:-1]]
    mag_g = ca[o[1:]] - ca[o[:-1]]
    nz = mag_g > 0
    for mode in ("compensated", "plain", "fp64"):
        got = acc.fold_seg("+", 0.0, vals, off, prec=mode).double()
        err = (got - ref_g).abs()
        res.setdefault("foldSeg_2^26_in_2^20", {})[mode] = {
            "max_err_over_seg_sum_abs": float((err[nz] / mag_g[nz]).max()),
            "max_abs_err": float(err.max())}
    acc.sync()
    res["reference"] = "torch float64 sum / cumsum on the device"
    return res


def batched_requests(torch, dev, count):
    """`count` independent requests, a quarter each of fold (+) and scanl1 (+)
    on Int32 and on Float32, sizes log-uniform in [2^8, 2^22]; returns the
    requests and their algorithmic bytes (fold 4n, scan 8n)."""
    rng = np.random.default_rng(SEED + 4)
    sizes = np.exp(rng.uniform(np.log(2 ** 8), np.log(2 ** 22), size=count)).astype(np.int64)
    kinds = ["fold", "scan", "fold", "scan"] * (count // 4)
    dts = [torch.int32, torch.int32, torch.float32, torch.float32] * (count // 4)
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 5)
    tot = {torch.int32: 0, torch.float32: 0}
    for n, dt in zip(sizes, dts):
        tot[dt] += int(n)
    pool = {torch.int32: torch.randint(-1000, 1000, (tot[torch.int32],), dtype=torch.int32, device=dev, generator=g),
            torch.float32: torch.randn(tot[torch.float32], dtype=torch.float32, device=dev, generator=g)}
    at = {torch.int32: 0, torch.float32: 0}
    reqs, nbytes = [], 0
    for n, dt, kind in zip(sizes, dts, kinds):
        n = int(n)
        xs = pool[dt][at[dt]:at[dt] + n]
        at[dt] += n
        out = torch.empty((1,) if kind == "fold" else (n,), dtype=dt, device=dev)
        reqs.append((kind, xs, out, 0 if kind == "fold" else None))
        nbytes += 4 * n if kind == "fold" else 8 * n
    return reqs, nbytes


def run_batched(torch, acc, args, dev, count=10_000):
    """10,000 requests (batched_requests): one persistent launch replayed as a
    CUDA graph (tiles from the autotuner) against the same requests as 10,000
    per-call launches."""
    reqs, nbytes = batched_requests(torch, dev, count)
    table = ROOT / "accelerate-llvm_gb300" / "_build" / "batch_tuning.json"
    t_tune = time.perf_counter()
    if table.exists():
        acc.batch_load_tuning(table)
        tuned = "loaded"
    else:
        table.parent.mkdir(exist_ok=True)
        acc.batch_autotune(str(table))
        tuned = "autotuned"
    t_tune = time.perf_counter() - t_tune
    b = acc.Batch("+", reqs)
    b.capture()
    stream = torch.cuda.current_stream()
    for _ in range(max(1, args.warmup)):
        b.launch()
    b.status()
    reps = max(3, args.steps)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.launch()
    e1.record(stream)
    torch.cuda.synchronize()
    b.status()
    ms_batch = e0.elapsed_time(e1) / reps
    batched_out = [r[2].clone() for r in reqs[:8]]
    b.close()

    def per_call():
        for kind, xs, out, z in reqs:
            if kind == "fold":
                acc.fold("+", z, xs)
            else:
                acc.scanl1("+", xs)

    per_call()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    e0.record(stream)
    per_call()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_call = max(e0.elapsed_time(e1), (time.perf_counter() - w0) * 1e3)
    acc.sync()
    for (kind, xs, out, z), got in zip(reqs[:8], batched_out):
        ref = acc.fold("+", z, xs).reshape(1) if kind == "fold" else acc.scanl1("+", xs)
        if xs.dtype == torch.int32:
            assert torch.equal(got, ref)
    return {"requests": count, "bytes": nbytes, "tiles": tuned, "tune_s": round(t_tune, 2),
            "batched_graph": {"ms": round(ms_batch, 3), "req_per_s": round(count / (ms_batch * 1e-3)),
                              "gbs": round(nbytes / (ms_batch * 1e-3) / 1e9, 1)},
            "per_call": {"ms": round(ms_call, 3), "req_per_s": round(count / (ms_call * 1e-3)),
                         "gbs": round(nbytes / (ms_call * 1e-3) / 1e9, 1)},
            "speedup": round(ms_call / ms_batch, 2)}


def request_bytes(r):
    """Algorithmic bytes of one serving request (inputs read + outputs written)."""
    k, xs, aux, out, n, m, t = r[:7]
    e = xs.element_size()
    if k == "fold":
        return n * e + e
    if k == "scan":
        return 2 * n * e
    if k == "foldseg":
        return n * e + 4 * (m + 1) + m * e
    if k == "permute":
        return 4 * n + 2 * 4 * m
    return 2 * n * m * e


def serving_stream(torch, dev, count, rate, rng, pools, check_every=0):
    """Mixed requests: 40 % fold, 25 % scanl1, 15 % foldSeg (lognormal
    segments), 10 % permute histograms into 2^12..2^16 bins, 10 % 5-point
    Float32 stencils on 256^2..4096^2 grids; sizes log-uniform in
    [2^10, 2^26]; Poisson arrivals at `rate` per second (rate 0: all at
    t = 0).  Inputs are slices of device-resident pools; every result is
    placed by the serving loop in its device arena (output None).  With
    `check_every` > 0, every check_every-th request whose result has at most
    2^20 elements also gets a host array that its result is copied back to."""
    vals, ivals, off, idx, offs_np = pools
    kinds = rng.choice(["fold", "scan", "foldseg", "permute", "stencil"], size=count, p=[0.4, 0.25, 0.15, 0.1, 0.1])
    sizes = np.exp(rng.uniform(np.log(2 ** 10), np.log(2 ** 26), size=count)).astype(np.int64)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count)) if rate > 0 else np.zeros(count)
    reqs = []
    for i in range(count):
        k, n = kinds[i], int(sizes[i])
        if k in ("fold", "scan"):
            xs = (vals if i % 2 else ivals)[:n]
            r = [k, xs, None, None, n, 0, float(t[i])]
            nres, dt = (1 if k == "fold" else n), xs.dtype
        elif k == "foldseg":
            nseg = int(np.searchsorted(offs_np, n, side="right")) - 1
            nv = int(offs_np[nseg])
            r = [k, vals[:nv], off, None, nv, nseg, float(t[i])]
            nres, dt = nseg, torch.float32
        elif k == "permute":
            m = int(2 ** rng.integers(12, 17))
            r = [k, idx[m][:n], None, None, n, m, float(t[i])]
            nres, dt = m, torch.int32
        else:
            side = int(np.exp(rng.uniform(np.log(256), np.log(4096))))
            r = [k, vals[:side * side].view(side, side), None, None, side, side, float(t[i])]
            nres, dt = side * side, torch.float32
        if check_every and i % check_every == 0 and 0 < nres <= (1 << 20):
            r.append(np.empty(nres, dtype={torch.float32: np.float32, torch.int32: np.int32}[dt]))
        reqs.append(tuple(r))
    return reqs


def check_served(torch, dev, reqs):
    """Every result copied back to a host array against a float64 / int64
    restatement computed with torch on the device: integers exact (wrapping
    Int32 sums), Float32 sums within 1e-6 |ref| + 1e-9 sum|x|, the stencil
    within 1e-6 of the grid's magnitude.  Returns the number checked."""
    checked = 0
    for r in reqs:
        if len(r) < 8:
            continue
        k, xs, aux, _, n, m, _, host = r
        got = torch.from_numpy(host).to(dev)
        if k == "permute":
            ref = torch.bincount(xs.long(), minlength=m).to(torch.int32)
            assert torch.equal(got, ref), "served permute differs"
        elif k == "stencil":
            g = torch.nn.functional.pad(xs.double()[None, None], (1, 1, 1, 1), mode="replicate")[0, 0]
            ref = 0.25 * (g[:-2, 1:-1] + g[2:, 1:-1] + g[1:-1, :-2] + g[1:-1, 2:]) - g[1:-1, 1:-1]
            assert float((got.double().view(n, m) - ref).abs().max()) <= 1e-6 * (1 + float(xs.abs().max())), \
                "served stencil differs"
        elif xs.dtype == torch.int32:
            x64 = xs.long()
            ref = (x64.sum().view(1) if k == "fold" else torch.cumsum(x64, 0))
            ref = ((ref + (1 << 31)) % (1 << 32) - (1 << 31)).to(torch.int32)
            assert torch.equal(got, ref), f"served Int32 {k} differs"
        else:
            x64 = xs.double()
            if k == "fold":
                ref, absum = x64.sum().view(1), x64.abs().sum().view(1)
            elif k == "scan":
                ref, absum = torch.cumsum(x64, 0), torch.cumsum(x64.abs(), 0)
            else:
                o = aux[: m + 1].long()
                seg = torch.repeat_interleave(torch.arange(m, device=dev), o[1:] - o[:-1])
                xv = x64[: int(o[-1])]
                ref = torch.zeros(m, dtype=torch.float64, device=dev).index_add_(0, seg, xv)
                absum = torch.zeros(m, dtype=torch.float64, device=dev).index_add_(0, seg, xv.abs())
            err = (got.double() - ref).abs()
            assert bool((err <= 1e-6 * ref.abs() + 1e-9 * absum + 1e-30).all()), f"served {k} differs"
        checked += 1
    return checked


def run_serving(torch, acc, args, dev):
    """The serving stream at 20k req/s for --serve-seconds, through the
    continuous-batching loop and through plain per-call launches; then each
    scheduler's capacity with every request arriving at once.  Results are
    placed by the loop in a device arena of the 40 GB budget (admission
    waits for room); a sample of them is copied back and checked."""
    rng = np.random.default_rng(SEED + 6)
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 7)
    n_pool = 1 << 26
    vals = torch.randn(n_pool, dtype=torch.float32, device=dev, generator=g)
    ivals = torch.randint(-1000, 1000, (n_pool,), dtype=torch.int32, device=dev, generator=g)
    off, _, _ = make_segments(torch, dev, n_pool, 1 << 20)
    idx = {m: torch.randint(0, m, (n_pool,), dtype=torch.int32, device=dev, generator=g) for m in [1 << b for b in range(12, 17)]}
    pools = (vals, ivals, off, idx, off.cpu().numpy().astype(np.int64))
    budget = 40 << 30
    res = {"rate_req_s": 20000, "seconds": args.serve_seconds, "budget_bytes": budget, "slots": 8,
           "results": "placed by the loop in a device arena of the budget; admission waits for room"}
    count = int(20000 * args.serve_seconds)
    stream = serving_stream(torch, dev, count, 20000.0, rng, pools, check_every=997)
    for mode in ("batching", "per_call"):
        lat, st = acc.serve(stream, budget, slots=8, mode=mode)
        lat = np.array(lat)
        res[mode] = {"served": st["served"], "wall_s": round(st["wall_s"], 3),
                     "req_per_s": round(st["served"] / st["wall_s"]),
                     "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
                     "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3),
                     "batches": st["batches"], "max_inflight": st["max_inflight"],
                     "peak_arena_bytes": st["peak_bytes"],
                     "checked": check_served(torch, dev, stream)}
    cap_n = min(count, 20000)
    burst = serving_stream(torch, dev, cap_n, 0.0, np.random.default_rng(SEED + 8), pools)
    burst_bytes = sum(request_bytes(r) for r in burst)
    peak, _ = peaks()
    res["capacity_burst"] = {"requests": cap_n, "bytes": burst_bytes,
                             "roofline_ms": round(burst_bytes / (peak * 1e9) * 1e3, 2)}
    for mode in ("batching", "per_call"):
        lat, st = acc.serve(burst, budget, slots=8, mode=mode)
        res[mode]["capacity_req_s"] = round(st["served"] / st["wall_s"])
        res[mode]["capacity_gbs"] = round(burst_bytes / st["wall_s"] / 1e9, 1)
    res["capacity_ratio"] = round(res["batching"]["capacity_req_s"] / res["per_call"]["capacity_req_s"], 2)
    # The most any scheduler could reach on this byte mix: every request at
    # the HBM roofline, against the per-call rate.
    res["capacity_ratio_ceiling"] = round(cap_n / (burst_bytes / (peak * 1e9)) / res["per_call"]["capacity_req_s"], 2)
    acc.sync()
    return res


def run_only(args):
    """One skeleton at 1/scale of its full size, `--steps` launches: the
    small-case command used for ncu captures."""
    import torch
    import __graft_entry__ as ge
    dev = torch.device("cuda", 0)
    acc = ge.load_package()
    acc.load()
    name = args.only
    stream = torch.cuda.current_stream()
    if name == "rowscan":
        return run_rowscan(torch, acc, args, dev)
    if name == "foldseg":
        off, vals, ivals = make_segments(torch, dev, N_SEG_VALUES // args.scale, N_SEGS // args.scale)
        fn, nbytes = (lambda: acc.fold_seg("+", 0.0, vals, off)), BYTES_FOLDSEG // args.scale
    elif name == "batched":
        # 10,000 / scale requests in one persistent launch (built-in tile sizes, no graph)
        reqs, nbytes = batched_requests(torch, dev, 10_000 // args.scale)
        b = acc.Batch("+", reqs)
        fn = b.launch
    elif name == "dotp":
        g = torch.Generator(device=dev)
        g.manual_seed(SEED + 9)
        xs = torch.randn(N_FOLD // args.scale, dtype=torch.float32, device=dev, generator=g)
        ys = torch.randn(N_FOLD // args.scale, dtype=torch.float32, device=dev, generator=g)
        fn, nbytes = (lambda: acc.dotp(xs, ys)), 8 * xs.numel()
    elif name == "stencil3d":
        # 3x3x3 Float32 stencil (weights 1/27) on a 512^3 grid / scale, clamp:
        # 8 B/element (read + write)
        g = torch.Generator(device=dev)
        g.manual_seed(SEED + 11)
        side = max(8, int(round(512 / args.scale ** (1.0 / 3.0))))
        grid3 = torch.rand((side, side, side), dtype=torch.float32, device=dev, generator=g)
        w27 = [[[1.0 / 27] * 3] * 3] * 3
        fn, nbytes = (lambda: acc.stencil3d(w27, grid3, "clamp")), 8 * grid3.numel()
    elif name == "scanzip":
        # scanl1 (+) (zipWith (*) xs ys) on Float32 with the zipWith fused into
        # the scan: 12 B/element (two reads, one write)
        g = torch.Generator(device=dev)
        g.manual_seed(SEED + 10)
        xs = torch.randn(N_FOLD // args.scale, dtype=torch.float32, device=dev, generator=g)
        ys = torch.randn(N_FOLD // args.scale, dtype=torch.float32, device=dev, generator=g)
        zout = acc.scan_zipwith("scanl1", "+", "*", None, xs, ys)
        ref = torch.cumsum(xs.double() * ys.double(), 0)
        err = float(((zout.double() - ref).abs() / torch.cumsum((xs.double() * ys.double()).abs(), 0)).max())
        assert err < 1e-6, f"scanl1 (+) (zipWith (*)) error {err}"
        del ref
        fn, nbytes = (lambda: acc.scan_zipwith("scanl1", "+", "*", None, xs, ys)), 12 * xs.numel()
    else:
        inp = make_inputs(torch, dev, args.scale)
        zeros = torch.zeros(M_PERM, dtype=torch.int32, device=dev)
        fn = {"scan": lambda: acc.scanl1("+", inp["scan"]), "fold": lambda: acc.fold("+", 0.0, inp["fold"]),
              "permute": lambda: acc.permute("+", zeros, inp["idx"], 1),
              "stencil": lambda: acc.stencil(W9, inp["grid"], "clamp")}[name]
        h = inp["grid"].shape[0]
        nbytes = {"scan": 16 * inp["scan"].numel(), "fold": 4 * inp["fold"].numel(),
                  "permute": 4 * inp["idx"].numel() + 8 * M_PERM, "stencil": 8 * h * h}[name]
    for _ in range(args.warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    acc.sync()
    ms = e0.elapsed_time(e1) / args.steps
    return {"only": name, "scale": args.scale, "ms": round(ms, 4), "gbs": round(nbytes / (ms * 1e-3) / 1e9, 1)}


def run_rowscan(torch, acc, args, dev):
    """scanl1 (+) over the rows of Int64 arrays of 2^28 / scale elements in
    four shapes (long rows to many short ones), 16 B per element (read +
    write), `--steps` calls each after `--warmup`."""
    total = (1 << 28) // args.scale
    res = {"only": "rowscan", "scale": args.scale, "shapes": {}}
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 12)
    x = torch.randint(-(1 << 20), 1 << 20, (total,), dtype=torch.int64, device=dev, generator=g)
    stream = torch.cuda.current_stream()
    for inner in (1 << 14, 1 << 18, 1 << 10, 1 << 8):
        xs = x.view(total // inner, inner)
        for _ in range(max(1, args.warmup)):
            acc.scanl1("+", xs)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            acc.scanl1("+", xs)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        res["shapes"][f"{total // inner}x{inner}"] = {"ms": round(ms, 4), "gbs": round(16 * total / (ms * 1e-3) / 1e9, 1)}
    acc.sync()
    return res


def link_rates(torch, dev, nbytes=1 << 30, trials=5):
    """This machine's host link with pinned buffers: H2D alone, D2H alone, and
    both at once (bytes of both directions over the time), each the best of
    several trials after a warm copy (the link's rate varies a little from
    moment to moment)."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    h2 = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    d2 = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def best(fn, moved):
        fn()
        torch.cuda.synchronize()
        top = 0.0
        for _ in range(trials):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s1)
            s2.wait_event(a)
            fn()
            s1.wait_stream(s2)
            b.record(s1)
            torch.cuda.synchronize()
            top = max(top, moved / (a.elapsed_time(b) * 1e-3) / 1e9)
        return top

    def up():
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)

    def down():
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    def both():
        up()
        down()

    r = {"h2d_gbs": best(up, nbytes), "d2h_gbs": best(down, nbytes), "both_gbs": best(both, 2 * nbytes)}
    del h, h2, d, d2
    return r


def run_e2e(torch, acc, inp, zeros, args, dev):
    """The same step end to end through the library's public API with host
    buffers (pinned): every step copies each input from host memory into its
    device copy in a memory table (acc_table_poke), runs the four skeletons
    on the device copies through the C ABI (acc_scan, acc_fold,
    acc_permute_clone, acc_stencil2d) and copies every result back to host
    memory (acc_table_peek).  The table's upload and download streams overlap
    the copies with each other and with the kernels; the skeletons go in the
    order scan, fold, permute, stencil, so that the scan's 2 GiB result
    drains while the other inputs upload.  Device time from the first upload
    to the last download (CUDA events; the compute stream joins the table's
    streams at the end)."""
    import ctypes
    lib = acc.lib()
    host = {k: v.cpu().pin_memory() for k, v in inp.items()}
    host_zeros = zeros.cpu().pin_memory()
    order = [("scan", "scan"), ("fold", "fold"), ("permute", "idx"), ("stencil", "grid")]
    h2d = sum(v.numel() * v.element_size() for v in host.values())
    res_host = {
        "scan": torch.empty(N_SCAN, dtype=torch.int64).pin_memory(),
        "fold": torch.empty((), dtype=torch.float32).pin_memory(),
        "permute": torch.empty(M_PERM, dtype=torch.int32).pin_memory(),
        "stencil": torch.empty((H_ST, W_ST), dtype=torch.float32).pin_memory(),
    }
    d2h = sum(v.numel() * v.element_size() for v in res_host.values())
    budget = h2d + d2h + host_zeros.numel() * 4 + (64 << 20)
    tb = acc.Table(budget)
    stream = torch.cuda.Stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    zero_f = ctypes.c_float(0.0)
    one_i = ctypes.c_int32(1)
    w9 = (ctypes.c_float * 9)(*[v for r in W9 for v in r])
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    d_zeros = tb.use(host_zeros, stream)  # resident defaults of the histogram, uploaded once

    def run_skeleton(name, din, dout):
        if name == "scan":
            st = lib.acc_scan(acc.ADD, acc.I64, 0, 0, 0, vp(din), vp(dout), None, 1, N_SCAN, None, sp)
        elif name == "fold":
            st = lib.acc_fold(acc.ADD, acc.F32, 0, vp(din), vp(dout), 1, N_FOLD,
                              ctypes.cast(ctypes.pointer(zero_f), ctypes.c_void_p), sp)
        elif name == "permute":
            st = lib.acc_permute_clone(acc.ADD, acc.I32, vp(d_zeros), None,
                                       ctypes.cast(ctypes.pointer(one_i), ctypes.c_void_p), vp(din),
                                       acc.I32, vp(dout), N_PERM, M_PERM, sp)
        else:
            st = lib.acc_stencil2d(acc.F32, 1, 1, ctypes.cast(w9, ctypes.c_void_p), acc.CLAMP, None,
                                   vp(din), vp(dout), H_ST, W_ST, sp)
        if st != 0:
            raise acc.AccError(st, name)

    def step(first=False, kev=None):
        for name, key in order:
            din = tb.use(host[key], stream)  # uploads on the first step only
            if not first:
                tb.poke(host[key], stream)   # every step: this step's input
            dout = tb.malloc(res_host[name], stream)
            if kev is not None:
                kev.append((name, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)))
                kev[-1][1].record(stream)
            run_skeleton(name, din, dout)
            if kev is not None:
                kev[-1][2].record(stream)
            tb.release(host[key], stream)
            tb.release(res_host[name], stream)
            tb.peek(res_host[name], stream)

    step(first=True)
    for _ in range(max(1, args.warmup // 2)):
        step()
    tb.join(stream)
    torch.cuda.synchronize()
    steps = max(2, args.steps // 2)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    w0 = time.perf_counter()
    t0.record(stream)
    for _ in range(steps):
        step()
    tb.join(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - w0) * 1e3 / steps
    acc.sync(stream)
    ms = t0.elapsed_time(t1) / steps
    # the results that came back are the step's
    assert int(res_host["scan"][-1]) == int(inp["scan"].sum().item())
    assert int(res_host["permute"].sum()) == N_PERM
    # Timeline of two more steps: every transfer of the table (its trace) and
    # every kernel (events on the compute stream), in ms after one origin.
    tb.trace(True)
    origin = torch.cuda.Event(enable_timing=True)
    origin.record(stream)
    kev = []
    for _ in range(2):
        step(kev=kev)
    tb.join(stream)
    torch.cuda.synchronize()
    timeline = [("kernel " + nm, 0, round(origin.elapsed_time(a), 3), round(origin.elapsed_time(b), 3))
                for nm, a, b in kev]
    timeline += [(kind, nb, round(a, 3), round(b, 3)) for kind, nb, a, b in tb.trace_records(origin)]
    timeline.sort(key=lambda r: r[2])
    tb.trace(False)
    stats = tb.stats()
    tb.close()
    # The host link's rates, measured after the timed steps: on a GB300 a
    # probe of fresh pinned buffers run before them left every later step at
    # about half the link's rate (58 ms instead of 24.5 ms per step).
    link = link_rates(torch, dev)
    bound_ms = max(h2d / (link["h2d_gbs"] * 1e9), d2h / (link["d2h_gbs"] * 1e9),
                   (h2d + d2h) / (link["both_gbs"] * 1e9)) * 1e3
    return {"value": round(sum(BYTES.values()) / (ms * 1e-3) / 1e9, 1), "unit": "GB/s", "ms_per_step": round(ms, 3),
            "wall_ms_per_step": round(wall_ms, 3),
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "link": {k: round(v, 1) for k, v in link.items()} | {
                "bound_ms_per_step": round(bound_ms, 2), "frac_of_link_bound": round(bound_ms / ms, 3)},
            "table": {"uploads": stats["uploads"], "downloads": stats["downloads"], "hits": stats["hits"],
                      "evictions": stats["evictions"]},
            "timeline_two_steps": timeline,
            "path": "C ABI: acc_table_use/poke/malloc/peek/release (memory table; pinned host buffers; "
                    "upload and download streams of the table) + acc_scan/acc_fold/acc_permute_clone/"
                    "acc_stencil2d on the device copies"}


# ----------------------------------------------------------------- CPU arm
def cpu_inputs(scale):
    rng = np.random.default_rng(SEED)
    n_scan, n_fold, n_perm = N_SCAN // scale, N_FOLD // scale, N_PERM // scale
    h = int(H_ST / np.sqrt(scale))
    x_scan = rng.integers(-(1 << 20), (1 << 20) + 1, size=n_scan, dtype=np.int64)
    x_fold = rng.standard_normal(n_fold, dtype=np.float32)
    p = 1.0 / np.arange(1, M_PERM + 1) ** 1.1
    cdf = np.cumsum(p / p.sum())
    perm = rng.permutation(M_PERM).astype(np.int32)
    # Inverse CDF through a table of 2^24 equal-probability cells (each cell
    # holds the bin of its midpoint): the same Zipf(1.1) law to within 2^-24
    # per bin, at one table lookup per index instead of a binary search.
    cells = np.minimum(np.searchsorted(cdf, (np.arange(1 << 24) + 0.5) / (1 << 24)), M_PERM - 1)
    table = perm[cells]
    idx = np.empty(n_perm, dtype=np.int32)
    chunk = 1 << 24
    for s0 in range(0, n_perm, chunk):
        k = min(chunk, n_perm - s0)
        idx[s0:s0 + k] = table[rng.integers(0, 1 << 24, size=k, dtype=np.int32)]
    grid = rng.random((h, h), dtype=np.float32)
    return {"scan": x_scan, "fold": x_fold, "idx": idx, "grid": grid, "h": h}


def cpu_step(orc, inp, nth):
    """One pass of the four skeletons on the host; returns seconds per skeleton."""
    t = {}
    s = time.perf_counter(); orc.scan("+", None, inp["scan"], 0, 0, nthreads=nth); t["scan"] = time.perf_counter() - s
    s = time.perf_counter(); orc.fold("+", np.float32(0), inp["fold"], nthreads=nth); t["fold"] = time.perf_counter() - s
    s = time.perf_counter(); orc.permute("+", np.zeros(M_PERM, np.int32), inp["idx"], cval=1, nthreads=nth)
    t["permute"] = time.perf_counter() - s
    s = time.perf_counter(); orc.stencil2d(W9, inp["grid"], 0, nthreads=nth); t["stencil"] = time.perf_counter() - s
    return t


def cpu_bytes(scale, h):
    return {"scan": BYTES["scan"] // scale, "fold": BYTES["fold"] // scale,
            "permute": 4 * (N_PERM // scale) + 8 * M_PERM, "stencil": 8 * h * h}


CPU_RUNS = 5  # the CPU baseline is the median of this many runs after one warm-up


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for ln in pathlib.Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_baseline(scale):
    import oracle
    scale = scale or 4
    nth = os.cpu_count() or 1
    inp = cpu_inputs(scale)
    cpu_step(oracle, inp, nth)
    runs = [cpu_step(oracle, inp, nth) for _ in range(CPU_RUNS)]
    sec = {k: statistics.median(r[k] for r in runs) for k in runs[0]}
    b = cpu_bytes(scale, inp["h"])
    return {"value": round(sum(b.values()) / sum(sec.values()) / 1e9, 2), "unit": "GB/s", "cores": nth,
            "cpu": cpu_model(), "kind": "port",
            "sample": f"1/{scale} of each input (scan {N_SCAN // scale}, fold {N_FOLD // scale}, permute "
                      f"{N_PERM // scale} -> 2^16, stencil {inp['h']}^2); median of {CPU_RUNS} after 1 warm-up",
            "per_skeleton_gbs": {k: round(b[k] / sec[k] / 1e9, 2) for k in sec}}


def workload_config(world):
    return {"workload": "scanl1 (+) Int64 2^28; fold (+) Float32 2^28; permute (+) histogram 2^28 Int32 "
                        "Zipf(1.1) -> 2^16 bins; stencil 3x3 Float32 8192^2 clamp",
            "l2": "every input > L2 (129 MB); no flush", "parallelism": f"replicas x{world}"}


def run_reference(args):
    import oracle
    nth = os.cpu_count() or 1
    scale = args.cpu_scale or 1
    inp = cpu_inputs(scale)
    for _ in range(args.warmup):
        cpu_step(oracle, inp, nth)
    runs = [cpu_step(oracle, inp, nth) for _ in range(args.steps)]
    b = cpu_bytes(scale, inp["h"])
    tot = sum(sum(r.values()) for r in runs)
    value = sum(b.values()) * args.steps / tot / 1e9
    line = {
        "impl": "reference",
        "metric": "HBM GB/s per skeleton vs peak (plain single-call kernels at full size)",
        "value": round(value, 2), "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(tot / args.steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64+f32+i32", "data": "synthetic (seeded, host)",
        "config": workload_config(args.gpus) if scale == 1 else
                  dict(workload_config(args.gpus), sample=f"1/{scale} of each input per step"),
        "cpu_baseline": {"value": round(value, 2), "unit": "GB/s", "cores": nth, "cpu": cpu_model(), "kind": "port",
                         "sample": "the full inputs" if scale == 1 else f"1/{scale} of each input per step"},
        "e2e": {"value": round(value, 2), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "per_skeleton_gbs": {k: round(b[k] * args.steps / sum(r[k] for r in runs) / 1e9, 2) for k in b},
    }
    return line


# ----------------------------------------------------------------- distributed
def dist_init():
    """One process per GPU under torchrun: NCCL with a GPU, gloo without one
    (the replica bookkeeping is the same)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return rank, world


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(world, v):
    """The maximum of v over the ranks (the slowest replica sets the time)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return v


def whole_job_gbs(world, step_bytes, ms_per_step):
    """Replicas only: every rank moves step_bytes per step, so the job moves
    world * step_bytes in the slowest rank's time."""
    return world * step_bytes / (ms_per_step * 1e-3) / 1e9


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-scale", type=int, default=None,
                    help="CPU sample = 1/scale of each input (default: 4 for the CPU baseline beside our arm, "
                         "1 -- the full inputs -- for --impl reference)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-launch workload")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="length of the 20k req/s serving stream (0: skip serving)")
    ap.add_argument("--only", choices=["scan", "fold", "permute", "stencil", "foldseg", "batched", "dotp", "scanzip",
                                       "stencil3d", "rowscan"],
                    help="time one skeleton alone (small-case driver for ncu captures)")
    ap.add_argument("--scale", type=int, default=1, help="with --only: 1/scale of the full input")
    args = ap.parse_args()
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank != 0:
            return
        print(json.dumps(run_reference(args)))
        return
    if args.only:
        print(json.dumps(run_only(args)))
        return
    rank, world = dist_init()
    line = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
