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
# DRAM bytes per launch from one ncu capture of each kernel (dram__bytes_read.sum
# + dram__bytes_write.sum), scaled to the full launch; see profiles/.
NCU_TRAFFIC = {"scan": None}


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
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
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

    # ---- end to end through the public API with host buffers
    e2e = run_e2e(torch, acc, inp, zeros, args, dev)

    peak, peak_kind = peaks()
    step_bytes = sum(BYTES.values())
    ms_per_step = total_ms / args.steps
    value = world * step_bytes / (ms_per_step * 1e-3) / 1e9
    scan_ms = statistics.mean(per["scan"])
    achieved = BYTES["scan"] / (scan_ms * 1e-3) / 1e9
    per_sk = {}
    for nm in names:
        ms = statistics.mean(per[nm])
        gbs = BYTES[nm] / (ms * 1e-3) / 1e9
        per_sk[nm] = {"ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / peak, 3)}
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
        "config": {"workload": "scanl1 (+) Int64 2^28; fold (+) Float32 2^28; permute (+) histogram 2^28 Int32 "
                               "Zipf(1.1) -> 2^16 bins; stencil 3x3 Float32 8192^2 clamp",
                   "l2": "every input > L2 (129 MB); no flush", "parallelism": f"replicas x{world}"},
        "per_skeleton": per_sk,
        "roofline": {"bound": "hbm", "kernel": "scan_lookback_kernel (scanl1 + Int64)", "achieved": round(achieved, 1),
                     "peak": peak, "peak_kind": f"{peak_kind} hbm_gbs (copy)", "unit": "GB/s",
                     "frac": round(achieved / peak, 3),
                     "traffic": NCU_TRAFFIC["scan"]},
        "e2e": e2e,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(args.cpu_scale)
    return line


def run_e2e(torch, acc, inp, zeros, args, dev):
    """Same step through the public API with pinned host inputs: H2D copy of
    every input, the four skeletons, D2H of every result, per step."""
    host = {k: v.cpu().pin_memory() for k, v in inp.items()}
    stream = torch.cuda.current_stream()
    h2d = sum(v.numel() * v.element_size() for v in host.values())
    res_host = {
        "scan": torch.empty(N_SCAN, dtype=torch.int64).pin_memory(),
        "fold": torch.empty((), dtype=torch.float32).pin_memory(),
        "permute": torch.empty(M_PERM, dtype=torch.int32).pin_memory(),
        "stencil": torch.empty((H_ST, W_ST), dtype=torch.float32).pin_memory(),
    }
    d2h = sum(v.numel() * v.element_size() for v in res_host.values())
    dev_in = {k: torch.empty_like(v, device=dev) for k, v in host.items()}

    def step():
        for k in host:
            dev_in[k].copy_(host[k], non_blocking=True)
        outs = {"scan": acc.scanl1("+", dev_in["scan"]), "fold": acc.fold("+", 0.0, dev_in["fold"]),
                "permute": acc.permute("+", zeros, dev_in["idx"], 1),
                "stencil": acc.stencil(W9, dev_in["grid"], "clamp")}
        for k, v in outs.items():
            res_host[k].copy_(v, non_blocking=True)

    for _ in range(max(1, args.warmup // 2)):
        step()
    torch.cuda.synchronize()
    steps = max(2, args.steps // 2)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(steps):
        step()
    t1.record(stream)
    torch.cuda.synchronize()
    acc.sync()
    ms = t0.elapsed_time(t1) / steps
    del dev_in
    return {"value": round(sum(BYTES.values()) / (ms * 1e-3) / 1e9, 1), "unit": "GB/s", "ms_per_step": round(ms, 3),
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}


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
    idx = perm[np.minimum(np.searchsorted(cdf, rng.random(n_perm)), M_PERM - 1)]
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


def cpu_baseline(scale):
    import oracle
    nth = os.cpu_count() or 1
    inp = cpu_inputs(scale)
    cpu_step(oracle, inp, nth)
    runs = [cpu_step(oracle, inp, nth) for _ in range(3)]
    sec = {k: statistics.median(r[k] for r in runs) for k in runs[0]}
    b = cpu_bytes(scale, inp["h"])
    return {"value": round(sum(b.values()) / sum(sec.values()) / 1e9, 2), "unit": "GB/s", "cores": nth,
            "kind": "port",
            "sample": f"1/{scale} of each input (scan {N_SCAN // scale}, fold {N_FOLD // scale}, permute "
                      f"{N_PERM // scale} -> 2^16, stencil {inp['h']}^2); median of 3 after 1 warm-up",
            "per_skeleton_gbs": {k: round(b[k] / sec[k] / 1e9, 2) for k in sec}}


def run_reference(args):
    import oracle
    nth = os.cpu_count() or 1
    scale = args.cpu_scale
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
        "config": {"workload": "scanl1 (+) Int64 2^28; fold (+) Float32 2^28; permute (+) histogram 2^28 Int32 "
                               "Zipf(1.1) -> 2^16 bins; stencil 3x3 Float32 8192^2 clamp",
                   "sample": f"1/{scale} of each input per step"},
        "cpu_baseline": {"value": round(value, 2), "unit": "GB/s", "cores": nth, "kind": "port",
                         "sample": f"1/{scale} of each input per step"},
        "e2e": {"value": round(value, 2), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "per_skeleton_gbs": {k: round(b[k] * args.steps / sum(r[k] for r in runs) / 1e9, 2) for k in b},
    }
    return line


# ----------------------------------------------------------------- distributed
def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    return rank, world


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(world, v):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([v], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return v


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-scale", type=int, default=4, help="CPU sample = 1/scale of each input")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank != 0:
            return
        print(json.dumps(run_reference(args)))
        return
    rank, world = dist_init()
    line = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
