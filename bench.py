#!/usr/bin/env python3
"""Benchmark of the point-cloud -> octree build on one GB300.

Workload (default): 10,000,000 points from a 32-component isotropic Gaussian
mixture (sigma 0.5% of the domain, 2% uniform noise), 64-bit Morton codes at
21 bits per axis, 5 onesweep passes over bits 23..62 carrying u32 point
indices and a run fixup over the low 23 bits (the same order as 8 passes),
unique, Karras radix tree + edge count, node offsets, octree make+link.  One step = one full
build of that cloud.  Metric: Mpoints/s of the full build.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gtc|reference]

The default line also carries `forms`: sort-only Mkeys/s of u32 and u64
pairs at 2^24 keys, the learned-bucket form against the plain onesweep at
2^26 keys, and the batched 512-cloud form, all measured in the same run, and
the oracle's CPU build on all host threads and on one (`cpu_baseline`,
`cpu_baseline_1t`).

--impl reference times the CPU restatement of the reference's path (the
oracle; the reference itself is Rust + Vulkan and cannot run here) on the
host cores with all threads.  Under torchrun (N > 1) every rank builds its
own cloud (replicas, weak scaling) and rank 0 prints the line.
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

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "glsl-tree-construction_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mpoints/s full octree build"
UNIT = "Mpoints/s"
N_POINTS = 10_000_000
LEARNED_KEYS = 64 << 20
KEY_BITS = 64
WORKLOAD = "octree_clustered_10M_u64"
SORT_BEGIN_BIT = 23  # the pipeline's 64-bit sort: onesweep passes over bits 23..62, then the run fixup
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["gtc", "reference"], default="gtc")
    ap.add_argument("--n", type=int, default=None,
                    help="points / keys (default: 10M for octree and sort, 64M (2^26) for learned)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="octree workload: skip the sort / learned / batched forms measured after the build")
    ap.add_argument("--workload", choices=["octree", "sort", "sort_sweep", "learned", "batched", "cub_sort"],
                    default="octree",
                    help="octree: the 10M clustered full build (default); sort: onesweep pairs sort only; "
                         "sort_sweep: the sort at n = 2^16..2^28 (powers of 4), u32 and u64; "
                         "learned: learned-bucket vs plain sort; batched: 512 clouds in one build; "
                         "cub_sort: CUB's radix sort beside this project's on the same keys (bench-only)")
    ap.add_argument("--begin-bit", type=int, default=0, help="cub_sort workload: first key bit sorted")
    ap.add_argument("--clouds", type=int, default=512, help="batched workload: number of clouds")
    ap.add_argument("--key-bits", type=int, default=64, help="sort workload: 32 or 64")
    ap.add_argument("--and-words", type=int, default=0, help="sort workload: AND of k uniform words (0 = uniform)")
    ap.add_argument("--sort-variant", type=int, default=None,
                    help="force a compiled onesweep variant (sort and octree workloads; skips the autotuner)")
    return ap.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def init_replicas(world):
    """Under torchrun every rank builds its own cloud on its own GPU (replicas,
    no data exchange): a gloo group serves only the barriers around the timed
    region and the max over ranks.  None for a single process."""
    if world <= 1:
        return None
    import torch.distributed as dist

    dist.init_process_group("gloo")
    return dist


def max_over_ranks(pg, value):
    """The slowest rank's figure (the whole job ends with it); value itself
    for a single process."""
    if pg is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, value):
    """The total over all ranks (units the whole job processes); value itself
    for a single process."""
    if pg is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


def job_rate(units, ms_per_step):
    """Whole-job throughput in millions of units per second: the units all
    ranks process in one step over the slowest rank's step time."""
    return units / (ms_per_step * 1e-3) / 1e6


def replica_rate(pg, units, seconds):
    """Whole-job rate of a figure every rank measures on its own (an end-to-end
    loop): all ranks' units over the slowest rank's seconds, in millions of
    units per second."""
    return job_rate(sum_over_ranks(pg, units), max_over_ranks(pg, seconds) * 1e3)


def measured_hbm_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


# ------------------------------------------------------------- clocks -----
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.5)  # nvidia-smi needs a moment before its first sample
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.path:
            return None
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------ algorithmic bytes --
def algorithmic_bytes(n, u, m, o, K=8):
    """Compulsory bytes of each stage reading its inputs once and writing its
    outputs once (per-stage figures of the reference's stage surface).  The
    sort counts the passes the pipeline runs: 64-bit codes take 5 passes over
    bits 23..62 plus one read of the keys by the run fixup; 32-bit codes take
    4 passes."""
    P = 5 if K == 8 else 4
    return {
        "morton": 16 * n + (K + 4) * n,
        "histogram": K * n,
        "onesweep": P * 2 * (K + 4) * n,
        "run_fixup": (K * n) if K == 8 else 0,
        "unique": (K + 4) * n + (K + 4) * u,
        "radix_tree": K * u + 11 * m,
        "edge_count": 10 * m,
        "prefix_sum": 8 * m,
        "octree_make": (17 + K) * m + 64 * o,
        "octree_link": (23 + K) * m + 8 * u,
    }


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ------------------------------------------------------------ config -------
def octree_config(n):
    """The workload's config object, the same in both arms (this project's
    build and the reference arm), so that the two lines name one workload."""
    name = WORKLOAD if n == N_POINTS else f"octree_clustered_{n}_u64"
    return {"workload": name, "n_points": n, "key_bits": KEY_BITS, "bits_per_axis": 21,
            "payload": "u32 point index",
            "cloud": "32-component Gaussian mixture (sigma 0.5% of the domain) + 2% uniform noise, seed = rank",
            "l2": "no flush: inputs larger than L2 (16 B points per point; a 10M build reads 160 MB of points "
                  "and moves ~3.2 GB)"}


# ------------------------------------------------------------ reference ---
def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import numpy as np

    import oracle
    from gtc import workloads as W

    oracle.build()
    threads = cpu_threads()
    pts = W.config2_points(args.n, seed=0)
    # Size the per-step sample so the whole run stays within ~2.5 minutes.
    t0 = time.perf_counter()
    oracle.build_octree(pts, KEY_BITS, threads=threads)
    t_full = time.perf_counter() - t0
    total_steps = args.steps + max(args.warmup - 1, 0)
    frac = min(1.0, 150.0 / max(total_steps * t_full, 1e-9))
    ns = max(1, int(args.n * frac))
    sample = np.ascontiguousarray(pts[:ns])
    for _ in range(max(args.warmup - 1, 0)):
        oracle.build_octree(sample, KEY_BITS, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.build_octree(sample, KEY_BITS, threads=threads)
    el = time.perf_counter() - t0
    value = ns * args.steps / el / 1e6
    desc = (f"first {ns} of the {args.n}-point clustered cloud per step" if ns < args.n
            else f"the full {args.n}-point clustered cloud per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": octree_config(args.n),
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port", "sample": desc,
                         "cpu": host_cpu()},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "details": {"sample_points": ns,
                    "what": "the oracle (C++ restatement of the reference's shaders, pinned to them; the "
                            "reference's Rust/Vulkan host cannot run here) on all host threads"},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(pts_np, threads, budget_s=10.0, max_reps=8):
    """The oracle's full build timed on the host cores (a bounded sample)."""
    import numpy as np

    import oracle

    oracle.build()
    n_all = pts_np.shape[0]
    # Single-threaded builds of 10M points take seconds each: use a prefix.
    ns = n_all if threads > 1 else min(n_all, 2_000_000)
    sample = np.ascontiguousarray(pts_np[:ns])
    reps = 0
    t0 = time.perf_counter()
    while True:
        oracle.build_octree(sample, KEY_BITS, threads=threads)
        reps += 1
        el = time.perf_counter() - t0
        if el >= budget_s or reps >= max_reps:
            break
    what = "the same" if ns == n_all else f"the first {ns} points of the"
    return {"value": round(ns * reps / el / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{reps} full builds of {what} {n_all}-point cloud with the oracle ({threads} thread"
                      f"{'s' if threads > 1 else ''})", "cpu": host_cpu()}


def host_cpu() -> str:
    """The host CPU as the OS names it, and its online core count."""
    import platform

    name = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware") and ":" in line:
                    name = line.split(":", 1)[1].strip()
                    break
                if key == "cpu part" and not name:  # Arm: implementer / part numbers only
                    name = "Arm part " + line.split(":", 1)[1].strip()
    except OSError:
        pass
    return f"{name or platform.processor() or platform.machine()}, {os.cpu_count()} cores online"


# --------------------------------------------------------- measurements ---
def events_ms(stream, fn, reps, before=None):
    """Mean CUDA-event time of fn() on `stream` over reps calls; before()
    (untimed, e.g. restoring an unsorted input) runs ahead of each call."""
    import torch

    total = 0.0
    for _ in range(reps):
        if before:
            before()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        total += e0.elapsed_time(e1)
    return total / reps


def graph_ms(stream, fn, reps):
    """Mean time per replay of fn() captured once into a CUDA graph: `reps`
    replays between two events on `stream`."""
    import torch

    fn()  # warm-up outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        g.capture_begin()
        fn()
        g.capture_end()
    torch.cuda.synchronize()
    for _ in range(2):
        g.replay()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        g.replay()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def sort_keys(n, kb, and_words=0):
    from gtc import workloads as W

    return W.config3_keys(n, kb, and_words=and_words, seed=1)


def measure_sort(ctx, kb, n, steps, warmup, and_words=0, variant=None):
    """Stable onesweep sort of (key, u32 index) pairs, bits [0, kb).  Returns
    timing, per-pass roofline and a sortedness / stable-permutation check."""
    import numpy as np
    import torch

    import gtc

    keys_np = sort_keys(n, kb, and_words)
    kd = np.int32 if kb == 32 else np.int64
    src_k = torch.from_numpy(keys_np.view(kd)).cuda()
    src_v = torch.arange(n, dtype=torch.int32, device="cuda")
    if variant is not None:
        ctx.set_sort_variant(kb, variant)
    else:  # the autotuner's pick for these keys (cached per key width, bits and ceil(log2 n))
        tune = ctx.autotune_sort(kb, n, 0, kb, keys=src_k, reps=3)
    ws = ctx.workspace(gtc.OP_SORT_PAIRS, n, kb)
    k, v = torch.empty_like(src_k), torch.empty_like(src_v)
    ka, va = torch.empty_like(src_k), torch.empty_like(src_v)
    stream = torch.cuda.current_stream()

    def restore():
        k.copy_(src_k)
        v.copy_(src_v)

    def step():
        ctx.sort_pairs(k, v, 0, kb, ws=ws, keys_alt=ka, vals_alt=va)

    for _ in range(max(warmup, 3)):
        restore()
        step()
    torch.cuda.synchronize()
    ctx.device_status()
    # Stage split: eager sorts with events between the kernels.
    ctx.set_profiling(True)
    ctx.stage_times(reset=True)
    eager_ms = events_ms(stream, step, steps, restore)
    stages = ctx.stage_times(reset=True)
    ctx.set_profiling(False)
    ctx.device_status()
    # Headline: CUDA-graph replays (no host launch cost, dependent launches on),
    # (restore + sort) minus restore alone, each replayed `steps` times.  Pairs
    # smaller than 512 MB would stay in the 129 MB L2 between iterations: both
    # graphs then also write a 256 MB buffer first (an L2 flush), so every
    # sort starts from DRAM.
    pair_bytes = (kb // 8 + 4) * n
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if pair_bytes < (512 << 20) else None

    def cold_restore():
        if flush is not None:
            flush.fill_(1)
        restore()

    ms = graph_ms(stream, lambda: (cold_restore(), step()), steps) - graph_ms(stream, cold_restore, steps)
    restore()
    step()
    torch.cuda.synchronize()
    ctx.device_status()
    kk = k.cpu().numpy().view(keys_np.dtype)
    vv = v.cpu().numpy().view(np.uint32)
    ok = bool(np.all(kk[1:] >= kk[:-1])) and bool(np.array_equal(keys_np[vv], kk))
    db = ctx.get_sort_digit_bits(kb, kb, n)
    passes = (kb + db - 1) // db
    K = kb // 8
    os_ms, os_n = stages["onesweep"]
    avg = os_ms / max(os_n, 1)
    pass_bytes = 2 * (K + 4) * n
    peak, _ = measured_hbm_peak()
    return {"mkeys_s": round(n / (ms * 1e-3) / 1e6, 1), "ms": round(ms, 4), "eager_ms": round(eager_ms, 4),
            "timing": "CUDA-graph replay of (restore + sort) minus replay of restore; stages from eager sorts",
            "l2": ("flushed: a 256 MB write before each timed sort" if flush is not None
                   else "no flush: the pairs are larger than L2"),
            "n": n, "passes": passes,
            "pass_ms": round(avg, 5), "pass_hbm_frac": round(pass_bytes / (avg * 1e-3) / 1e9 / peak, 4),
            "sort_hbm_frac": round((K * n + passes * pass_bytes) / (ms * 1e-3) / 1e9 / peak, 4),
            "hist_ms": round(stages["histogram"][0] / max(stages["histogram"][1], 1), 4),
            "sort_variant": variant if variant is not None else gtc.autotune_lookup(kb, kb, n),
            "digit_bits": ctx.get_sort_digit_bits(kb, kb, n),
            "digit_ms": None if variant is not None else {str(d): (round(t, 4) if t else None)
                                                          for d, t in tune["digit_ms"].items()},
            "sorted_ok": ok}, stages


def measure_learned(ctx, n, steps, warmup, shifted_n=8_000_000):
    """Learned-bucket sort vs the plain onesweep on the learned workload's
    64-bit Morton keys; the model trained on a 1% sample of a prior run's
    sorted keys.  Both outputs are compared; a shifted mixture must fall back
    and stay exact."""
    import torch

    import gtc
    from gtc import workloads as W

    def keys_of(seed, shifted=False, count=n):
        pts = torch.from_numpy(W.config5_points(count, seed=seed, shifted=shifted)).cuda()
        k, _ = ctx.morton(pts, 64, with_idx=False)
        del pts
        return k

    stream = torch.cuda.current_stream()
    prior = keys_of(1)
    ctx.sort_pairs(prior, None, 0, 64)  # the pipeline's own previous sort
    B = gtc.learned_buckets_for(n)
    model = gtc.LearnedModel(ctx, B)
    t0 = time.perf_counter()
    loss = model.train(prior, stride=100)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    del prior
    keys = keys_of(2)
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    ko, vo = torch.empty_like(keys), torch.empty_like(vals)
    ws = ctx.workspace(gtc.OP_LEARNED_SORT, n, 64)
    wk, wv = torch.empty_like(keys), torch.empty_like(vals)
    ka, va = torch.empty_like(keys), torch.empty_like(vals)
    sws = ctx.workspace(gtc.OP_SORT_PAIRS, n, 64)
    # both sorts run the autotuner's pick for these keys
    ctx.autotune_sort(64, n, 0, 64, keys=keys, reps=2)
    ltune = model.autotune(keys, vals, ws=ws, keys_out=ko, vals_out=vo, reps=2)
    flags = []

    def learned_step():
        flags.append(model.sort(keys, vals, ws=ws, keys_out=ko, vals_out=vo)[2])

    def plain_step():
        ctx.sort_pairs(wk, wv, 0, 64, ws=sws, keys_alt=ka, vals_alt=va)

    def restore():
        wk.copy_(keys)
        wv.copy_(vals)

    for _ in range(max(warmup, 3)):
        learned_step()
        restore()
        plain_step()
    torch.cuda.synchronize()
    flags.clear()
    learned_ms = events_ms(stream, learned_step, steps)
    plain_ms = events_ms(stream, plain_step, steps, restore)
    fl = max(int(f.item()) for f in flags)
    identical = bool(torch.equal(ko, wk) and torch.equal(vo, wv))
    ctx.device_status()
    del wk, wv, ka, va, sws
    shifted = keys_of(3, shifted=True, count=min(n, shifted_n))
    sko, svo, sflags = model.sort(shifted)
    sk2, sv2 = shifted.clone(), torch.arange(shifted.numel(), dtype=torch.int32, device="cuda")
    ctx.sort_pairs(sk2, sv2, 0, 64)
    shifted_ok = bool(torch.equal(sko, sk2) and torch.equal(svo, sv2))
    counts = model.histogram(keys).cpu()
    out = {"learned_mkeys_s": round(n / (learned_ms * 1e-3) / 1e6, 1), "learned_ms": round(learned_ms, 4),
           "plain_mkeys_s": round(n / (plain_ms * 1e-3) / 1e6, 1), "plain_ms": round(plain_ms, 4),
           "speedup_vs_plain": round(plain_ms / learned_ms, 3), "identical": identical, "flags": fl, "n": n,
           "buckets": B, "plain_sort_variant": gtc.autotune_lookup(64, 64, n), "learned_variant": ltune["best"],
           "autotune_learned_ms": [round(t, 4) for t in ltune["ms"]], "train_loss": loss,
           "train_s": round(train_s, 3),
           "bucket_max_over_mean": round(float(counts.max()) / (n / B), 3),
           "shifted_n": int(shifted.numel()), "shifted_flags": int(sflags.item()), "shifted_exact": shifted_ok}
    model.close()
    return out


def measure_batched(ctx, S, steps, warmup, seed=0, pts_np=None, offs_np=None):
    """The batched build of S clouds (config-4 sizes and shapes) as one
    CUDA-graph replay per step, plus an eager pass with per-stage events."""
    import numpy as np
    import torch

    import gtc
    from gtc import workloads as W

    if pts_np is None:
        pts_np, offs_np = W.config4_clouds(S, seed=seed)
    n = pts_np.shape[0]
    pts = torch.from_numpy(pts_np).cuda()
    offs = torch.from_numpy(offs_np.view(np.int32)).cuda()
    plan = gtc.BatchPlan(ctx, n, S, nodes_capacity=n + (n >> 1) + S)
    # the autotuner's pick of the segmented onesweep's tile shape for this batch
    tune = plan.autotune(pts, offs, reps=2)
    for _ in range(max(warmup, 3)):
        plan.launch(pts, offs)
    torch.cuda.synchronize()
    ctx.device_status()
    ko, no, cc = plan.host_offsets()
    u, o = int(ko[S]), int(no[S])
    m = int(cc[:, 1].sum())
    stream = torch.cuda.current_stream()
    ctx.set_profiling(True)
    ctx.stage_times(reset=True)
    eager_ms = events_ms(stream, lambda: plan.launch(pts, offs), steps)
    stages = ctx.stage_times(reset=True)
    ctx.set_profiling(False)
    ctx.device_status()
    plan.capture(pts, offs)
    for _ in range(3):
        plan.replay()
    torch.cuda.synchronize()
    graph_ms = events_ms(stream, plan.replay, steps)
    ctx.device_status()
    return dict(plan=plan, pts=pts, offs=offs, pts_np=pts_np, offs_np=offs_np, n=n, u=u, m=m, o=o,
                eager_ms=eager_ms, graph_ms=graph_ms, stages=stages, variant=tune["best"],
                tune_ms=[round(t, 4) for t in tune["ms"]])


# ----------------------------------------------------------------- gtc ----
def run_gtc(args):
    import ctypes

    import numpy as np
    import torch

    import gtc
    from gtc import workloads as W

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    pg = init_replicas(world)

    n = args.n
    pts_np = W.config2_points(n, seed=rank)
    pts = torch.from_numpy(pts_np).to(f"cuda:{local}")
    ctx = gtc.Context(local)
    # Autotune the onesweep shape on this workload's own Morton codes (the
    # pipeline's sort: 63 bits of 64-bit keys); the choice is cached per
    # (key width, bits, ceil(log2 n)) and picked up by the build below.
    # --sort-variant pins the shape instead (e.g. for a profiler run, where
    # the serialised launches would distort the autotuner's timings).
    if args.sort_variant is not None:
        ctx.set_sort_variant(KEY_BITS, args.sort_variant)
        tune = {"best": args.sort_variant, "ms": []}
    else:
        codes, _ = ctx.morton(pts, KEY_BITS, with_idx=False)
        tune = ctx.autotune_sort(KEY_BITS, n, SORT_BEGIN_BIT, 63, keys=codes, reps=3)
        del codes
    plan = gtc.OctreePlan(ctx, n, KEY_BITS, nodes_capacity=n + (n >> 1))
    for _ in range(max(args.warmup, 3)):
        plan.launch(pts)
    torch.cuda.synchronize()
    ctx.device_status()
    u, m, o = plan.counts_host()

    def barrier():
        if pg:
            pg.barrier()

    # --- per-stage breakdown: K eager builds with CUDA events around every stage
    stream = torch.cuda.current_stream()
    ctx.set_profiling(True)
    ctx.stage_times(reset=True)
    eager_ms = events_ms(stream, lambda: plan.launch(pts), args.steps)
    stages = ctx.stage_times(reset=True)
    ctx.set_profiling(False)
    ctx.device_status()

    # --- timed region: K full builds, each one replay of the whole pipeline
    # captured once as a CUDA graph (how a caller runs repeated builds)
    plan.capture(pts)
    for _ in range(3):
        plan.replay()
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        g0.record(stream)
        for _ in range(args.steps):
            plan.replay()
        g1.record(stream)
        torch.cuda.synchronize()
        barrier()
    elapsed_ms = g0.elapsed_time(g1)
    clocks = clk.summary()
    ctx.device_status()
    elapsed_ms = max_over_ranks(pg, elapsed_ms)

    # --- end to end through the host-buffer entry point (pinned host memory)
    L = ctx.L
    hp = ctypes.c_void_p()
    hn = ctypes.c_void_p()
    ctx.check(L.gtc_host_alloc(ctypes.byref(hp), n * 16))
    cap = o + 1024
    ctx.check(L.gtc_host_alloc(ctypes.byref(hn), cap * 64))
    ctypes.memmove(hp, pts_np.ctypes.data, n * 16)
    counts = np.zeros(3, np.uint32)
    cp = counts.ctypes.data_as(ctypes.c_void_p)
    for _ in range(2):
        ctx.check(L.gtc_build_octree_host(ctx.h, hp, n, 0.0, 1024.0, KEY_BITS, hn, cap, cp))
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.check(L.gtc_build_octree_host(ctx.h, hp, n, 0.0, 1024.0, KEY_BITS, hn, cap, cp))
    e2e_sync_s = (time.perf_counter() - t0) / e2e_steps
    assert tuple(int(c) for c in counts) == (u, m, o)
    # Back-to-back builds through the queued entry point: uploads, node
    # read-backs and kernels of consecutive builds overlap.  Every step still
    # moves its own points in and its nodes out; each build in flight has its
    # own node and count buffers.
    NQ = 3
    outs = [hn] + [ctypes.c_void_p() for _ in range(NQ - 1)]
    hc = [ctypes.c_void_p() for _ in range(NQ)]
    for h in outs[1:]:
        ctx.check(L.gtc_host_alloc(ctypes.byref(h), cap * 64))
    for c in hc:
        ctx.check(L.gtc_host_alloc(ctypes.byref(c), 16))
    for i in range(2 * NQ):
        ctx.check(L.gtc_build_octree_host_async(ctx.h, hp, n, 0.0, 1024.0, KEY_BITS, outs[i % NQ], cap, hc[i % NQ]))
    ctx.check(L.gtc_build_octree_host_wait(ctx.h))
    q_steps = max(6, min(args.steps, 30))
    t0 = time.perf_counter()
    for i in range(q_steps):
        ctx.check(L.gtc_build_octree_host_async(ctx.h, hp, n, 0.0, 1024.0, KEY_BITS, outs[i % NQ], cap, hc[i % NQ]))
    ctx.check(L.gtc_build_octree_host_wait(ctx.h))
    e2e_rate = replica_rate(pg, n, (time.perf_counter() - t0) / q_steps)
    e2e_sync_rate = replica_rate(pg, n, e2e_sync_s)
    for c in hc:
        got = np.ctypeslib.as_array((ctypes.c_uint32 * 3).from_address(c.value))
        assert tuple(int(x) for x in got) == (u, m, o)
        L.gtc_host_free(c)
    L.gtc_host_free(hp)
    for h in outs:
        L.gtc_host_free(h)

    if rank != 0:
        return

    # --- roofline of the dominant kernel (onesweep digit-binning pass)
    os_ms, os_launches = stages["onesweep"]
    avg_pass_ms = os_ms / max(os_launches, 1)
    pass_bytes = 2 * (8 + 4) * n
    achieved = pass_bytes / (avg_pass_ms * 1e-3) / 1e9
    peak, peak_kind = measured_hbm_peak()
    traffic = None
    tp = os.path.join(REPO, "profiles", "onesweep_traffic.json")
    if os.path.exists(tp):
        try:
            tj = json.load(open(tp))
            traffic = tj["dram_bytes_per_launch_per_key_u64"] * n
        except Exception:
            traffic = None
    alg = algorithmic_bytes(n, u, m, o, 8)
    alg_total = sum(alg.values())
    ms_per_step = elapsed_ms / args.steps
    value = job_rate(world * n, ms_per_step)  # every rank builds an n-point cloud
    kernels_per_step = 1 + 5 + 1 + 1 + 2 + 1 + 1  # morton+hist, 5 passes, run fixup, unique, tree + long splits, scan, octree
    stage_ms = {k: round(v[0] / args.steps, 4) for k, v in stages.items() if v[1]}

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": octree_config(n),
        "details": {"onesweep_passes": 5, "sort_bits": "23..62, then the run fixup over bits 0..22",
                    "n_unique": u, "n_brt_nodes": m, "n_oct_nodes": o, "parallelism": f"replicas{world}",
                    "l2": "inputs larger than L2 (160 MB of points, ~1 GB working set per build)",
                    "timing": "CUDA-graph replay of the whole build per step",
                    "eager_ms_per_step": round(eager_ms, 4), "stage_ms_per_step": stage_ms,
                    "algorithmic_GB_per_step": round(alg_total / 1e9, 4),
                    "pipeline_hbm_frac": round(alg_total / (ms_per_step * 1e-3) / 1e9 / peak, 4),
                    "sort_variant": (args.sort_variant if args.sort_variant is not None
                                     else gtc.autotune_lookup(KEY_BITS, 63 - SORT_BEGIN_BIT, n)),
                    "autotune_sort_ms": [round(t, 4) for t in tune["ms"]],
                    "autotune_digit_ms": {str(d): (round(t, 4) if t else None)
                                          for d, t in tune.get("digit_ms", {}).items()}},
        "roofline": {"bound": "hbm", "kernel": "onesweep_kernel (one 8-bit digit pass, u64 key + u32 value)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                     "bytes_per_launch": pass_bytes, "avg_launch_ms": round(avg_pass_ms, 5)},
        "e2e": {"value": round(e2e_rate, 2), "unit": UNIT, "h2d_bytes_per_step": n * 16,
                "d2h_bytes_per_step": o * 64 + 12,
                "api": "gtc_build_octree_host_async x steps + gtc_build_octree_host_wait (pinned host buffers, "
                       "consecutive builds overlapped)",
                "sync_value": round(e2e_sync_rate, 2),
                "sync_api": "gtc_build_octree_host, one build at a time"},
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": clocks,
    }
    del plan, pts
    torch.cuda.empty_cache()
    if not args.no_forms:
        line["forms"] = measure_forms(ctx, args)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(pts_np, cpu_threads())
        line["cpu_baseline_1t"] = cpu_baseline(pts_np, 1)
    print(json.dumps(line), flush=True)
    ctx.close()


def measure_forms(ctx, args):
    """The rest of the metric, measured in the same run on the same GPU:
    sort-only Mkeys/s of u32 and u64 pairs at 2^24 keys (uniform), the
    learned-bucket form against the plain onesweep at 2^26 keys, and the
    batched form over 512 clouds."""
    import torch

    steps = max(3, min(args.steps, 20))
    forms = {}
    for kb in (32, 64):
        forms[f"sort_u{kb}_2p24"], _ = measure_sort(ctx, kb, 1 << 24, steps, 3)
        torch.cuda.empty_cache()
    forms["learned_vs_plain_2p26"] = measure_learned(ctx, LEARNED_KEYS, steps, 3)
    torch.cuda.empty_cache()
    b = measure_batched(ctx, 512, steps, 3)
    forms["batched_512_clouds"] = {
        "mpoints_s": round(b["n"] / (b["graph_ms"] * 1e-3) / 1e6, 1), "ms": round(b["graph_ms"], 4),
        "n_points": b["n"], "eager_ms": round(b["eager_ms"], 4), "batched_variant": b["variant"],
        "autotune_batched_ms": b["tune_ms"],
        "stage_ms": {k: round(v[0] / steps, 4) for k, v in b["stages"].items() if v[1]}}
    del b
    torch.cuda.empty_cache()
    return forms


def run_gtc_sort(args):
    """Sort-only workload: stable onesweep sort of (key, u32 index) pairs."""
    import gtc

    kb, n = args.key_bits, args.n
    ctx = gtc.Context(0)
    with ClockSampler(0) as clk:
        r, _ = measure_sort(ctx, kb, n, args.steps, args.warmup, args.and_words, args.sort_variant)
    peak, peak_kind = measured_hbm_peak()
    K = kb // 8
    line = {
        "metric": "Mkeys/s sort", "value": r["mkeys_s"], "unit": "Mkeys/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": f"u{kb}", "data": "synthetic",
        "config": {"workload": f"sort_pairs_u{kb}_n{n}_and{args.and_words}", "n": n, "key_bits": kb,
                   "l2": r["l2"]},
        "details": r,
        "roofline": {"bound": "hbm", "kernel": "onesweep pass",
                     "achieved": round(2 * (K + 4) * n / (r["pass_ms"] * 1e-3) / 1e9, 1), "peak": peak,
                     "unit": "GB/s", "frac": r["pass_hbm_frac"], "traffic": None, "peak_kind": peak_kind,
                     "avg_launch_ms": r["pass_ms"]},
        "gpu_launches": (1 + r["passes"]) * args.steps,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def run_gtc_sort_sweep(args):
    """Sort-only sweep of the sort config: n = 2^16 .. 2^28 in powers of 4,
    u32 and u64 pairs (u32 values = the input index), uniform keys; each size
    runs the autotuner's pick for its keys.  One JSON line; its value is the
    u64 rate at the largest size."""
    import torch

    import gtc

    ctx = gtc.Context(0)
    rows = []
    with ClockSampler(0) as clk:
        for kb in (32, 64):
            for lg in range(16, 29, 2):
                r, _ = measure_sort(ctx, kb, 1 << lg, args.steps, args.warmup, 0, args.sort_variant)
                rows.append({"key_bits": kb, "log2n": lg, "mkeys_s": r["mkeys_s"], "ms": r["ms"],
                             "pass_hbm_frac": r["pass_hbm_frac"], "sort_hbm_frac": r["sort_hbm_frac"],
                             "variant": r["sort_variant"], "digit_bits": r["digit_bits"], "l2": r["l2"],
                             "sorted_ok": r["sorted_ok"]})
                torch.cuda.empty_cache()
    top = rows[-1]
    line = {
        "metric": "Mkeys/s sort", "value": top["mkeys_s"], "unit": "Mkeys/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": top["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": "sort_sweep_2p16_2p28_u32_u64", "n": 1 << 28, "key_bits": 64,
                   "l2": "flushed (a 256 MB write) before each timed sort where the pairs are smaller than 512 MB, "
                         "else inputs larger than L2"},
        "details": {"sweep": rows, "all_sorted_ok": all(r["sorted_ok"] for r in rows)},
        "gpu_launches": None, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def cub_library():
    """Builds (once) and loads bench-only libcubref.so: CUB's
    DeviceRadixSort::SortPairs behind a C ABI, the comparison point of the
    cub_sort workload.  Never part of libgtc.so."""
    import ctypes

    from gtc import _build

    src = os.path.join(_build.PKG_ROOT, "bench", "cub_sort.cu")
    out = os.path.join(_build.BUILD_DIR, "libcubref.so")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        os.makedirs(_build.BUILD_DIR, exist_ok=True)
        cmd = [_build._nvcc(), *_build.ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
               src, "-o", out]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("libcubref build failed:\n" + r.stdout + r.stderr)
    L = ctypes.CDLL(out)
    P = ctypes.c_void_p
    L.cubref_ws_bytes.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]
    L.cubref_sort_pairs.argtypes = [P, P, P, P, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int, P,
                                    ctypes.c_size_t, P, ctypes.POINTER(ctypes.c_int)]
    return L


def run_cub_sort(args):
    """CUB's onesweep (cub::DeviceRadixSort::SortPairs) beside this project's
    sort on the same keys, bit range and GPU: the reference point for the
    onesweep pass's roofline fraction.  --begin-bit picks the bit range
    (23 = the pipeline's 64-bit sort over bits 23..62)."""
    import ctypes

    import numpy as np
    import torch

    import gtc

    kb, n = args.key_bits, args.n
    end = 63 if (kb == 64 and args.begin_bit > 0) else kb
    L = cub_library()
    keys_np = sort_keys(n, kb, args.and_words)
    kd = np.int32 if kb == 32 else np.int64
    src_k = torch.from_numpy(keys_np.view(kd)).cuda()
    src_v = torch.arange(n, dtype=torch.int32, device="cuda")
    k, v = torch.empty_like(src_k), torch.empty_like(src_v)
    ka, va = torch.empty_like(src_k), torch.empty_like(src_v)
    b = ctypes.c_size_t()
    assert L.cubref_ws_bytes(n, kb, ctypes.byref(b)) == 0
    ws = torch.empty(max(b.value, 256), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sel = ctypes.c_int()

    def restore():
        k.copy_(src_k)
        v.copy_(src_v)

    def cub_step():
        assert L.cubref_sort_pairs(k.data_ptr(), v.data_ptr(), ka.data_ptr(), va.data_ptr(), n, kb, args.begin_bit,
                                   end, ws.data_ptr(), ws.numel(), stream.cuda_stream, ctypes.byref(sel)) == 0

    for _ in range(max(args.warmup, 3)):
        restore()
        cub_step()
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        cub_ms = events_ms(stream, cub_step, args.steps, restore)
    got_k = (ka if sel.value else k).clone()
    got_v = (va if sel.value else v).clone()
    ctx = gtc.Context(0)
    gws = ctx.workspace(gtc.OP_SORT_PAIRS, n, kb)

    def gtc_step():
        ctx.sort_pairs(k, v, args.begin_bit, end, ws=gws, keys_alt=ka, vals_alt=va)

    for _ in range(max(args.warmup, 3)):
        restore()
        gtc_step()
    torch.cuda.synchronize()
    ctx.set_profiling(True)
    ctx.stage_times(reset=True)
    gtc_ms = events_ms(stream, gtc_step, args.steps, restore)
    stages = ctx.stage_times(reset=True)
    ctx.set_profiling(False)
    identical = bool(torch.equal(k, got_k) and torch.equal(v, got_v))
    passes = (end - args.begin_bit + 7) // 8
    K = kb // 8
    peak, peak_kind = measured_hbm_peak()
    pass_bytes = 2 * (K + 4) * n
    os_ms, os_n = stages["onesweep"]
    line = {
        "metric": "Mkeys/s sort (CUB comparison)", "value": round(n / (cub_ms * 1e-3) / 1e6, 1), "unit": "Mkeys/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(cub_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": f"u{kb}", "data": "synthetic",
        "config": {"workload": f"cub_sort_pairs_u{kb}_n{n}_bits{args.begin_bit}_{end}", "n": n, "key_bits": kb,
                   "l2": "inputs as given by --n (larger than L2 from 2^24 pairs)"},
        "details": {"impl": "cub::DeviceRadixSort::SortPairs (bench-only comparison)", "passes": passes,
                    "cub_ms": round(cub_ms, 4), "cub_ms_per_pass": round(cub_ms / passes, 5),
                    "gtc_ms": round(gtc_ms, 4), "gtc_pass_ms": round(os_ms / max(os_n, 1), 5),
                    "gtc_hist_ms": round(stages["histogram"][0] / max(stages["histogram"][1], 1), 5),
                    "gtc_over_cub": round(cub_ms / gtc_ms, 3), "identical_output": identical,
                    "cub_pass_hbm_frac_upper": round(pass_bytes / (cub_ms / passes * 1e-3) / 1e9 / peak, 4),
                    "gtc_pass_hbm_frac": round(pass_bytes / (os_ms / max(os_n, 1) * 1e-3) / 1e9 / peak, 4)},
        "gpu_launches": None,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def run_gtc_learned(args):
    """Learned-bucket sort vs plain onesweep on clustered 64-bit Morton keys
    (64-component Gaussian mixture, sigma 0.3-3% of the domain, Dirichlet(1)
    weights, 5% noise).  The model is trained on a 1% sample of a prior run's
    sorted keys (same mixture, another seed); both sorts must give identical
    output; a shifted mixture must take the onesweep fallback."""
    import gtc

    n = args.n
    ctx = gtc.Context(0)
    with ClockSampler(0) as clk:
        r = measure_learned(ctx, n, args.steps, args.warmup)
    peak, peak_kind = measured_hbm_peak()
    # compulsory bytes of the learned path per key: model read 8, bucket
    # scatter read 12 + write 12, in-bucket sort read 12 + write 12
    lbytes = 56 * n
    line = {
        "metric": "Mkeys/s learned-bucket sort", "value": r["learned_mkeys_s"], "unit": "Mkeys/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["learned_ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": f"learned_sort_u64_n{n}", "n": n, "key_bits": 64,
                   "l2": "no flush: inputs larger than L2 (12 B per key)"},
        "details": r,
        "roofline": {"bound": "hbm", "kernel": "learned path (model + bucket scatter + in-bucket sort)",
                     "achieved": round(lbytes / (r["learned_ms"] * 1e-3) / 1e9, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(lbytes / (r["learned_ms"] * 1e-3) / 1e9 / peak, 4), "traffic": None,
                     "peak_kind": peak_kind},
        "gpu_launches": None,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def run_gtc_batched(args):
    """Batched workload: 512 clouds with sizes log-uniform in [1K, 1M],
    alternately uniform and 8-cluster Gaussian (sigma 1% of the domain),
    32-bit codes; one step = one batched build of all clouds, timed eagerly
    (per-stage events) and as one CUDA-graph replay.  Metric: Mpoints/s."""
    import numpy as np
    import torch

    import gtc
    from gtc import workloads as W

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    pg = init_replicas(world)
    S = args.clouds
    pts_np, offs_np = W.config4_clouds(S, seed=rank)
    ctx = gtc.Context(local)
    b = measure_batched(ctx, S, 3, args.warmup, pts_np=pts_np, offs_np=offs_np)
    plan, pts, offs, n, u, m, o = b["plan"], b["pts"], b["offs"], b["n"], b["u"], b["m"], b["o"]
    stages = b["stages"]
    stream = torch.cuda.current_stream()
    # Timed region: one CUDA-graph replay of the whole batch per step.
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        if pg:
            pg.barrier()
        torch.cuda.synchronize()
        g0.record(stream)
        for _ in range(args.steps):
            plan.replay()
        g1.record(stream)
        torch.cuda.synchronize()
        if pg:
            pg.barrier()
    elapsed_ms = g0.elapsed_time(g1)
    clocks = clk.summary()
    ctx.device_status()
    elapsed_ms = max_over_ranks(pg, elapsed_ms)
    n_job = sum_over_ranks(pg, n)  # the ranks' clouds differ (seed = rank)

    # End to end: pinned host points in, every cloud's octree nodes out.
    hp = torch.empty_like(pts, device="cpu").pin_memory()
    hp.copy_(torch.from_numpy(pts_np))
    hn = torch.empty((o, 16), dtype=torch.int32).pin_memory()
    dp = torch.empty_like(pts)
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        dp.copy_(hp, non_blocking=True)
        plan.launch(dp, offs)
        hn.copy_(plan.nodes[:o], non_blocking=True)
        torch.cuda.synchronize()
    e2e_rate = replica_rate(pg, n, (time.perf_counter() - t0) / e2e_steps)
    ctx.device_status()
    if rank != 0:
        return
    os_ms, os_launches = stages["onesweep"]
    avg_pass_ms = os_ms / max(os_launches, 1)
    pass_bytes = 2 * (4 + 4) * n
    achieved = pass_bytes / (avg_pass_ms * 1e-3) / 1e9
    peak, peak_kind = measured_hbm_peak()
    alg_total = sum(algorithmic_bytes(n, u, m, o, 4).values())
    ms_per_step = elapsed_ms / args.steps
    stage_ms = {k: round(v[0] / 3, 4) for k, v in stages.items() if v[1]}
    sizes = np.diff(offs_np.astype(np.int64))
    line = {
        "metric": "Mpoints/s batched octree build", "value": round(job_rate(n_job, ms_per_step), 2),
        "unit": "Mpoints/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_per_step, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic",
        "config": {"workload": f"batched_{S}_clouds_u32", "n_clouds": S, "n_points": n,
                   "l2": "no flush: inputs larger than L2 (16 B points per point)"},
        "details": {"cloud_min": int(sizes.min()), "cloud_max": int(sizes.max()), "n_unique": u, "n_oct_nodes": o,
                    "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (points alone exceed 1 GB)",
                    "timing": "CUDA-graph replay of the whole batch per step",
                    "eager_ms_per_step": round(b["eager_ms"], 4), "stage_ms_per_step": stage_ms,
                    "batched_variant": b["variant"], "autotune_batched_ms": b["tune_ms"],
                    "algorithmic_GB_per_step": round(alg_total / 1e9, 4),
                    "pipeline_hbm_frac": round(alg_total / (ms_per_step * 1e-3) / 1e9 / peak, 4)},
        "roofline": {"bound": "hbm", "kernel": "bt_onesweep_kernel (one segmented 8-bit pass, u32 key + u32 value)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": None, "peak_kind": peak_kind, "bytes_per_launch": pass_bytes,
                     "avg_launch_ms": round(avg_pass_ms, 5)},
        "e2e": {"value": round(e2e_rate, 2), "unit": "Mpoints/s", "h2d_bytes_per_step": n * 16,
                "d2h_bytes_per_step": o * 64, "api": "gtc_build_octree_batched between pinned host copies"},
        "gpu_launches": 13 * args.steps,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    ctx.close()


def main():
    args = parse_args()
    if args.n is None:
        args.n = LEARNED_KEYS if args.workload == "learned" else N_POINTS
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "cub_sort":
        run_cub_sort(args)
    elif args.workload == "sort_sweep":
        run_gtc_sort_sweep(args)
    elif args.workload == "sort":
        run_gtc_sort(args)
    elif args.workload == "learned":
        run_gtc_learned(args)
    elif args.workload == "batched":
        run_gtc_batched(args)
    else:
        run_gtc(args)


if __name__ == "__main__":
    main()
