#!/usr/bin/env python
"""Benchmark of the GB300 onesweep LSD radix sort (libgbsort.so, C ABI).

    python bench.py [--gpus N] [--steps K] [--warmup W]
                    [--config c2b|c1|c2a|c3a|c3b|c4|c5] [--impl gbsort|reference]
                    [--n N] [--segments S] [--rate R] [--e2e-steps S]
                    [--cpu-seconds T] [--no-cpu-baseline] [--no-cub] [--headline-only]

One step = one sort (histogram upsweep + one onesweep pass per key byte) of a
fresh batch of synthetic keys already resident in HBM.  Before each step the
next batch is generated on the device (splitmix64 stream, new seed) and a
512 MiB buffer is written to flush L2; CUDA events on the sort's stream (a
stream of its own) time the sort alone, and `value` = keys sorted / summed
event time.  The K timed steps are bracketed by a barrier +
torch.cuda.synchronize() on both sides.

Default workload (the headline): 2^28 uint32 keys, uniform full range,
ascending, keys only, 8-bit digits / 4 passes.  c1, c2a, c3a, c3b are the
reference benchmark's other plain configurations; c4 is the batched sort of
4096 uneven segments (step = one replay of the batched run, compared with
looping the plain sort over the same segments); c5 is the sort server under
Poisson arrivals from host memory (capacity, then p50/p99 latency at a
fraction of it).  --n shrinks a plain configuration for profiling; --rate
sets c5's arrival rate.

Extra keys on the JSON line:
  roofline      the dominant kernel (the onesweep pass): algorithmic bytes per
                launch (n * 2 * (key + value bytes)) / its mean CUDA-event
                duration, against MEASURED_PEAKS.json's HBM copy bandwidth;
                `traffic` = ncu dram bytes per launch from profiles/ when a
                capture of this workload is committed there
  sort_roofline the whole sort: (K + P*2*(K+V)) bytes per key / sort time
  step_ms       mean, std, p50, p99, min, max of the per-step CUDA-event times
  e2e           same metric through gbsort_sort_host with pinned HOST buffers,
                H2D + sort + D2H inside the timed region; `checked`: the
                returned keys are in order and a permutation of the input
  cpu_baseline  the CPU oracle (std::stable_sort of twiddled keys, 1 thread)
                on a bounded sample of the same workload (rank 0, N=1 only)
  clocks        nvidia-smi samples taken during the timed region
The default run (c2b, one GPU) adds the rest of the benchmark metric after
the headline, each measured the way its own --config run measures it (fewer
steps, no CPU baseline): `plain_configs` (c1, c2a, c3a, c3b: value, roofline,
CUB on the same GPU, e2e), `batched` (c4: value, speedup_vs_loop, roofline,
e2e) and `serving` (c5: capacity, p50/p99 latency at 70 % load,
identical_alone_and_in_mix).  --headline-only skips them.
--impl reference times the reference path's CPU implementation (the oracle
port: parallel stable sort on every host core) on samples of the workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "cuda-fast-sort_gb300")
sys.path.insert(0, PKG)

CONFIGS = {
    "c2b": dict(key="u32", n=1 << 28, dist=0, vb=0, desc=False,
                workload="u32 keys-only, n=2^28, uniform full-range (splitmix64), ascending, 8-bit radix x 4 passes"),
    "c1": dict(key="u32", n=1 << 20, dist=0, vb=0, desc=False,
               workload="u32 keys-only, n=2^20, uniform full-range (splitmix64), ascending, 8-bit radix x 4 passes"),
    "c2a": dict(key="f32", n=1 << 28, dist=1, vb=4, desc=False,
                workload="f32 keys N(0,1) with 1% -0.0 / 0.1% +-inf / 0.01% NaN + u32 index values, n=2^28, "
                         "ascending"),
    "c3a": dict(key="u64", n=1 << 27, dist=2, vb=8, desc=True,
                workload="u64 keys (upper 32 bits from 256 values) + u64 index values, n=2^27, descending"),
    "c3b": dict(key="u128", n=1 << 26, dist=0, vb=0, desc=True,
                workload="u128 keys (two uniform 64-bit halves), keys-only, n=2^26, descending "
                         "(most significant digit first: two splits + local sorts of 65536 groups)"),
    "c4": dict(key="u32", n=0, dist=0, vb=4, desc=False, segments=4096, seg_log2=(8, 20),
               workload="batched: 4096 independent u32-key/u32-value sorts, segment lengths log-uniform in "
                        "[2^8, 2^20] (seeded), keys uniform 32-bit, ascending, one batched run per step"),
    "c5": dict(key="mixed", n=0, dist=0, vb=4, desc=False, serving=True, size_log2=(10, 24), pool=64 << 30,
               streams=6, load=0.7,
               workload="serving: Poisson arrivals, request sizes log-uniform in [2^10, 2^24], key type u32 / u64 / "
                        "f32 with equal probability, 50% carry u32 values, ascending, host pinned buffers, "
                        "64 GiB device pool"),
}
KEY_BYTES = {"u32": 4, "f32": 4, "u64": 8, "u128": 16}
# The reference's own published throughput for the same workload (rsort on an
# RTX 3080 Ti, data/logs/benchmark_data.py of the reference, ms -> Gkeys/s).
PUBLISHED = {
    "c2b": (22.4, "rsort, u32 keys 2^28, RTX 3080 Ti (benchmark_data.py:42: 11.972 ms)"),
    "c1": (14.4, "rsort, u32 keys 2^20, RTX 3080 Ti (benchmark_data.py:34: 0.073 ms)"),
    "c3a": (3.03, "rsort, u64 keys + u64 values 2^27, RTX 3080 Ti (benchmark_data.py:196: 44.281 ms)"),
    "c3b": (1.53, "rsort, u128 keys 2^26, RTX 3080 Ti (benchmark_data.py:118: 43.993 ms)"),
}
PLAIN_METRIC = "sort throughput (Gkeys/s) and HBM roofline fraction"
BATCHED_METRIC = "batched segmented sort throughput (Gkeys/s)"
SERVING_METRIC = "serving throughput (Gkeys/s) under continuous batching, p50/p99 latency at load"


def metric_of(cfg) -> str:
    if cfg.get("serving"):
        return SERVING_METRIC
    return BATCHED_METRIC if "segments" in cfg else PLAIN_METRIC
FALLBACK_HBM_GBS = 6800.0
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def step_stats(ms: list) -> dict:
    """Mean, standard deviation and percentiles of per-step device times (ms)."""
    v = sorted(ms)
    pick = lambda q: v[min(len(v) - 1, int(round(q * (len(v) - 1))))]  # noqa: E731
    return {"mean": round(statistics.mean(v), 4), "std": round(statistics.pstdev(v), 4),
            "p50": round(pick(0.5), 4), "p99": round(pick(0.99), 4), "min": round(v[0], 4),
            "max": round(v[-1], 4), "n": len(v)}


def committed_traffic(config: str, n: int):
    """DRAM bytes (read + write) per pass launch from the committed ncu
    capture of this configuration's pass kernel, scaled to n keys when the
    capture ran a smaller case (traffic grows with the tiles processed)."""
    path = os.path.join(REPO, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            e = json.load(f).get(config)
        if not e:
            return None, None
        scaled = e["dram_bytes_per_launch"] * n / e["captured_n"]
        return int(scaled), f"ncu capture at n={e['captured_n']} scaled to n={n} ({e['summary']})"
    except Exception:
        return None, None


class TimedRange:
    """An NVTX push/pop range named "timed" around a timed region, so that a
    launch list can be restricted to it (ncu --nvtx --nvtx-include "timed]").
    Host-side only; a missing NVTX library leaves it a no-op."""

    def __enter__(self):
        try:
            import torch

            torch.cuda.nvtx.range_push("timed")
            self.on = True
        except Exception:
            self.on = False
        return self

    def __exit__(self, *exc):
        if self.on:
            try:
                import torch

                torch.cuda.nvtx.range_pop()
            except Exception:
                pass
        return False


class ClockSampler:
    """nvidia-smi -lms 200 in the background while the timed region runs."""

    def __init__(self, gpu_index: int):
        self.rows = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={CLOCK_FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(gpu_index)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.rows.append([x.strip() for x in ln.split(",")])

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm = []
        mx = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for i, nm in enumerate(names):
                    if r[5 + i].lower().startswith("active"):
                        reasons.add(nm)
            except Exception:
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if os.environ.get("GBSORT_BENCH_BACKEND") != "gloo" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_sample_bits(cfg, n_sample: int, seed: int):
    from gbsort import gen

    return gen.generate(cfg["dist"], KEY_BYTES[cfg["key"]], n_sample, seed)


def run_cpu_oracle(cfg, n_sample: int, threads: int, reps_min: int, budget_s: float):
    """Times the oracle (test infrastructure, the CPU checker) on a sample."""
    import numpy as np

    sys.path.insert(0, os.path.join(REPO, "tests"))
    import _oracle

    oracle = _oracle.load()
    raw = cpu_sample_bits(cfg, n_sample, seed=99)
    vals = np.arange(n_sample, dtype=np.uint32 if cfg["vb"] == 4 else np.uint64) if cfg["vb"] else None
    times = []
    t_start = time.time()
    while len(times) < reps_min or (time.time() - t_start < budget_s and len(times) < 50):
        t0 = time.perf_counter()
        oracle.sort(cfg["key"], raw, cfg["desc"], vals, threads=threads)
        times.append(time.perf_counter() - t0)
    return n_sample / statistics.mean(times) / 1e9, times


def bench_reference(args, cfg, world, rank):
    """The reference path's CPU implementation (oracle port), all host cores."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    import numpy as np

    sys.path.insert(0, os.path.join(REPO, "tests"))
    import _oracle

    oracle = _oracle.load()
    if "segments" in cfg or cfg.get("serving"):
        return bench_reference_items(args, cfg, world, oracle, cores)
    # size the per-step sample so the whole run stays within ~2 minutes
    n_cfg = cfg["n"]
    probe_n = min(n_cfg, 1 << 22)
    probe = cpu_sample_bits(cfg, probe_n, seed=6)
    t0 = time.perf_counter()
    oracle.sort(cfg["key"], probe, cfg["desc"], None, threads=cores)
    per_key = (time.perf_counter() - t0) / probe_n * (2.0 if cfg["vb"] else 1.0)
    budget = 120.0 / max(1, args.steps + args.warmup)
    n_sample = int(min(n_cfg, 1 << 26, max(1 << 20, budget / max(per_key, 1e-12))))
    raw = cpu_sample_bits(cfg, n_sample, seed=7)
    vals = np.arange(n_sample, dtype=np.uint32 if cfg["vb"] == 4 else np.uint64) if cfg["vb"] else None
    for _ in range(args.warmup):
        oracle.sort(cfg["key"], raw, cfg["desc"], vals, threads=cores)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.sort(cfg["key"], raw, cfg["desc"], vals, threads=cores)
        times.append(time.perf_counter() - t0)
    value = n_sample / statistics.mean(times) / 1e9
    sample = f"{n_sample} keys of the same distribution per step (libstdc++ parallel stable_sort of twiddled keys)"
    line = {
        "impl": "reference", "metric": metric_of(cfg), "value": round(value, 4), "unit": "Gkeys/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * statistics.mean(times), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": cfg["key"], "data": "synthetic",
        "config": {"workload": cfg["workload"], "sample_keys": n_sample, "flush": "inputs larger than L2"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Gkeys/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Gkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_reference_items(args, cfg, world, oracle, cores):
    """Reference arm of the batched and serving configurations: the oracle
    sorts a bounded sample of the workload's independent items (segments or
    requests, drawn from the same distribution) one after another, each with
    every host core."""
    import numpy as np

    from gbsort import gen

    rng = np.random.default_rng(4040)
    items = []
    if "segments" in cfg:
        sizes = gen.log_uniform_sizes(cfg["segments"], cfg["seg_log2"][0], cfg["seg_log2"][1], seed=2026)
        items = [(cfg["key"], int(m), cfg["vb"]) for m in sizes]
    else:
        lo, hi = cfg["size_log2"]
        for _ in range(4096):
            kt = ("u32", "u64", "f32")[int(rng.integers(3))]
            items.append((kt, int(np.floor(2.0 ** rng.uniform(lo, hi))), 4 if rng.random() < 0.5 else 0))
    rng.shuffle(items)
    budget = 100.0 / max(1, args.steps + args.warmup)  # seconds per step
    times, keys_done = [], []
    pos = 0
    for step in range(args.warmup + args.steps):
        t_step, k_step = 0.0, 0
        while t_step < budget and k_step < (1 << 27):
            kt, m, vb = items[pos % len(items)]
            pos += 1
            raw = gen.generate(1 if kt == "f32" else 0, KEY_BYTES[kt], m, 100 + pos)
            vals = np.arange(m, dtype=np.uint32) if vb else None
            t0 = time.perf_counter()
            oracle.sort(kt, raw, cfg["desc"], vals, threads=cores)
            t_step += time.perf_counter() - t0
            k_step += m
        if step >= args.warmup:
            times.append(t_step)
            keys_done.append(k_step)
    value = sum(keys_done) / sum(times) / 1e9
    what = "segments" if "segments" in cfg else "requests"
    sample = (f"{sum(keys_done) // max(1, len(keys_done))} keys per step in whole {what} of the workload's "
              f"distribution, sorted one after another (libstdc++ parallel stable_sort of twiddled keys)")
    line = {
        "impl": "reference", "metric": metric_of(cfg), "value": round(value, 4), "unit": "Gkeys/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * statistics.mean(times), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": cfg["key"], "data": "synthetic",
        "config": {"workload": cfg["workload"], "flush": "inputs larger than L2"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Gkeys/s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Gkeys/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_gbsort(args, cfg, world, rank, local):
    import torch

    import gbsort

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # a stream of its own (not the legacy default stream): input generation,
    # flush, sorts and events are all ordered on it
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    kt, n, vb, desc = cfg["key"], cfg["n"], cfg["vb"], cfg["desc"]
    kbytes = KEY_BYTES[kt]
    passes = kbytes
    # bench batches: two key buffers (+ values) used alternately; regenerated each step
    keys = [torch.empty(n * kbytes, dtype=torch.uint8, device=dev) for _ in range(2)]
    vals = [torch.empty(n * vb, dtype=torch.uint8, device=dev) for _ in range(2)] if vb else [None, None]
    tb = gbsort.temp_bytes(kt, n, vb)
    ws = torch.empty(tb, dtype=torch.uint8, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    seed_base = 1000 * (rank + 1)

    def prepare(slot, seed):
        gbsort.generate(cfg["dist"], kbytes, keys[slot], n, seed, stream)
        if vb:
            gbsort.generate(3, vb, vals[slot], n, 0, stream)  # values = original index
        flush.fill_(seed & 0xFF)  # evict the fresh batch from L2

    def run(slot):
        gbsort.sort(keys[slot], n, kt, ws, tb, values=vals[slot], value_bytes=vb, descending=desc, stream=stream)

    for w in range(args.warmup):
        prepare(w & 1, seed_base + w)
        run(w & 1)
    torch.cuda.synchronize()
    st = gbsort.workspace_status(kt, n, ws, vb, stream)
    if st != gbsort.OK:
        raise RuntimeError(f"warm-up sort reported {gbsort.status_string(st)}")

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local) if rank == 0 else None
    barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    for i in range(args.steps):
        slot = i & 1
        prepare(slot, seed_base + args.warmup + i)
        ev[i][0].record(stream)
        run(slot)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - wall0
    clk = clocks.stop() if clocks else None
    st = gbsort.workspace_status(kt, n, ws, vb, stream)
    if st != gbsort.OK:
        raise RuntimeError(f"timed sort reported {gbsort.status_string(st)}")
    sort_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(world, sum(sort_ms))
    value = world * args.steps * n / (total_ms / 1e3) / 1e9

    # sanity check of the last timed batch on the device (ascending u32 only)
    ok = None
    if kt == "u32" and not desc and not vb:
        k = keys[(args.steps - 1) & 1].view(torch.int32).to(torch.int64) & 0xFFFFFFFF
        ok = bool((k[1:] >= k[:-1]).all().item())
        del k

    # per-kernel event times (dominant kernel: the pass) on fresh batches
    hbm, peak_kind = peaks()
    per_kernel = []
    for r in range(3):
        prepare(r & 1, 77 + r)
        per_kernel.append(gbsort.sort_timed(keys[r & 1], n, kt, ws, tb, values=vals[r & 1], value_bytes=vb,
                                            descending=desc, stream=stream))
    traffic, traffic_src = committed_traffic(args.config, n)
    sort_bytes = n * (kbytes + passes * 2 * (kbytes + vb))
    mean_sort_ms = total_ms / args.steps
    fused = all(len(p) == 1 for p in per_kernel)  # the whole short sort in one launch
    pinfo = gbsort.plan(kt, n, vb)
    msd_keys = pinfo.msd_region_keys if fused else 0
    stages = None
    if not fused and pinfo.msd_stages:
        # keys only, most significant digit first: the top digit's histogram
        # (K bytes a key), top split (2K), pair count (K), scan, second split
        # (2K), local sorts (2K); the other digits' histogram and the digit
        # passes exit at once
        names = ["msd_top_kernel (top split)", "msd_count_kernel (pair count)", "msd_scan_kernel (group offsets)",
                 "msd_second_kernel (second split)", "msd_local_kernel (local sorts)"]
        nbytes = [2 * kbytes * n, kbytes * n, 65536 * 8, 2 * kbytes * n, 2 * kbytes * n]
        means = [statistics.mean(p[1 + i] for p in per_kernel) for i in range(5)]
        dom = max(range(5), key=lambda i: means[i])
        ups_ms = statistics.mean(p[0] for p in per_kernel)
        launch_ms, launch_bytes, kernel = means[dom], nbytes[dom], names[dom]
        sort_bytes = n * 8 * kbytes
        stages = {"upsweep (top digit)": round(ups_ms, 4)}
        for i in range(5):
            stages[names[i]] = {"ms": round(means[i], 4),
                                "frac": round(nbytes[i] / (means[i] / 1e3) / 1e9 / hbm, 4) if i != 2 else None}
        rest = [statistics.mean(p[i] for p in per_kernel) for i in range(6, len(per_kernel[0]))]
        stages["other digits' histogram + digit passes + fix-up (exit at once)"] = round(sum(rest), 4)
    if stages is not None:
        pass
    elif fused and msd_keys:
        # most significant digit first: every key read, written to its
        # top-digit region, read back by its bucket's CTA, written home
        launch_ms = statistics.mean(p[0] for p in per_kernel)
        sort_bytes = n * 4 * kbytes
        launch_bytes, kernel, ups_ms = sort_bytes, "fused_short_kernel (MSD partition, bucket sorts)", None
    elif fused:
        launch_ms = statistics.mean(p[0] for p in per_kernel)
        launch_bytes, kernel, ups_ms = sort_bytes, "fused_short_kernel (counts, every pass, fix-up)", None
    else:
        ups_ms = statistics.mean(p[0] for p in per_kernel)
        launch_ms = statistics.mean(statistics.mean(p[1:1 + passes]) for p in per_kernel)
        launch_bytes, kernel = n * 2 * (kbytes + vb), "onesweep_pass_kernel"
    achieved = launch_bytes / (launch_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1),
                "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s", "algorithmic_bytes_per_launch": launch_bytes,
                "mean_launch_ms": round(launch_ms, 4), "upsweep_ms": None if ups_ms is None else round(ups_ms, 4),
                "traffic_source": traffic_src}
    if stages is not None:
        roofline["msd_stages"] = stages
    sort_roofline = {"bytes_per_key": sort_bytes // n, "achieved": round(
        sort_bytes / (mean_sort_ms / 1e3) / 1e9, 1), "peak": hbm, "unit": "GB/s",
        "frac": round(sort_bytes / (mean_sort_ms / 1e3) / 1e9 / hbm, 4)}

    # comparator: CUB DeviceRadixSort (toolkit) on the same buffers, same timing
    cub = None
    cub_kind = {"c2b": 0, "c1": 0, "c2a": 1, "c3a": 2}.get(args.config)
    cub_lib_path = os.path.join(PKG, "lib", "libcubcompare.so")
    if rank == 0 and cub_kind is not None and os.path.exists(cub_lib_path) and not args.no_cub:
        import ctypes

        cl = ctypes.CDLL(cub_lib_path)
        cl.cubcmp_sort.restype = ctypes.c_int
        cl.cubcmp_sort.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4 + [
            ctypes.c_size_t, ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p,
            ctypes.POINTER(ctypes.c_int)]
        k_alt = torch.empty(n * kbytes, dtype=torch.uint8, device=dev)
        v_alt = torch.empty(max(1, n * vb), dtype=torch.uint8, device=dev)
        ctb = ctypes.c_size_t(0)
        sel = ctypes.c_int(0)
        vptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        cl.cubcmp_sort(cub_kind, int(desc), keys[0].data_ptr(), k_alt.data_ptr(), vptr(vals[0]), v_alt.data_ptr(), n,
                       None, ctypes.byref(ctb), ctypes.c_void_p(stream.cuda_stream), ctypes.byref(sel))
        ctemp = torch.empty(max(1, ctb.value), dtype=torch.uint8, device=dev)
        cub_ms = []
        for i in range(args.warmup + min(args.steps, 30)):
            prepare(i & 1, 555 + i)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            rc = cl.cubcmp_sort(cub_kind, int(desc), keys[i & 1].data_ptr(), k_alt.data_ptr(), vptr(vals[i & 1]),
                                v_alt.data_ptr(), n, ctemp.data_ptr(), ctypes.byref(ctb),
                                ctypes.c_void_p(stream.cuda_stream), ctypes.byref(sel))
            b.record(stream)
            if rc != 0:
                raise RuntimeError(f"CUB comparator failed: {rc}")
            if i >= args.warmup:
                cub_ms.append((a, b))
        torch.cuda.synchronize()
        cms = statistics.mean(a.elapsed_time(b) for a, b in cub_ms)
        cub = {"value": round(n / (cms / 1e3) / 1e9, 3), "unit": "Gkeys/s", "ms_per_step": round(cms, 4),
               "impl": "cub::DeviceRadixSort (CUDA 13.0 toolkit, DoubleBuffer)", "steps": len(cub_ms)}
        del k_alt, v_alt, ctemp

    # e2e: host buffers through the C ABI, copies inside the timed region
    e2e = None
    if (rank == 0 or world > 1) and args.e2e_steps > 0:
        e2e_steps = max(1, min(args.steps, args.e2e_steps))
        hbytes = n * kbytes
        h_src = torch.empty(hbytes, dtype=torch.uint8, pin_memory=True)
        h_work = torch.empty(hbytes, dtype=torch.uint8, pin_memory=True)
        hv_src = torch.empty(n * vb, dtype=torch.uint8, pin_memory=True) if vb else None
        hv_work = torch.empty(n * vb, dtype=torch.uint8, pin_memory=True) if vb else None
        prepare(0, 4242)
        h_src.copy_(keys[0])
        if vb:
            hv_src.copy_(vals[0])
        dbytes = gbsort.host_buffer_bytes(kt, n, vb)
        dbuf = torch.empty(dbytes, dtype=torch.uint8, device=dev)
        e2e_t = []
        for _ in range(e2e_steps + 1):
            h_work.copy_(h_src)
            if vb:
                hv_work.copy_(hv_src)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            gbsort.sort_host(h_work, n, kt, dbuf, dbytes, h_values=hv_work, value_bytes=vb, descending=desc,
                             stream=stream)
            e2e_t.append(time.perf_counter() - t0)
        e2e_t = e2e_t[1:]  # first call is a warm-up
        # the last result, back on the device: in order, and a permutation of the input
        chk = dbuf[:hbytes]
        chk.copy_(h_work)
        torch.cuda.synchronize()
        ordered = gbsort.check_order(chk, n, kt, descending=desc) == 0
        sum_out = gbsort.checksum(chk, n, kt)
        chk.copy_(h_src)
        torch.cuda.synchronize()
        e2e_ok = ordered and sum_out == gbsort.checksum(chk, n, kt)
        e2e = {"value": round(n / statistics.mean(e2e_t) / 1e9, 4), "unit": "Gkeys/s",
               "h2d_bytes_per_step": n * (kbytes + vb), "d2h_bytes_per_step": n * (kbytes + vb),
               "steps": e2e_steps, "ms_per_step": round(1000 * statistics.mean(e2e_t), 3),
               "api": "gbsort_sort_host (pinned host buffers)", "checked": e2e_ok}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        n_sample = min(n, 1 << 24)
        v, times = run_cpu_oracle(cfg, n_sample, threads=1, reps_min=1, budget_s=args.cpu_seconds)
        cpu = {"value": round(v, 5), "unit": "Gkeys/s", "cores": 1, "kind": "port",
               "sample": f"{n_sample} keys of the same distribution, std::stable_sort of twiddled keys, "
                         f"{len(times)} reps ({sum(times):.1f} s)"}

    if rank != 0:
        return None
    plan = gbsort.plan(kt, n, vb)
    line = {
        "metric": PLAIN_METRIC, "value": round(value, 3),
        "unit": "Gkeys/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_ms / args.steps, 4), "step_ms": step_stats(sort_ms),
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": (round(value / PUBLISHED[args.config][0], 3)
                        if args.config in PUBLISHED and cfg["n"] == CONFIGS[args.config]["n"] else None),
        "baseline_published": PUBLISHED.get(args.config, (None, None))[1],
        "dtype": kt, "data": "synthetic",
        "config": {"workload": cfg["workload"], "n": n, "key": kt, "value_bytes": vb, "descending": desc,
                   "passes": passes, "radix_bits": 8, "tile_items": plan.tile_items,
                   "threads": plan.threads, "items_per_thread": plan.items_per_thread,
                   "pass_ctas": plan.pass_ctas, "status_word_bytes": plan.status_word_bytes,
                   "flush": "inputs (>= 1 GiB) larger than L2, plus a 512 MiB L2 flush before every step",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "wall_ms_per_step_incl_input_generation": round(1000 * wall / args.steps, 3)},
        "roofline": roofline,
        "sort_roofline": sort_roofline,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "comparators": {"cub": cub},
        "clocks": clk,
        "gpu_launches": args.steps * (plan.kernel_launches + 1 + (1 if vb else 0)),
        "gpu_launches_note": "per step: generate (+values), then the sort's upsweep, one pass per key byte and "
                             "the pass-skip fix-up copy (exits at once when no pass was skipped), or for short "
                             "keys-only arrays one launch doing all of it, or for large keys-only 8- and 16-byte "
                             "keys also the six MSD kernels (the passes then exit at once); plus one memset",
        "sorted_check": ok,
    }
    return line


def bench_batched(args, cfg, world, rank, local):
    """Batched segmented sort vs looping the plain sort over the same segments."""
    import numpy as np
    import torch

    import gbsort
    from gbsort import gen

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    kt, vb = cfg["key"], cfg["vb"]
    # N GPUs: a global batch of N x segments, split by bytes (the same greedy
    # assignment on every rank, no collective); each rank sorts its share
    sizes_all = gen.log_uniform_sizes(cfg["segments"] * world, cfg["seg_log2"][0], cfg["seg_log2"][1], seed=2026)
    off_all = np.concatenate([[0], np.cumsum(sizes_all)]).astype(np.uint64)
    owner, rank_bytes = gbsort.partition_segments(off_all, world, KEY_BYTES[kt], vb)
    off, mine = gbsort.shard_offsets(off_all, owner, rank)
    sizes = sizes_all[mine]
    n = int(off[-1])
    keys = torch.empty(n, dtype=torch.int32, device=dev)
    vals = torch.empty(n, dtype=torch.int32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    # autotune the size buckets of this workload (not timed)
    scratch_bytes = (4 + vb) * (24 << 20) + (64 << 20)
    scratch = torch.empty(scratch_bytes, dtype=torch.uint8, device=dev)
    t0 = time.time()
    report = gbsort.autotune_segmented(kt, vb, scratch, scratch_bytes, cfg["seg_log2"][0], cfg["seg_log2"][1],
                                       stream=stream)
    tune_s = time.time() - t0
    del scratch

    plan = gbsort.SegmentedPlan(kt, off, vb)
    info = plan.info()
    ws = torch.empty(info["workspace_bytes"], dtype=torch.uint8, device=dev)
    plan.bind(keys, ws, info["workspace_bytes"], values=vals, stream=stream)

    def prepare(seed):
        with torch.cuda.stream(stream):
            gbsort.generate(0, 4, keys, n, seed, stream)
            gbsort.generate(3, 4, vals, n, 0, stream)  # value = index
            flush.fill_(seed & 0xFF)

    for w in range(args.warmup):
        prepare(10 + w)
        plan.run(stream=stream)
    if plan.status(stream=stream) != gbsort.OK:
        raise RuntimeError("batched warm-up reported an error")
    steps = max(1, min(args.steps, 40))
    ev = []
    clocks = ClockSampler(local) if rank == 0 else None
    barrier(world)
    torch.cuda.synchronize()
    for i in range(steps):
        prepare(100 + i)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        with TimedRange():
            plan.run(stream=stream)
        b.record(stream)
        ev.append((a, b))
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop() if clocks else None
    st = plan.status(stream=stream)
    if st != gbsort.OK:
        raise RuntimeError(f"batched run reported {gbsort.status_string(st)}")
    ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = max_over_ranks(world, sum(ms))
    value = steps * int(off_all[-1]) / (total_ms / 1e3) / 1e9  # every rank's keys / the slowest rank's time

    # device-side check of the last batch: every segment ascending, and each
    # (key, value) pair is an input pair (values are original indices)
    prepare(4242)
    with torch.cuda.stream(stream):
        orig = keys.clone()
    plan.run(stream=stream)
    torch.cuda.synchronize()
    seg_id = torch.repeat_interleave(torch.arange(len(sizes), device=dev), torch.as_tensor(sizes, device=dev))
    k64 = keys.to(torch.int64) & 0xFFFFFFFF
    ordered = bool(((k64[1:] >= k64[:-1]) | (seg_id[1:] != seg_id[:-1])).all().item())
    paired = bool(torch.equal(orig[vals.to(torch.int64)], keys))
    in_seg = bool(torch.equal(seg_id[vals.to(torch.int64)], seg_id))
    ok = ordered and paired and in_seg
    del k64, orig

    # baseline: the plain sort called once per segment, same GPU and data
    max_seg = int(sizes.max())
    tb = gbsort.temp_bytes(kt, max_seg, vb)
    lws = torch.empty(tb, dtype=torch.uint8, device=dev)
    loop_ms = []
    for r in range(2):
        prepare(300 + r)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        kp, vp = keys.data_ptr(), vals.data_ptr()
        for s in range(len(sizes)):
            m = int(sizes[s])
            o = int(off[s])
            gbsort.sort(kp + 4 * o, m, kt, lws, tb, values=vp + 4 * o, value_bytes=vb, stream=stream)
        b.record(stream)
        torch.cuda.synchronize()
        loop_ms.append(a.elapsed_time(b))
    loop_value = n / (min(loop_ms) / 1e3) / 1e9

    # e2e: the batch arrives in pinned host memory and goes back there, through
    # gbsort_segmented_sort_host (planning, copies and sorting inside the
    # timed region); every call gets the same unsorted input
    e2e = None
    if args.e2e_steps > 0:
        h_src_k = torch.empty(n * 4, dtype=torch.uint8, pin_memory=True)
        h_src_v = torch.empty(n * vb, dtype=torch.uint8, pin_memory=True)
        hk = torch.empty(n * 4, dtype=torch.uint8, pin_memory=True)
        hv = torch.empty(n * vb, dtype=torch.uint8, pin_memory=True)
        prepare(777)
        torch.cuda.synchronize()
        h_src_k.copy_(keys.view(torch.uint8))
        h_src_v.copy_(vals.view(torch.uint8))
        hbytes = gbsort.segmented_host_buffer_bytes(kt, off, vb)
        del plan, ws  # the batched run's plan and workspace are not needed any more
        torch.cuda.empty_cache()
        dbuf = torch.empty(hbytes, dtype=torch.uint8, device=dev)
        e2e_t = []
        for _ in range(min(args.e2e_steps, 3) + 1):
            hk.copy_(h_src_k)
            hv.copy_(h_src_v)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            gbsort.segmented_sort_host(hk, kt, off, dbuf, hbytes, h_values=hv, value_bytes=vb, stream=stream)
            e2e_t.append(time.perf_counter() - t0)
        e2e_t = e2e_t[1:]
        # the last result, back on the device: every segment ascending and
        # each (key, value) pair an input pair (values are original indices)
        keys.view(torch.uint8).copy_(h_src_k)
        torch.cuda.synchronize()
        orig = keys.clone()
        keys.view(torch.uint8).copy_(hk)
        vals.view(torch.uint8).copy_(hv)
        torch.cuda.synchronize()
        k64 = keys.to(torch.int64) & 0xFFFFFFFF
        e2e_ok = bool(((k64[1:] >= k64[:-1]) | (seg_id[1:] != seg_id[:-1])).all().item()) and \
            bool(torch.equal(orig[vals.to(torch.int64)], keys)) and \
            bool(torch.equal(seg_id[vals.to(torch.int64)], seg_id))
        del k64, orig, dbuf
        e2e = {"value": round(n / statistics.mean(e2e_t) / 1e9, 3), "unit": "Gkeys/s",
               "h2d_bytes_per_step": n * (4 + vb), "d2h_bytes_per_step": n * (4 + vb), "steps": len(e2e_t),
               "ms_per_step": round(1e3 * statistics.mean(e2e_t), 3),
               "api": "gbsort_segmented_sort_host (pinned host buffers; groups of segments copied in, sorted "
                      "and copied back on overlapping streams)", "checked": e2e_ok}
        del hk, hv

    # CPU oracle on a bounded sample of the segments (1 thread)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "tests"))
        import _oracle

        oracle = _oracle.load()
        spent, done_keys, count = 0.0, 0, 0
        for s in np.random.default_rng(6).permutation(len(sizes)):
            if spent > min(args.cpu_seconds, 15.0):
                break
            m = int(sizes[s])
            raw = gen.generate(0, 4, m, 1000 + count)
            t1 = time.perf_counter()
            oracle.sort(kt, raw, False, np.arange(m, dtype=np.uint32))
            spent += time.perf_counter() - t1
            done_keys += m
            count += 1
        cpu = {"value": round(done_keys / spent / 1e9, 5), "unit": "Gkeys/s", "cores": 1, "kind": "port",
               "sample": f"{count} segments of the workload ({done_keys} keys), std::stable_sort of twiddled keys "
                         f"with u32 values, 1 thread"}

    hbm, peak_kind = peaks()
    algo_bytes = info["keys_in_cta"] * 2 * (4 + vb) + info["keys_in_onesweep"] * (4 + 4 * 2 * (4 + vb))
    run_traffic, run_traffic_src = committed_traffic(args.config, n)
    mean_ms = total_ms / steps
    if rank != 0:
        return None
    line = {
        "metric": BATCHED_METRIC, "value": round(value, 3), "unit": "Gkeys/s",
        "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": round(mean_ms, 4),
        "step_ms": step_stats(ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": kt,
        "data": "synthetic",
        "config": {"workload": cfg["workload"], "n_keys": n, "segments": len(sizes), "value_bytes": vb,
                   "sharding": {"global_segments": len(sizes_all), "ranks": world,
                                "rank_bytes": [int(x) for x in rank_bytes]} if world > 1 else None,
                   "paths": {k: info[k] for k in ("cta_small4_segments", "cta_small_segments",
                                                  "cta_large_segments", "onesweep_segments", "onesweep_tiles",
                                                  "keys_in_cta", "keys_in_onesweep")},
                   "graph": "captured on the first run, replayed", "flush": "512 MiB L2 flush before every step"},
        "loop_baseline": {"value": round(loop_value, 3), "unit": "Gkeys/s", "ms": round(min(loop_ms), 3),
                          "impl": "gbsort_sort_pairs called once per segment (4096 calls), same GPU and data"},
        "speedup_vs_loop": round(value / loop_value, 2),
        "roofline": {"bound": "hbm", "kernel": "the batched run (segment upsweep, CTA sorts, onesweep passes over "
                                                "the tile list) as one graph",
                     "algorithmic_bytes": algo_bytes,
                     "achieved": round(algo_bytes / (mean_ms / 1e3) / 1e9, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(algo_bytes / (mean_ms / 1e3) / 1e9 / hbm, 4), "traffic": run_traffic,
                     "traffic_source": run_traffic_src,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "note": "CTA-sorted keys move 2*(K+V) bytes, onesweep keys K + P*2*(K+V); timed per replay; "
                             "traffic: DRAM bytes of one run, from a smaller capture scaled by keys (a lower "
                             "estimate: the smaller run keeps part of each pass in L2)"},
        "e2e": e2e,
        "cpu_baseline": cpu,
        "clocks": clk,
        "autotune": {"seconds": round(tune_s, 1), "report": report.strip().splitlines()},
        "sorted_check": ok,
        "gpu_launches": steps * (info["kernel_launches"] + 2),
        "gpu_launches_note": "per step: the batched run's kernels plus two input-generation kernels",
    }
    return line


def bench_serving(args, cfg, world, rank, local):
    """Sort server (continuous batching) fed from pinned host buffers.

    Phase 1, capacity: a backlog of requests is submitted at once and the
    time to drain it gives the sustained throughput (value).  Phase 2, load:
    Poisson arrivals at `--rate` (default: cfg load x capacity) give the
    p50/p99 latency from submit to result-in-host-memory.  A sample of
    requests gets its own output buffers and is compared, bit for bit, with
    the same request sorted alone by the plain sort."""
    import numpy as np
    import torch

    import gbsort

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rng = np.random.default_rng(5150 + rank)
    lo, hi = cfg["size_log2"]
    pool_keys = 1 << (hi + 1)
    types = ("u32", "u64", "f32")
    dist = {"u32": 0, "u64": 0, "f32": 1}
    host_in = {}
    for i, kt in enumerate(types):
        d = torch.empty(pool_keys * KEY_BYTES[kt], dtype=torch.uint8, device=dev)
        gbsort.generate(dist[kt], KEY_BYTES[kt], d, pool_keys, 71 + i)
        torch.cuda.synchronize()
        host_in[kt] = d.cpu().pin_memory()
        del d
    vals_in = torch.arange(pool_keys, dtype=torch.int32).pin_memory()
    # outputs of unchecked requests land in one shared pinned scratch area
    out_keys = torch.empty((1 << hi) * 8, dtype=torch.uint8).pin_memory()
    out_vals = torch.empty((1 << hi) * 4, dtype=torch.uint8).pin_memory()

    def draw():
        kt = types[int(rng.integers(3))]
        n = int(np.floor(2.0 ** rng.uniform(lo, hi)))
        has_v = bool(rng.random() < 0.5)
        off = int(rng.integers(0, pool_keys - n + 1))
        return kt, n, has_v, off

    checks = []
    check_out = {}

    def plan_checks(reqs, tag):
        """Pinned outputs of every 64th request, allocated before timing."""
        for i, (kt, n, has_v, off) in enumerate(reqs):
            if i % 64 == 0:
                ko = torch.empty(n * KEY_BYTES[kt], dtype=torch.uint8).pin_memory()
                vo = torch.empty(n * 4, dtype=torch.uint8).pin_memory() if has_v else None
                check_out[(tag, i)] = (ko, vo)
                checks.append((reqs[i], ko, vo))

    def submit(srv, req, key=None):
        kt, n, has_v, off = req
        kb = KEY_BYTES[kt]
        kin = host_in[kt].data_ptr() + off * kb
        vin = vals_in.data_ptr() + off * 4 if has_v else None
        if key in check_out:
            ko, vo = check_out[key]
            kout, vout = ko.data_ptr(), (vo.data_ptr() if has_v else None)
        else:
            kout, vout = out_keys.data_ptr(), (out_vals.data_ptr() if has_v else None)
        return srv.submit(kt, n, kin, kout, vin, vout, value_bytes=4 if has_v else 0)

    # host link: plain pinned copies of 256 MiB each way
    probe = host_in["u64"]
    dprobe = torch.empty(probe.numel(), dtype=torch.uint8, device=dev)
    link = {}
    for name, dst, src in (("h2d_gbs", dprobe, probe), ("d2h_gbs", probe, dprobe)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(4):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        link[name] = round(4 * probe.numel() / (time.perf_counter() - t1) / 1e9, 1)
    # both directions at once (the serving pattern): H2D of one buffer while
    # another comes back, on two streams
    probe2 = host_in["u32"]
    dprobe2 = torch.empty(probe2.numel(), dtype=torch.uint8, device=dev)
    s_up, s_dn = torch.cuda.Stream(), torch.cuda.Stream()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(4):
        with torch.cuda.stream(s_up):
            dprobe.copy_(probe, non_blocking=True)
        with torch.cuda.stream(s_dn):
            out_keys[:probe2.numel()].copy_(dprobe2, non_blocking=True)
    torch.cuda.synchronize()
    link["bidir_gbs"] = round(4 * (probe.numel() + probe2.numel()) / (time.perf_counter() - t1) / 1e9, 1)
    del dprobe, dprobe2

    srv = gbsort.Server(pool_bytes=cfg["pool"], streams=cfg["streams"])
    # warm-up: every kernel shape once
    for _ in range(max(3, args.warmup) * 10):
        submit(srv, draw())
    if srv.drain(600.0) != gbsort.OK:
        raise RuntimeError("server warm-up did not drain")

    # phase 1: capacity under a backlog
    n_cap = max(200, args.steps * 20)
    reqs = [draw() for _ in range(n_cap)]
    plan_checks(reqs, "cap")
    keys_cap = sum(r[1] for r in reqs)
    bytes_in = sum(r[1] * (KEY_BYTES[r[0]] + (4 if r[2] else 0)) for r in reqs)
    sort_bytes = sum(r[1] * (KEY_BYTES[r[0]] + KEY_BYTES[r[0]] * 2 * (KEY_BYTES[r[0]] + (4 if r[2] else 0)))
                     for r in reqs)
    srv.reset_stats()
    clock = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tickets = [submit(srv, r, ("cap", i)) for i, r in enumerate(reqs)]
    if srv.drain(1200.0) != gbsort.OK:
        raise RuntimeError("server did not drain")
    t_cap = time.perf_counter() - t0
    torch.cuda.synchronize()
    barrier(world)
    clocks = clock.stop()
    cap_stats = srv.stats()
    bad = [t for t in tickets if srv.poll(t) != gbsort.OK]
    t_cap = max_over_ranks(world, t_cap)
    value = world * keys_cap / t_cap / 1e9
    cap_rps = n_cap / t_cap

    # phase 2: Poisson arrivals at a fraction of capacity
    rate = args.rate if args.rate > 0 else cfg["load"] * cap_rps
    n_load = max(200, args.steps * 10)
    reqs2 = [draw() for _ in range(n_load)]
    plan_checks(reqs2, "load")
    gaps = rng.exponential(1.0 / rate, n_load)
    srv.reset_stats()
    late = 0.0
    t0 = time.perf_counter()
    t_next = t0
    tickets2 = []
    for i, r in enumerate(reqs2):
        t_next += gaps[i]
        while True:
            now = time.perf_counter()
            if now >= t_next:
                break
            if t_next - now > 2e-4:
                time.sleep((t_next - now) * 0.5)
        late = max(late, now - t_next)
        tickets2.append(submit(srv, r, ("load", i)))
    if srv.drain(1200.0) != gbsort.OK:
        raise RuntimeError("server did not drain under load")
    t_load = time.perf_counter() - t0
    load_stats = srv.stats()
    bad += [t for t in tickets2 if srv.poll(t) != gbsort.OK]
    srv.close()

    # alone vs in the mix: the checked requests, re-sorted by the plain sort
    same = 0
    for (kt, n, has_v, off), ko, vo in checks:
        kb = KEY_BYTES[kt]
        dk = host_in[kt][off * kb:(off + n) * kb].to(dev)
        dv = vals_in[off:off + n].to(dev) if has_v else None
        tb = gbsort.temp_bytes(kt, n, 4 if has_v else 0)
        ws = torch.empty(tb, dtype=torch.uint8, device=dev)
        gbsort.sort(dk, n, kt, ws, tb, values=dv, value_bytes=4 if has_v else 0)
        torch.cuda.synchronize()
        ok = torch.equal(dk.cpu(), ko) and (not has_v or torch.equal(dv.cpu().view(torch.uint8), vo))
        same += int(ok)
    identical = same == len(checks) and not bad

    # CPU oracle on a bounded sample of requests (1 thread)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "tests"))
        import _oracle

        oracle = _oracle.load()
        budget = min(args.cpu_seconds, 20.0)
        done_keys, spent, count = 0, 0.0, 0
        while spent < budget and count < 200:
            kt, n, has_v, off = draw()
            kb = KEY_BYTES[kt]
            raw = host_in[kt][off * kb:(off + n) * kb].numpy().view(np.uint32 if kb == 4 else np.uint64).copy()
            v = vals_in[off:off + n].numpy().view(np.uint32).copy() if has_v else None
            t1 = time.perf_counter()
            oracle.sort(kt, raw, False, v)
            spent += time.perf_counter() - t1
            done_keys += n
            count += 1
        cpu = {"value": round(done_keys / spent / 1e9, 5), "unit": "Gkeys/s", "cores": 1, "kind": "port",
               "sample": f"{count} requests of the same distribution ({done_keys} keys), std::stable_sort of "
                         f"twiddled keys, 1 thread, sorting only (no copies)"}
    if rank != 0:
        return None
    mean_keys = keys_cap / n_cap
    hbm, _ = peaks()
    line = {
        "metric": SERVING_METRIC,
        "value": round(value, 3), "unit": "Gkeys/s", "n_gpus": world, "steps": n_cap, "warmup": args.warmup,
        "ms_per_step": round(1e3 * t_cap / n_cap, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32/u64/f32 keys, u32 values", "data": "synthetic",
        "config": {"workload": cfg["workload"], "step": "one request (capacity phase: backlog of all requests)",
                   "requests_capacity_phase": n_cap, "requests_load_phase": n_load,
                   "mean_request_keys": round(mean_keys), "pool_bytes": cfg["pool"], "streams": cfg["streams"],
                   "flush": "inputs (1.5 GiB of pinned host pools) larger than L2; every request is copied in"},
        "capacity": {"seconds": round(t_cap, 4), "requests_per_s": round(cap_rps, 1),
                     "batches": cap_stats["batches"], "mean_batch_requests": round(cap_stats["mean_batch_requests"], 2),
                     "max_batch_requests": cap_stats["max_batch_requests"],
                     "pool_peak_gib": round(cap_stats["pool_peak_bytes"] / 2**30, 2),
                     "link_gbs": round(2 * bytes_in / t_cap / 1e9, 1), "link_probe": link,
                     "host_plan_s": round(cap_stats["host_plan_seconds"], 4),
                     "host_launch_s": round(cap_stats["host_launch_seconds"], 4),
                     "batch_s_sum": round(cap_stats["batch_seconds"], 4),
                     "stage_device_s": {"h2d": round(cap_stats["h2d_seconds"], 4),
                                        "sort": round(cap_stats["sort_seconds"], 4),
                                        "d2h": round(cap_stats["d2h_seconds"], 4)}},
        "latency": {"rate_rps": round(rate, 1), "load_fraction": round(rate / cap_rps, 3),
                    "p50_ms": round(load_stats["latency_p50_us"] / 1e3, 3),
                    "p99_ms": round(load_stats["latency_p99_us"] / 1e3, 3),
                    "mean_ms": round(load_stats["latency_mean_us"] / 1e3, 3),
                    "max_ms": round(load_stats["latency_max_us"] / 1e3, 3),
                    "queue_p50_ms": round(load_stats["queue_p50_us"] / 1e3, 3),
                    "queue_p99_ms": round(load_stats["queue_p99_us"] / 1e3, 3),
                    "sustained_gkeys": round(load_stats["keys_sorted"] / max(load_stats["active_seconds"], 1e-9)
                                             / 1e9, 3),
                    "mean_batch_requests": round(load_stats["mean_batch_requests"], 2),
                    "arrival_max_late_ms": round(1e3 * late, 3), "seconds": round(t_load, 3)},
        "e2e": {"value": round(value, 3), "unit": "Gkeys/s", "h2d_bytes_per_step": int(bytes_in / n_cap),
                "d2h_bytes_per_step": int(bytes_in / n_cap),
                "api": "gbsort_server_submit / drain with pinned HOST buffers (value is already end to end)"},
        "roofline": {"bound": "hbm", "kernel": "batched sort (onesweep_pass_kernel over the batch's tile list)",
                     "achieved": round(sort_bytes / max(cap_stats["sort_seconds"], 1e-9) / 1e9, 1), "peak": hbm,
                     "unit": "GB/s", "frac": round(sort_bytes / max(cap_stats["sort_seconds"], 1e-9) / 1e9 / hbm, 4),
                     "traffic": None, "algorithmic_bytes": sort_bytes,
                     "note": "K + P*2*(K+V) bytes per key over the batches' summed sort time (CUDA events on the "
                             "sort stream); the request mix is bound by the host link, see link_roofline"},
        "link_roofline": {"achieved": round(2 * bytes_in / t_cap / 1e9, 1), "peak": link.get("bidir_gbs"),
                          "unit": "GB/s", "frac": round(2 * bytes_in / t_cap / 1e9 / max(link.get("bidir_gbs", 1), 1e-9),
                                                        4),
                          "note": "host<->device bytes of the capacity phase over its wall time, against pinned "
                                  "copies in both directions at once"},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": cap_stats["kernel_launches"],
        "identical_alone_and_in_mix": identical, "checked_requests": len(checks), "failed_requests": len(bad),
    }
    return line


def _sub_args(args, config, steps):
    """Arguments of a companion run: few steps, no CPU baseline (the headline
    line carries it), short e2e."""
    import copy

    sub = copy.copy(args)
    sub.config = config
    sub.steps = steps
    sub.warmup = 3
    sub.no_cpu_baseline = True
    sub.e2e_steps = min(args.e2e_steps, 2)
    sub.n = 0
    sub.rate = 0.0
    sub.segments = 0
    return sub


def _release_device_memory():
    import gc

    import torch

    gc.collect()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()


def companion_runs(args, local) -> dict:
    """The rest of the benchmark metric beside the 2^28 u32 headline, on the
    same GPU after it: the other plain configurations (c1, c2a, c3a, c3b),
    the batched sort of 4096 segments against looping the plain sort (c4) and
    the sort server's capacity and p50/p99 latency at load (c5).  Each is the
    same measurement as its own --config run, with fewer steps."""
    out = {}
    plain = {}
    for c, steps in (("c1", 50), ("c2a", 10), ("c3a", 8), ("c3b", 8)):
        t0 = time.time()
        try:
            ln = bench_gbsort(_sub_args(args, c, steps), CONFIGS[c], 1, 0, local)
            plain[c] = {
                "workload": ln["config"]["workload"], "value": ln["value"], "unit": ln["unit"],
                "ms_per_step": ln["ms_per_step"], "steps": ln["steps"], "vs_baseline": ln["vs_baseline"],
                "baseline_published": ln["baseline_published"],
                "roofline": {k: ln["roofline"][k] for k in ("kernel", "achieved", "peak", "unit", "frac",
                                                            "mean_launch_ms", "algorithmic_bytes_per_launch")},
                "sort_roofline": ln["sort_roofline"], "passes": ln["config"]["passes"],
                "e2e": ln["e2e"], "cub": (ln["comparators"]["cub"] or {}).get("value"),
                "sorted_check": ln["sorted_check"], "clocks": ln["clocks"],
                "seconds": round(time.time() - t0, 1)}
        except Exception as e:  # one companion failing does not void the headline
            plain[c] = {"error": f"{type(e).__name__}: {e}"}
        _release_device_memory()
    out["plain_configs"] = plain
    t0 = time.time()
    try:
        ln = bench_batched(_sub_args(args, "c4", 10), CONFIGS["c4"], 1, 0, local)
        out["batched"] = {
            "metric": ln["metric"], "workload": ln["config"]["workload"], "value": ln["value"], "unit": ln["unit"],
            "ms_per_step": ln["ms_per_step"], "steps": ln["steps"], "n_keys": ln["config"]["n_keys"],
            "segments": ln["config"]["segments"], "speedup_vs_loop": ln["speedup_vs_loop"],
            "loop_baseline": ln["loop_baseline"], "roofline": ln["roofline"], "e2e": ln["e2e"],
            "paths": ln["config"]["paths"], "sorted_check": ln["sorted_check"], "clocks": ln["clocks"],
            "gpu_launches": ln["gpu_launches"], "seconds": round(time.time() - t0, 1)}
    except Exception as e:
        out["batched"] = {"error": f"{type(e).__name__}: {e}"}
    _release_device_memory()
    t0 = time.time()
    try:
        ln = bench_serving(_sub_args(args, "c5", 20), CONFIGS["c5"], 1, 0, local)
        out["serving"] = {
            "metric": ln["metric"], "workload": ln["config"]["workload"], "value": ln["value"], "unit": ln["unit"],
            "requests_capacity_phase": ln["config"]["requests_capacity_phase"],
            "requests_load_phase": ln["config"]["requests_load_phase"], "capacity": ln["capacity"],
            "latency": ln["latency"], "identical_alone_and_in_mix": ln["identical_alone_and_in_mix"],
            "checked_requests": ln["checked_requests"], "failed_requests": ln["failed_requests"],
            "roofline": ln["roofline"], "link_roofline": ln["link_roofline"], "e2e": ln["e2e"],
            "clocks": ln["clocks"], "gpu_launches": ln["gpu_launches"], "seconds": round(time.time() - t0, 1)}
    except Exception as e:
        out["serving"] = {"error": f"{type(e).__name__}: {e}"}
    _release_device_memory()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", default="c2b", choices=sorted(CONFIGS))
    ap.add_argument("--impl", default="gbsort", choices=["gbsort", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cub", action="store_true", help="skip the CUB comparator")
    ap.add_argument("--n", type=int, default=0,
                    help="override the configuration's key count (a smaller case for profiling)")
    ap.add_argument("--segments", type=int, default=0,
                    help="c4: override the number of segments (a smaller batch for profiling)")
    ap.add_argument("--rate", type=float, default=0.0,
                    help="c5: Poisson arrival rate in requests/s (0: the configured fraction of measured capacity)")
    ap.add_argument("--headline-only", action="store_true",
                    help="c2b: skip the companion runs (other plain configurations, batched, serving)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)  # timing rule: at least 3 warm-up steps
    world, rank, local = dist_init()
    cfg = CONFIGS[args.config]
    if args.n > 0 and cfg["n"]:
        cfg = dict(cfg, n=args.n, workload=cfg["workload"] + f" (n overridden to {args.n})")
    if args.segments > 0 and "segments" in cfg:
        cfg = dict(cfg, segments=args.segments, workload=cfg["workload"] + f" (segments overridden to {args.segments})")
    if args.impl == "reference":
        bench_reference(args, cfg, world, rank)
    else:
        if cfg.get("serving"):
            line = bench_serving(args, cfg, world, rank, local)
        elif "segments" in cfg:
            line = bench_batched(args, cfg, world, rank, local)
        else:
            line = bench_gbsort(args, cfg, world, rank, local)
        if line is not None and args.config == "c2b" and args.n == 0 and world == 1 and not args.headline_only:
            _release_device_memory()
            t0 = time.time()
            line.update(companion_runs(args, local))
            line["companion_seconds"] = round(time.time() - t0, 1)
        if line is not None:
            print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
