"""Benchmark and validation command line of gbsort, with the reference's
options and defaults (benchmark/bench_parser.cpp:11-106, bench_parser.h:14-17,
benchmark/radix_gpu.cu):

    python -m gbsort.cli [--n N] [--iterations I] [--warmup W] [--warmup_ms MS]
                         [--descending] [--validation] [--help]

Without --validation it benchmarks one sort (default: 2^27 random uint32_t,
ascending) and prints the reference's statistics block plus p50/p99 and the
post-sort checks [order, counts, pairs].  --validation runs the reference's
sweep (benchmark/validate_sort.cuh:20-147): 13 key types x values (none, u32,
u8, u16, u64, u128) x input modes (random, byte_skip, asc) x both orders x
sizes 1000, 100, 10 and 11 powers of two, checking each result on the device.

Options beyond the reference: --type / --values / --mode pick the benchmarked
key type, value type and input mode; --scaling LO:HI with --dump FILE times
n = 2^LO .. 2^HI and writes the times in the layout of the reference's
plotting data (data/logs/benchmark_data.py: scaling_avg / scaling_std,
{type: {log2 n: (ms, ...)}}); --max_log2 caps the validation sizes.
"""

from __future__ import annotations

import argparse
import math
import statistics
import sys
import time

import gbsort

# C type names the reference prints -> gbsort key types
TYPE_NAMES = {
    "uint8_t": "u8", "uint16_t": "u16", "uint32_t": "u32", "uint64_t": "u64", "unsigned __int128": "u128",
    "int8_t": "i8", "int16_t": "i16", "int32_t": "i32", "int64_t": "i64", "__int128": "i128",
    "float": "f32", "double": "f64", "long double": "f128",
}
SHORT_TO_C = {v: k for k, v in TYPE_NAMES.items()}
VALUE_TYPES = {"none": 0, "uint32_t": 4, "uint8_t": 1, "uint16_t": 2, "uint64_t": 8, "unsigned __int128": 16}
MODES = {"random": 4, "byte_skip": 5, "asc": 3}  # gbsort_generate distributions (the reference's init_keys)
# validation order of the reference (validate_sort.cuh:34-44)
VALIDATION_TYPES = ["uint32_t", "uint8_t", "uint16_t", "uint64_t", "unsigned __int128", "int16_t", "int8_t",
                    "int32_t", "int64_t", "__int128", "float", "double", "long double"]


def key_type(name: str) -> str:
    if name in TYPE_NAMES:
        return TYPE_NAMES[name]
    if name in gbsort.KEY_TYPES:
        return name
    raise SystemExit(f"Error: unknown key type: {name}")


class Bench:
    """Device buffers of one (type, values, n) case: input keys (kept),
    working keys, values, workspace."""

    def __init__(self, torch, kt: str, vb: int, n: int, mode: str, desc: bool):
        self.torch, self.kt, self.vb, self.n, self.mode, self.desc = torch, kt, vb, n, mode, desc
        self.kb = gbsort.KEY_BYTES[kt]
        dev = torch.device("cuda")
        self.src = torch.empty(max(1, n * self.kb), dtype=torch.uint8, device=dev)
        self.keys = torch.empty_like(self.src)
        self.vsrc = torch.empty(max(1, n * vb), dtype=torch.uint8, device=dev) if vb else None
        self.vals = torch.empty_like(self.vsrc) if vb else None
        self.tb = gbsort.temp_bytes(kt, n, vb)
        self.ws = torch.empty(max(1, self.tb), dtype=torch.uint8, device=dev)
        self.stream = torch.cuda.current_stream()
        self.seed = 1

    def fill(self):
        """Fresh input (a new seed each time), copied into the working buffers."""
        self.seed += 1
        if self.n:
            gbsort.generate(MODES[self.mode], self.kb, self.src, self.n, self.seed, self.stream)
            if self.vb:  # values = original index where it fits, else random bits
                dist = 3 if self.vb in (4, 8) else 0
                gbsort.generate(dist, self.vb, self.vsrc, self.n, self.seed ^ 0x55, self.stream)
        self.keys.copy_(self.src)
        if self.vb:
            self.vals.copy_(self.vsrc)

    def sort(self):
        gbsort.sort(self.keys, self.n, self.kt, self.ws, self.tb, values=self.vals, value_bytes=self.vb,
                    descending=self.desc, stream=self.stream)

    def checks(self):
        """[order, counts, pairs] of the last sort, on the device."""
        n, kt = self.n, self.kt
        order = gbsort.check_order(self.keys, n, kt, self.desc) == 0
        counts = gbsort.checksum(self.keys, n, kt) == gbsort.checksum(self.src, n, kt)
        pairs = True
        if self.vb in (4, 8):
            pairs = gbsort.check_pairs(self.src, self.keys, self.vals, self.vb, n, kt) == 0
        elif self.vb:
            pairs = gbsort.checksum(self.vals, n * self.vb, "u8") == gbsort.checksum(self.vsrc, n * self.vb, "u8")
        ok = gbsort.workspace_status(kt, n, self.ws, self.vb) == gbsort.OK
        return order and ok, counts, pairs

    def time(self, iterations: int, warmups: int, warm_ms: float):
        torch = self.torch
        t_end = time.perf_counter() + warm_ms / 1e3
        done = 0
        while done < warmups or time.perf_counter() < t_end:
            self.fill()
            self.sort()
            torch.cuda.synchronize()
            done += 1
        ms = []
        for _ in range(iterations):
            self.fill()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(self.stream)
            self.sort()
            b.record(self.stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return ms, done


def stats(ms):
    s = sorted(ms)
    pick = lambda q: s[min(len(s) - 1, int(round(q * (len(s) - 1))))]  # noqa: E731
    return {"avg": statistics.mean(ms), "std_us": (statistics.pstdev(ms) * 1e3) if len(ms) > 1 else 0.0,
            "p50": pick(0.5), "p99": pick(0.99)}


def run_benchmark(torch, args) -> int:
    kt = key_type(args.type)
    vb = VALUE_TYPES[args.values]
    b = Bench(torch, kt, vb, args.n, args.mode, args.descending)
    ms, warm = b.time(args.iterations, args.warmup, args.warmup_ms)
    st = stats(ms)
    plan = gbsort.plan(kt, args.n, vb)
    order, counts, pairs = b.checks()
    prop = torch.cuda.get_device_properties(0)
    print(f"\nGPU: {prop.name}\n")
    print(f"RADIX\t=\t{plan.radix_bits}\nN\t=\t{args.n}\nType\t=\t{SHORT_TO_C[kt]}\nBlocks\t=\t{plan.num_tiles}\n"
          f"Threads\t=\t{plan.threads}\nit/thd\t=\t{plan.items_per_thread}\n"
          f"Memory\t=\t{b.tb / 1048576:.3f} MB\nTime\t=\t{st['avg']:.3f} ms (+- {st['std_us']:.3f} us)\n"
          f"\t\t({len(ms)} avg w/ {warm} wm)\n"
          f"p50/p99\t=\t{st['p50']:.3f} / {st['p99']:.3f} ms\n"
          f"it/s\t=\t{int(args.n / (st['avg'] / 1e3)) if st['avg'] > 0 else 0}\n"
          f"ps/el\t=\t{(st['avg'] * 1e9 / args.n) if args.n else 0:.3f}\n"
          f"Mode\t=\t{args.mode}\nOrder\t=\t{'DESC' if args.descending else 'ASC'}\n"
          f"Pairs\t=\t{args.values if vb else 'No'}\n"
          f"Passes\t=\t{plan.passes} (uniform-digit passes skipped on the device: "
          f"{'on' if gbsort.get_pass_skip() else 'off'})")
    print(f"Post sort checks [order, hist, pair]: [{int(order)}, {int(counts)}, {int(pairs)}]")
    return 0 if (order and counts and pairs) else 1


def run_scaling(torch, args) -> int:
    lo, hi = (int(x) for x in args.scaling.split(":"))
    kt = key_type(args.type)
    vb = VALUE_TYPES[args.values]
    cname = SHORT_TO_C[kt]
    avg, std = {}, {}
    ok_all = True
    for e in range(lo, hi + 1):
        b = Bench(torch, kt, vb, 1 << e, args.mode, args.descending)
        ms, _ = b.time(args.iterations, args.warmup, args.warmup_ms)
        st = stats(ms)
        ok_all &= all(b.checks())
        avg[e], std[e] = st["avg"], st["std_us"] / 1e3
        print(f"2^{e}: {st['avg']:.3f} ms (+- {st['std_us']:.3f} us)", flush=True)
        del b
    if args.dump:
        with open(args.dump, "w") as f:
            f.write("import numpy as np\n\n# gbsort (GB300 onesweep), ms per sort\n\n")
            for name, d in (("scaling_avg", avg), ("scaling_std", std)):
                f.write(f"{name} = {{\n    \"{cname}\": {{\n")
                for e in sorted(d):
                    f.write(f"        {e}: ({d[e]:.3f},),\n")
                f.write("    },\n}\n\n")
        print(f"wrote {args.dump}")
    return 0 if ok_all else 1


def max_array_bits(total_bytes: int, bytes_per_el: int) -> int:
    """Largest power of two whose keys, values, input copy and workspace fit
    in about a quarter of the device memory."""
    return max(10, int(math.floor(math.log2(max(1, total_bytes // 4) / (3 * bytes_per_el)))))


def run_validation(torch, args) -> int:
    total = passed = 0
    mem = torch.cuda.get_device_properties(0).total_memory
    for mode in MODES:
        for desc in (False, True):
            for cname in VALIDATION_TYPES:
                kt = TYPE_NAMES[cname]
                for vname, vb in VALUE_TYPES.items():
                    bit_end = min(args.max_log2, max_array_bits(mem, gbsort.KEY_BYTES[kt] + vb))
                    bit_start = bit_end - 10
                    sizes = [1000, 100, 10] + [1 << i for i in range(bit_start, bit_end + 1)]
                    for n in sizes:
                        b = Bench(torch, kt, vb, n, mode, desc)
                        ms, warm = b.time(args.iterations, args.warmup, 0.0)
                        ok = all(b.checks())
                        total += 1
                        passed += int(ok)
                        pair = f"Pair: {vname}, " if vb else ""
                        print(f"Sorting {n} els of type {cname}, {pair}({b.tb / 1048576:.3f} MB)"
                              f"({'DESC' if desc else 'ASC'}), {mode} array - {statistics.mean(ms):.3f} ms"
                              f"({len(ms)} avg + {warm} wm)... {'passed' if ok else 'failed'}", flush=True)
                        del b
    print(f"\nDone... passed {passed}/{total} tests.")
    return 0 if passed == total else 1


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m gbsort.cli", description=__doc__.split("\n\n")[0],
                                 formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--n", type=int, default=1 << 27, help="Number of elements")
    ap.add_argument("--iterations", type=int, default=30, help="Timed iterations")
    ap.add_argument("--warmup", type=int, default=10, help="Warmup iterations")
    ap.add_argument("--warmup_ms", type=float, default=250.0, help="Minimum warmup time (ms)")
    ap.add_argument("--descending", action="store_true", help="Sort descending")
    ap.add_argument("--validation", action="store_true", help="Validate algorithm")
    ap.add_argument("--type", default="uint32_t", help="key type (C name or u32, f64, ...)")
    ap.add_argument("--values", default="none", choices=list(VALUE_TYPES), help="value type")
    ap.add_argument("--mode", default="random", choices=list(MODES), help="input mode")
    ap.add_argument("--scaling", default=None, help="LO:HI: time n = 2^LO .. 2^HI")
    ap.add_argument("--dump", default=None, help="with --scaling: write the plotting data file")
    ap.add_argument("--max_log2", type=int, default=24, help="largest validation size (log2)")
    args = ap.parse_args(argv)
    import torch

    if not torch.cuda.is_available():
        print("Error: no CUDA device", file=sys.stderr)
        return 2
    if args.validation:
        return run_validation(torch, args)
    if args.scaling:
        return run_scaling(torch, args)
    return run_benchmark(torch, args)


if __name__ == "__main__":
    sys.exit(main())
