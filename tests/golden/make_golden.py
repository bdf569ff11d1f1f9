"""Generates tests/golden/ fixtures by running the reference's own code.

Run where a checkout of the reference sources exists:

    python tests/golden/make_golden.py --reference DIR
    (or RSORT_REFERENCE_DIR=DIR python tests/golden/make_golden.py)

It builds oracle/_ref/ref_probe (oracle/Makefile target ``ref``), which
compiles the reference's include/rsort/detail/tuning.cuh + utils.cuh on the
host and calls its radix_traits::twiddle_in/out, mix32 and set_seed_radix.
The probe's output is written verbatim to tests/golden/twiddle_ref.txt and
tests/golden/mix32_ref.txt; the CPU tests check the oracle (and the device
twiddle, through the GPU tests) against them.  Nothing here runs on the GPU
box: only the committed .txt files travel.
"""

from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "cuda-fast-sort_gb300"))

import numpy as np  # noqa: E402

from gbsort import gen  # noqa: E402

TYPES = ["u8", "u16", "u32", "u64", "u128", "i8", "i16", "i32", "i64", "i128", "f32", "f64", "f128"]
WIDTH = {"u8": 1, "u16": 2, "u32": 4, "u64": 8, "u128": 16, "i8": 1, "i16": 2, "i32": 4,
         "i64": 8, "i128": 16, "f32": 4, "f64": 8, "f128": 16}

FLOAT_EDGES = {
    4: [0x00000000, 0x80000000, 0x3F800000, 0xBF800000, 0x7F800000, 0xFF800000, 0x7FC00000,
        0xFFC00000, 0x7F800001, 0x00000001, 0x80000001, 0x007FFFFF, 0x7F7FFFFF, 0xFF7FFFFF],
    8: [0x0, 0x8000000000000000, 0x3FF0000000000000, 0xBFF0000000000000, 0x7FF0000000000000,
        0xFFF0000000000000, 0x7FF8000000000000, 0xFFF8000000000000, 0x1, 0x8000000000000001,
        0x7FEFFFFFFFFFFFFF],
    16: [0x0, 1 << 127, (0x3FFF << 112), (0xBFFF << 112), (0x7FFF << 112), (0xFFFF << 112),
         (0x7FFF8 << 108), 1, (1 << 127) | 1],
}


def edges(width: int) -> list[int]:
    top = 1 << (8 * width - 1)
    full = (1 << (8 * width)) - 1
    out = [0, 1, 2, 0x7F, 0x80, 0xFF, top - 1, top, top + 1, full - 1, full]
    return [v & full for v in out]


def random_values(width: int, count: int, seed: int) -> list[int]:
    s = gen.splitmix64(seed, 0, 2 * count)
    vals = []
    for k in range(count):
        v = int(s[2 * k]) | (int(s[2 * k + 1]) << 64)
        vals.append(v & ((1 << (8 * width)) - 1))
    return vals


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("RSORT_REFERENCE_DIR", ""),
                    help="checkout of the reference rsort (default: $RSORT_REFERENCE_DIR)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("name the reference checkout with --reference or RSORT_REFERENCE_DIR")
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref",
                    f"REFERENCE={args.reference}"], check=True)
    probe = os.path.join(REPO, "oracle", "_ref", "ref_probe")

    lines = []
    for ti, t in enumerate(TYPES):
        w = WIDTH[t]
        vals = edges(w) + random_values(w, 48, 1000 + ti)
        if t.startswith("f"):
            vals = FLOAT_EDGES[w] + vals
        for v in vals:
            lines.append(f"{t} {v:0{2 * w}x}")
    mix_in = [int(x) for x in gen.splitmix64(7, 0, 64) & np.uint64(0xFFFFFFFF)] + [0, 1, 12345, 0xFFFFFFFF]
    mix_lines = [f"mix32 {x:08x}" for x in mix_in] + [f"seed {i}" for i in range(40)]

    out = subprocess.run([probe], input="\n".join(lines + mix_lines) + "\n",
                         capture_output=True, text=True, check=True).stdout.splitlines()
    tw = [ln for ln in out if not ln.startswith(("mix32", "seed"))]
    mx = [ln for ln in out if ln.startswith(("mix32", "seed"))]
    header = ("# Generated by tests/golden/make_golden.py from the reference's own\n"
              "# radix_traits::twiddle_in/out (include/rsort/detail/tuning.cuh:352-384)\n"
              "# compiled and run on the host.  Columns: type raw in_asc in_desc "
              "out_asc(raw) out_desc(raw), hex of the key's raw bits.\n")
    with open(os.path.join(HERE, "twiddle_ref.txt"), "w") as f:
        f.write(header + "\n".join(tw) + "\n")
    with open(os.path.join(HERE, "mix32_ref.txt"), "w") as f:
        f.write("# Generated by tests/golden/make_golden.py from the reference's mix32\n"
                "# (utils.cuh:228-242) and set_seed_radix (utils.cuh:435-437).\n")
        f.write("\n".join(mx) + "\n")
    print(f"wrote {len(tw)} twiddle vectors and {len(mx)} mix32/seed vectors")


if __name__ == "__main__":
    main()
