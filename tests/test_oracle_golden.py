"""Pins the oracle against vectors the reference's own code produced.

tests/golden/twiddle_ref.txt and mix32_ref.txt were printed by
oracle/ref_probe.cpp, which compiles the reference's
include/rsort/detail/tuning.cuh (radix_traits::twiddle_in/out, :352-384) and
utils.cuh (mix32, :228-242; set_seed_radix, :435-437) on the host
(tests/golden/make_golden.py).  The oracle's restated twiddle and the numpy
generators must reproduce them bit for bit.
"""

import os

import numpy as np
import pytest

from _oracle import KEY_BYTES, RAW_DTYPE

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load_twiddle():
    rows = {}
    with open(os.path.join(GOLDEN, "twiddle_ref.txt")) as f:
        for ln in f:
            if ln.startswith("#") or not ln.strip():
                continue
            t, raw, ia, idd, oa, od = ln.split()
            rows.setdefault(t, []).append(tuple(int(x, 16) for x in (raw, ia, idd, oa, od)))
    return rows


def _to_raw(vals, width):
    if width == 16:
        a = np.zeros((len(vals), 2), dtype=np.uint64)
        for i, v in enumerate(vals):
            a[i, 0] = v & ((1 << 64) - 1)
            a[i, 1] = v >> 64
        return a.view(np.uint8).reshape(len(vals), 16)
    return np.array(vals, dtype=RAW_DTYPE[width])


def _from_raw(a, width):
    if width == 16:
        w = a.reshape(-1, 16).view(np.uint64).reshape(-1, 2)
        return [int(lo) | (int(hi) << 64) for lo, hi in w]
    return [int(x) for x in a]


TWIDDLE = _load_twiddle()


def test_golden_covers_every_key_type():
    assert sorted(TWIDDLE) == sorted(KEY_BYTES)
    assert sum(len(v) for v in TWIDDLE.values()) >= 13 * 50


@pytest.mark.parametrize("kt", sorted(KEY_BYTES))
def test_oracle_twiddle_matches_reference(oracle, kt):
    rows = TWIDDLE[kt]
    w = KEY_BYTES[kt]
    raw = _to_raw([r[0] for r in rows], w)
    assert _from_raw(oracle.twiddle_in(kt, raw, False), w) == [r[1] for r in rows]
    assert _from_raw(oracle.twiddle_in(kt, raw, True), w) == [r[2] for r in rows]
    assert _from_raw(oracle.twiddle_out(kt, raw, False), w) == [r[3] for r in rows]
    assert _from_raw(oracle.twiddle_out(kt, raw, True), w) == [r[4] for r in rows]


@pytest.mark.parametrize("kt", sorted(KEY_BYTES))
def test_twiddle_round_trip_and_order(oracle, kt):
    """twiddle_out(twiddle_in(x)) == x and the twiddled order is the key order
    rsort defines (-NaN < -inf < ... < -0.0 < +0.0 < ... < +inf < +NaN)."""
    rows = TWIDDLE[kt]
    w = KEY_BYTES[kt]
    raw = _to_raw([r[0] for r in rows], w)
    for desc in (False, True):
        back = oracle.twiddle_out(kt, oracle.twiddle_in(kt, raw, desc), desc)
        assert _from_raw(back, w) == [r[0] for r in rows]
    if kt == "f32":
        order = [0xFFC00000, 0xFF800000, 0xBF800000, 0x80000001, 0x80000000, 0x00000000, 0x00000001,
                 0x3F800000, 0x7F800000, 0x7FC00000]
        t = _from_raw(oracle.twiddle_in(kt, np.array(order, dtype=np.uint32), False), 4)
        assert t == sorted(t)
        td = _from_raw(oracle.twiddle_in(kt, np.array(order, dtype=np.uint32), True), 4)
        assert td == sorted(td, reverse=True)


def test_mix32_and_seed_match_reference():
    from gbsort import gen

    with open(os.path.join(GOLDEN, "mix32_ref.txt")) as f:
        lines = [ln.split() for ln in f if ln.strip() and not ln.startswith("#")]
    mix = [(int(a, 16), int(b, 16)) for t, a, b in lines if t == "mix32"]
    seeds = [(int(a), int(b)) for t, a, b in lines if t == "seed"]
    assert len(mix) >= 64 and len(seeds) >= 40
    got = gen.mix32(np.array([m[0] for m in mix], dtype=np.uint32))
    assert [int(x) for x in got] == [m[1] for m in mix]
    # set_seed_radix(i) = (i + 81) * 17, the reference's validation seeding.
    assert all(b == (a + 81) * 17 for a, b in seeds)
