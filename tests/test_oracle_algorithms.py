"""The oracle's two forms agree, and agree with an independent Python sort.

- ``oracle_sort``: std::stable_sort on twiddled keys (the checker);
- ``oracle_lsd_sort``: a literal restatement of the reference's pass loop
  (include/rsort/detail/radix_kernel.cuh:412-465: one stable 8-bit counting
  pass per byte, least significant first, ping-pong);
- a pure-Python ``sorted`` by twiddled value (small n).
Also covers the reference's own property checks (utils.cuh:341-432: order,
pairing, stability; benchmark_sort.cuh:26-59: digit-histogram equality) as
they apply to the oracle's output.
"""

import numpy as np
import pytest

from _oracle import KEY_BYTES, KEY_TYPES, raw_keys, raw_values


def _as_ints(raw, w):
    if w == 16:
        q = raw.reshape(-1, 16).view(np.uint64).reshape(-1, 2)
        return [int(lo) | (int(hi) << 64) for lo, hi in q]
    return [int(x) for x in raw]


@pytest.mark.parametrize("kt", KEY_TYPES)
@pytest.mark.parametrize("desc", [False, True])
def test_stable_sort_equals_lsd_restatement(oracle, kt, desc):
    for n, dist in ((0, 0), (1, 0), (7, 0), (1000, 0), (3001, 4), (2048, 5)):
        raw = raw_keys(kt, n, seed=11 + n, dist=dist)
        for vb in (0, 4, 8, 16, 2):
            vals = raw_values(vb, n, seed=5)
            a = oracle.sort(kt, raw, desc, vals)
            b = oracle.sort(kt, raw, desc, vals, lsd=True)
            if vals is None:
                assert np.array_equal(a, b)
            else:
                assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


@pytest.mark.parametrize("kt", KEY_TYPES)
def test_stable_sort_equals_python_sorted(oracle, kt):
    w = KEY_BYTES[kt]
    n = 600
    raw = raw_keys(kt, n, seed=3)
    # add duplicates to exercise stability
    raw[n // 2:] = raw[: n - n // 2]
    for desc in (False, True):
        bits = _as_ints(oracle.twiddle_in(kt, raw, desc), w)
        order = sorted(range(n), key=lambda i: bits[i])  # Python sort is stable
        keys, idx = oracle.sort(kt, raw, desc, np.arange(n, dtype=np.uint64))
        assert [int(i) for i in idx] == order
        assert _as_ints(keys, w) == [_as_ints(raw, w)[i] for i in order]


@pytest.mark.parametrize("kt", ["u32", "f32", "u64", "i16", "f128"])
def test_reference_property_checks_hold(oracle, kt):
    """Order, key/value pairing, stability and per-pass digit-histogram
    equality, the reference's three post-sort checks."""
    n = 5000
    raw = raw_keys(kt, n, seed=21, dist=4)
    raw[::3] = raw[0]  # many equal keys
    vals = np.arange(n, dtype=np.uint64)
    keys, idx = oracle.sort(kt, raw, False, vals)
    w = KEY_BYTES[kt]
    tb = _as_ints(oracle.twiddle_in(kt, keys, False), w)
    assert all(tb[i] <= tb[i + 1] for i in range(n - 1))
    orig = _as_ints(raw, w)
    sk = _as_ints(keys, w)
    assert all(sk[i] == orig[int(idx[i])] for i in range(n))
    assert all(not (tb[i] == tb[i + 1] and idx[i] > idx[i + 1]) for i in range(n - 1))
    assert np.array_equal(oracle.histogram(kt, raw), oracle.histogram(kt, keys))


def test_histogram_matches_numpy(oracle):
    raw = raw_keys("u32", 10000, seed=9)
    h = oracle.histogram("u32", raw)
    for p in range(4):
        ref = np.bincount((raw >> np.uint32(8 * p)) & np.uint32(0xFF), minlength=256)
        assert np.array_equal(h[p], ref.astype(np.uint64))


def test_parallel_oracle_equals_serial(oracle):
    raw = raw_keys("f32", 200000, seed=4, dist=1)
    vals = np.arange(raw.size, dtype=np.uint32)
    a = oracle.sort("f32", raw, False, vals)
    b = oracle.sort("f32", raw, False, vals, threads=max(2, oracle.max_threads()))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
