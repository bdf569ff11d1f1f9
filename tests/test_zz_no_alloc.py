"""gbsort_sort_keys_noalloc: the keys-only sort for callers that may not
allocate device memory where they sort (allocation can block or synchronize
the device, and some hosts own all device memory).  Its workspace is a 16 MiB
static device array inside the library.

Checks, through the C ABI:
  - two calls in a row give exactly what the CPU oracle (std::stable_sort of
    the twiddled keys) gives, and what the ordinary entry point
    (gbsort_sort_keys with a caller workspace) gives on the same keys —
    integer/byte results, so bit-exact;
  - the largest n whose size query still fits the 16 MiB (found by bisection
    on the size query; its lookback status words end at the last bytes of
    the array) sorts correctly, for 4- and 16-byte keys, on a caller stream;
  - an n beyond the static capacity is refused without device work;
  - a device-side failure (bounded waits that run out under a 1 ns limit) is
    reported by gbsort_noalloc_status, and the next call sorts correctly.
Collected last on purpose; passes alone in a fresh process and after the
other tests.
"""

import ctypes

import numpy as np
import pytest

from _oracle import raw_keys
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu

CAPACITY = 16 << 20


def _noalloc(gb):
    f = gb.lib().gbsort_sort_keys_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    return f


def _noalloc_status(gb):
    f = gb.lib().gbsort_noalloc_status
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p]
    return f


def _with_workspace(gb, cuda, kt, raw, desc):
    n = raw.shape[0]
    d = to_dev(cuda, raw)
    tb = gb.temp_bytes(kt, n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    gb.sort(d, n, kt, ws, tb, descending=desc)
    cuda.cuda.synchronize()
    return from_dev(d, raw)


def _noalloc_sort(gb, cuda, kt, raw, desc, stream=None):
    n = raw.shape[0]
    d = to_dev(cuda, raw)
    cuda.cuda.synchronize()
    sp = None if stream is None else stream.cuda_stream
    st = _noalloc(gb)(gb.KEY_TYPES[kt], int(desc), d.data_ptr(), n, sp)
    assert st == gb.OK, gb.status_string(st) + " " + gb.last_error()
    st = _noalloc_status(gb)(gb.KEY_TYPES[kt], n, sp)
    assert st == gb.OK, gb.status_string(st)
    return from_dev(d, raw)


def _oracle_keys(oracle, kt, raw, desc):
    return np.ascontiguousarray(oracle.sort(kt, raw, desc))


@pytest.mark.parametrize("kt,n,desc", [("u32", 1 << 20, False), ("f32", 3_000_001, True),
                                       ("u64", 777_777, False), ("u128", 300_000, True), ("i8", 5_000_000, False)])
def test_noalloc_matches_oracle_two_calls(gb, cuda, oracle, kt, n, desc):
    assert gb.temp_bytes(kt, n) <= CAPACITY
    for call in range(2):  # the static scratch keeps the last call's contents
        raw = raw_keys(kt, n, seed=100 + call, dist=0 if call == 0 else 4)
        got = _noalloc_sort(gb, cuda, kt, raw, desc)
        assert np.array_equal(got.view(np.uint8), _oracle_keys(oracle, kt, raw, desc).view(np.uint8)), \
            f"{kt} call {call}: differs from the oracle"
        want = _with_workspace(gb, cuda, kt, raw, desc)
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"{kt} call {call}: differs from sort_keys"


def _largest_fitting_n(gb, kt):
    lo, hi = 1, 1 << 26  # temp_bytes(lo) fits, temp_bytes(hi) does not
    assert gb.temp_bytes(kt, lo) <= CAPACITY < gb.temp_bytes(kt, hi)
    while hi - lo > 1:
        mid = (lo + hi) // 2
        if gb.temp_bytes(kt, mid) <= CAPACITY:
            lo = mid
        else:
            hi = mid
    return lo


@pytest.mark.parametrize("kt,desc", [("u32", False), ("u128", True)])
def test_noalloc_largest_fitting_n_on_a_stream(gb, cuda, oracle, kt, desc):
    n = _largest_fitting_n(gb, kt)
    assert gb.temp_bytes(kt, n + 1) > CAPACITY
    stream = cuda.cuda.Stream()
    for call in range(2):
        raw = raw_keys(kt, n, seed=300 + call, dist=0 if call == 0 else 4)
        with cuda.cuda.stream(stream):
            got = _noalloc_sort(gb, cuda, kt, raw, desc, stream=stream)
        stream.synchronize()
        assert np.array_equal(got.view(np.uint8), _oracle_keys(oracle, kt, raw, desc).view(np.uint8)), \
            f"{kt} n={n} call {call}"


def test_noalloc_rejects_sizes_beyond_capacity(gb, cuda):
    n = 1 << 22  # u32: about 17 MiB of workspace
    assert gb.temp_bytes("u32", n) > CAPACITY
    raw = raw_keys("u32", 1000, seed=1)
    d = to_dev(cuda, raw)  # far smaller than n: the call must not touch it
    st = _noalloc(gb)(gb.KEY_TYPES["u32"], 0, d.data_ptr(), n, None)
    assert st == gb.ERR_WORKSPACE_TOO_SMALL
    assert "static scratch" in gb.last_error()
    assert _noalloc_status(gb)(gb.KEY_TYPES["u32"], n, None) == gb.ERR_WORKSPACE_TOO_SMALL
    cuda.cuda.synchronize()
    assert np.array_equal(from_dev(d, raw), raw)


def test_noalloc_status_reports_a_device_timeout(gb, cuda, oracle):
    kt, n = "u32", 1 << 21
    raw = raw_keys(kt, n, seed=7)
    f, status = _noalloc(gb), _noalloc_status(gb)
    old = gb.get_wait_limit_ns()
    seen = gb.OK
    try:
        gb.set_wait_limit_ns(1)  # every bounded device wait runs out at once
        for _ in range(3):
            d = to_dev(cuda, raw)
            cuda.cuda.synchronize()
            assert f(gb.KEY_TYPES[kt], 0, d.data_ptr(), n, None) == gb.OK  # the host call itself succeeds
            seen = status(gb.KEY_TYPES[kt], n, None)
            if seen != gb.OK:
                break
    finally:
        gb.set_wait_limit_ns(old)
    assert seen == gb.ERR_TIMEOUT, gb.status_string(seen)
    got = _noalloc_sort(gb, cuda, kt, raw, False)  # the next call clears the record and sorts
    assert np.array_equal(got, _oracle_keys(oracle, kt, raw, False))
