"""gbsort_sort_keys_noalloc: the keys-only sort for callers that may not
allocate device memory where they sort (allocation can block or synchronize
the device, and some hosts own all device memory).  Its workspace is a 16 MiB
static device array inside the library.

Checks, through the C ABI: two calls in a row give exactly what the ordinary
entry point (gbsort_sort_keys with a caller workspace) gives on the same
keys — integer/byte results, so bit-exact — and an n beyond the static
capacity is refused without device work.  Collected last on purpose; passes
alone in a fresh process and after the other tests.
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


def _with_workspace(gb, cuda, kt, raw, desc):
    n = raw.shape[0]
    d = to_dev(cuda, raw)
    tb = gb.temp_bytes(kt, n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    gb.sort(d, n, kt, ws, tb, descending=desc)
    cuda.cuda.synchronize()
    return from_dev(d, raw)


def _noalloc_sort(gb, cuda, kt, raw, desc):
    n = raw.shape[0]
    d = to_dev(cuda, raw)
    st = _noalloc(gb)(gb.KEY_TYPES[kt], int(desc), d.data_ptr(), n, None)
    assert st == gb.OK, gb.status_string(st) + " " + gb.last_error()
    cuda.cuda.synchronize()
    return from_dev(d, raw)


@pytest.mark.parametrize("kt,n,desc", [("u32", 1 << 20, False), ("f32", 3_000_001, True),
                                       ("u64", 777_777, False), ("u128", 300_000, True), ("i8", 5_000_000, False)])
def test_noalloc_matches_workspace_entry_two_calls(gb, cuda, kt, n, desc):
    assert gb.temp_bytes(kt, n) <= CAPACITY
    for call in range(2):  # the static scratch keeps the last call's contents
        raw = raw_keys(kt, n, seed=100 + call, dist=0 if call == 0 else 4)
        want = _with_workspace(gb, cuda, kt, raw, desc)
        got = _noalloc_sort(gb, cuda, kt, raw, desc)
        assert np.array_equal(got.view(np.uint8), want.view(np.uint8)), f"{kt} call {call}"


def test_noalloc_rejects_sizes_beyond_capacity(gb, cuda):
    n = 1 << 22  # u32: about 17 MiB of workspace
    assert gb.temp_bytes("u32", n) > CAPACITY
    raw = raw_keys("u32", 1000, seed=1)
    d = to_dev(cuda, raw)  # far smaller than n: the call must not touch it
    st = _noalloc(gb)(gb.KEY_TYPES["u32"], 0, d.data_ptr(), n, None)
    assert st == gb.ERR_WORKSPACE_TOO_SMALL
    assert "static scratch" in gb.last_error()
    cuda.cuda.synchronize()
    assert np.array_equal(from_dev(d, raw), raw)
