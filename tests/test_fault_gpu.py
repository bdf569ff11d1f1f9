"""Failure detection without a GPU fault: every device wait is bounded and
reports GBSORT_ERR_TIMEOUT through the host instead of hanging (the
reference spins without limit, include/rsort/detail/lookback.cuh:233-238).

The probe runs the sort's own bounded lookback wait on a status word that
nothing publishes, with a short limit, and checks that the status comes back
and the context stays usable.
"""

import time

import numpy as np
import pytest

from _oracle import raw_keys
from gpu_util import gpu_sort

pytestmark = pytest.mark.gpu


def test_wait_on_unpublished_word_times_out(gb, cuda, oracle):
    scratch = cuda.zeros(64, dtype=cuda.uint8, device="cuda")
    t0 = time.time()
    st = gb.probe_wait_timeout(scratch, 2_000_000)  # 2 ms limit
    assert st == gb.ERR_TIMEOUT
    assert time.time() - t0 < 5.0
    # the context is still healthy: a sort right after is exact
    raw = raw_keys("u32", 100000, seed=1)
    assert np.array_equal(gpu_sort(gb, cuda, "u32", raw), oracle.sort("u32", raw))


def test_normal_sort_reports_ok(gb, cuda):
    n = 1 << 16
    d = cuda.empty(n, dtype=cuda.int32, device="cuda")
    gb.generate(0, 4, d, n, 5)
    tb = gb.temp_bytes("u32", n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    gb.sort(d, n, "u32", ws, tb)
    assert gb.workspace_status("u32", n, ws) == gb.OK


def test_wait_limit_is_process_setting(gb):
    old = gb.get_wait_limit_ns()
    try:
        gb.set_wait_limit_ns(123456)
        assert gb.get_wait_limit_ns() == 123456
    finally:
        gb.set_wait_limit_ns(old)
