"""One-launch sort of short keys-only arrays (fused_short.cuh): the digit
counts, every pass and the fix-up in one cooperative launch with a bounded
grid barrier between them.

Every other GPU test of keys-only arrays up to 2^21 keys already runs through
this path (it is the default).  Here:
  - the plan reports one launch up to 2^21 keys and the multi-launch path
    above, and both sides of the switch equal the oracle;
  - the one-launch and multi-launch paths give identical bytes for every key
    type, both orders, and for inputs whose uniform digits skip passes;
  - the grid barrier's bounded wait runs out on a barrier nothing completes
    (GBSORT_ERR_TIMEOUT) and the context stays usable;
  - a one-launch sort whose waits all run out (1 ns limit) reports
    GBSORT_ERR_TIMEOUT, and the next sort is correct;
  - the MSD partition + bucket sorts give the same bytes as every digit
    taking a pass, and a top-digit bucket too big for one CTA falls back to
    the passes (both against the oracle);
  - the bucket split (a counting pass on the bits below the top digit, then
    a comparison rank inside sub-buckets) beside buckets whose sub-buckets
    are too big for it (bits below the top digit that coincide, keys
    repeated a few or many times), against the oracle.
"""

import numpy as np
import pytest

from _oracle import KEY_BYTES, KEY_TYPES, raw_keys
from gpu_util import gpu_sort, from_dev, to_dev

pytestmark = pytest.mark.gpu

FUSED_MAX = 1 << 21


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.fixture
def fused_default(gb):
    old = gb.get_short_fused()
    gb.set_short_fused(True)
    yield
    gb.set_short_fused(old)


@pytest.mark.parametrize("n", [1, 100, 4095, 4096, 4097, 1 << 20, FUSED_MAX - 1, FUSED_MAX, FUSED_MAX + 1])
def test_plan_switch_and_oracle(gb, cuda, oracle, fused_default, n):
    info = gb.plan("u32", n)
    if n <= FUSED_MAX:
        assert info.kernel_launches == 1 and info.hist_ctas == 0
    else:
        assert info.kernel_launches > 1
    raw = raw_keys("u32", n, seed=n % 1000 + 3)
    assert _eq(gpu_sort(gb, cuda, "u32", raw), oracle.sort("u32", raw, False))


def test_plan_reports_the_msd_regions(gb, fused_default, msd_default):
    gb.set_short_msd(True)
    info = gb.plan("u32", 1 << 20)
    assert 4096 < info.msd_region_keys <= 8192  # the mean bucket plus a margin, within a CTA's local sort
    assert gb.plan("u8", 1 << 20).msd_region_keys == 0  # one digit: nothing below it
    assert gb.plan("u32", FUSED_MAX).msd_region_keys == 0  # buckets of ~8192 keys outgrow the local sort
    gb.set_short_msd(False)
    assert gb.plan("u32", 1 << 20).msd_region_keys == 0


def test_values_and_long_arrays_keep_the_multi_launch_path(gb, fused_default):
    assert gb.plan("u32", 1 << 20, 4).kernel_launches > 1
    assert gb.plan("u64", FUSED_MAX + 1).kernel_launches > 1


def _both_paths(gb, cuda, kt, raw, desc):
    gb.set_short_fused(True)
    one = gpu_sort(gb, cuda, kt, raw, desc)
    gb.set_short_fused(False)
    try:
        multi = gpu_sort(gb, cuda, kt, raw, desc)
    finally:
        gb.set_short_fused(True)
    return one, multi


@pytest.mark.parametrize("kt", KEY_TYPES)
@pytest.mark.parametrize("desc", [False, True])
def test_one_launch_equals_multi_launch(gb, cuda, oracle, fused_default, kt, desc):
    raw = raw_keys(kt, 300_007, seed=11 + len(kt))
    one, multi = _both_paths(gb, cuda, kt, raw, desc)
    assert _eq(one, multi)
    assert _eq(one, oracle.sort(kt, raw, desc))


@pytest.mark.parametrize("kt,dist", [("u32", 5), ("u64", 5), ("u16", 3), ("u128", 3)])
def test_one_launch_with_skipped_passes(gb, cuda, oracle, fused_default, kt, dist):
    raw = raw_keys(kt, 123_457, seed=5, dist=dist)  # constant bytes: their passes are skipped
    one, multi = _both_paths(gb, cuda, kt, raw, False)
    assert _eq(one, multi)
    assert _eq(one, oracle.sort(kt, raw, False))


def test_grid_barrier_wait_runs_out(gb, cuda):
    scratch = cuda.empty(64, dtype=cuda.uint8, device="cuda")
    assert gb.probe_barrier_timeout(scratch, 2_000_000) == gb.ERR_TIMEOUT  # 2 ms
    cuda.cuda.synchronize()
    x = cuda.arange(10, device="cuda")
    assert int(x.sum().item()) == 45  # the context is still usable


def test_one_launch_reports_timed_out_waits(gb, cuda, oracle, fused_default):
    n = 1 << 20
    assert gb.plan("u32", n).kernel_launches == 1
    raw = raw_keys("u32", n, seed=77)
    tb = gb.temp_bytes("u32", n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    old = gb.get_wait_limit_ns()
    seen = gb.OK
    try:
        gb.set_wait_limit_ns(1)
        for _ in range(3):
            d = to_dev(cuda, raw)
            gb.sort(d, n, "u32", ws, tb)
            seen = gb.workspace_status("u32", n, ws)
            if seen != gb.OK:
                break
    finally:
        gb.set_wait_limit_ns(old)
    assert seen == gb.ERR_TIMEOUT, gb.status_string(seen)
    d = to_dev(cuda, raw)
    gb.sort(d, n, "u32", ws, tb)
    cuda.cuda.synchronize()
    assert gb.workspace_status("u32", n, ws) == gb.OK
    assert _eq(from_dev(d, raw), oracle.sort("u32", raw, False))


@pytest.fixture
def msd_default(gb):
    old = gb.get_short_msd()
    yield
    gb.set_short_msd(old)


@pytest.mark.parametrize("kt", ["u16", "i32", "f32", "u64", "f64", "u128", "f128"])
@pytest.mark.parametrize("desc", [False, True])
def test_msd_buckets_equal_digit_passes(gb, cuda, oracle, fused_default, msd_default, kt, desc):
    raw = raw_keys(kt, 200_003, seed=21 + len(kt))  # buckets of ~800 keys: the partition applies
    gb.set_short_msd(True)
    part = gpu_sort(gb, cuda, kt, raw, desc)
    gb.set_short_msd(False)
    passes = gpu_sort(gb, cuda, kt, raw, desc)
    assert _eq(part, passes)
    assert _eq(part, oracle.sort(kt, raw, desc))


@pytest.mark.parametrize("n", [1 << 20, (1 << 21) - 3])
def test_msd_big_bucket_falls_back(gb, cuda, oracle, fused_default, msd_default, n):
    raw = raw_keys("u32", n, seed=9)
    raw[::5] = (raw[::5] & np.uint32(0x00FFFFFF)) | np.uint32(0x55000000)  # one bucket of n/5 keys
    gb.set_short_msd(True)
    got = gpu_sort(gb, cuda, "u32", raw)
    assert _eq(got, oracle.sort("u32", raw, False))
    gb.set_short_msd(False)
    assert _eq(gpu_sort(gb, cuda, "u32", raw), got)


def _coincide_below_top(kt, raw):
    """The keys whose top bit is set get one value for every bit between the
    top byte and the lowest byte: their buckets have a single sub-bucket."""
    out = raw.copy()
    kb = KEY_BYTES[kt]
    if kb == 16:
        h = out.view(np.uint64).reshape(-1, 2)  # little-endian: column 1 holds the top byte
        m = (h[:, 1] >> np.uint64(63)) == 1
        h[m, 1] = (h[m, 1] & np.uint64(0xFF00000000000000)) | np.uint64(0x00ABCDEF12345678)
        h[m, 0] &= np.uint64(0xFF)
        return out
    keep, const = {4: (0xFF0000FF, 0x00ABCD00), 8: (0xFF000000000000FF, 0x00ABCDEF12345600)}[kb]
    t = out.dtype.type
    m = (out >> t(8 * kb - 1)) == 1
    out[m] = (out[m] & t(keep)) | t(const)
    return out


def _repeated(raw, distinct, seed):
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(raw[:distinct][rng.integers(0, distinct, raw.shape[0])])


@pytest.mark.parametrize("kt", ["u32", "f32", "u64", "i64", "u128"])
@pytest.mark.parametrize("shape", ["coincide", "repeat8", "repeat3000"])
@pytest.mark.parametrize("desc", [False, True])
def test_bucket_split_and_its_fallback(gb, cuda, oracle, fused_default, msd_default, kt, shape, desc):
    n = 1 << 19 if kt == "u128" else 1 << 20
    raw = raw_keys(kt, n, seed=41 + len(kt))
    if shape == "coincide":
        raw = _coincide_below_top(kt, raw)
    else:  # about 8 copies of each key: sub-buckets with ties; 3000 keys: too big
        raw = _repeated(raw, n // 8 if shape == "repeat8" else 3000, seed=n)
    gb.set_short_msd(True)
    got = gpu_sort(gb, cuda, kt, raw, desc)
    assert _eq(got, oracle.sort(kt, raw, desc))
    gb.set_short_msd(False)
    assert _eq(gpu_sort(gb, cuda, kt, raw, desc), got)
