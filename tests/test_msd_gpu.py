"""Keys-only sorts of 8- and 16-byte keys above the short range, most
significant digit first (msd.cuh): top split, pair count, scan, second
split, in-place local sorts of the (top, second) digit groups.

  - the plan reports the path for keys-only 8- and 16-byte keys in its size
    range and not for pairs, narrower keys or sizes outside;
  - every 8- and 16-byte key type, both orders: equal to the oracle and to
    the digit passes (the path switched off);
  - the input-preserving and DoubleBuffer forms, and the sort of a
    host-memory array (copy, sort, copy back);
  - inputs whose groups outgrow a local sort (keys sharing their top 16
    bits, a few distinct top-16-bit prefixes) fall back to the digit passes
    on the device, and so does a group whose local sort gives up (a
    sub-bucket too big for the comparison rank), from the keys as the local
    sorts left them; repeated keys;
  - the timed sort reports the six kernels between the histogram and the
    digit passes.
"""

import numpy as np
import pytest

from _oracle import KEY_BYTES, raw_keys
from gpu_util import from_dev, gpu_sort, to_dev

pytestmark = pytest.mark.gpu

N8 = (3 << 23) + 77   # 8-byte keys: groups of ~384 keys
N16 = (1 << 22) + 33  # 16-byte keys: groups of ~64 keys


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.fixture
def msd_on(gb):
    old = gb.get_msd()
    gb.set_msd(True)
    yield
    gb.set_msd(old)


def _both(gb, cuda, kt, raw, desc):
    gb.set_msd(True)
    on = gpu_sort(gb, cuda, kt, raw, desc)
    gb.set_msd(False)
    try:
        off = gpu_sort(gb, cuda, kt, raw, desc)
    finally:
        gb.set_msd(True)
    return on, off


def test_plan_reports_the_path(gb, msd_on):
    assert gb.plan("u64", N8).msd_stages == 6
    assert gb.plan("f128", N16).msd_stages == 6
    assert gb.plan("u64", 1 << 28).msd_stages == 6
    assert gb.plan("u128", 1 << 27).msd_stages == 6
    assert gb.plan("u64", N8, 8).msd_stages == 0      # pairs keep the stable passes
    assert gb.plan("u32", 1 << 24).msd_stages == 0    # 4-byte keys: digit passes
    assert gb.plan("u64", 1 << 24).msd_stages == 0    # below the range
    assert gb.plan("u128", 1 << 20).msd_stages == 0   # the one-launch sort's
    assert gb.plan("u128", 3 << 19).msd_stages == 6
    assert gb.plan("u128", (1 << 27) + 1).msd_stages == 0  # above it
    tb = gb.temp_bytes("u64", N8)
    gb.set_msd(False)
    assert gb.plan("u64", N8).msd_stages == 0
    assert gb.temp_bytes("u64", N8) == tb  # the size query does not depend on the switch


@pytest.mark.parametrize("kt", ["u64", "i64", "f64", "u128", "i128", "f128"])
@pytest.mark.parametrize("desc", [False, True])
def test_equals_oracle_and_digit_passes(gb, cuda, oracle, msd_on, kt, desc):
    n = N16 if KEY_BYTES[kt] == 16 else N8
    raw = raw_keys(kt, n, seed=5 + len(kt) + int(desc))
    on, off = _both(gb, cuda, kt, raw, desc)
    assert _eq(on, oracle.sort(kt, raw, desc))
    assert _eq(on, off)


@pytest.mark.parametrize("kt", ["u64", "f128"])
def test_input_preserving_and_double_buffer(gb, cuda, oracle, msd_on, kt):
    n = N16 if KEY_BYTES[kt] == 16 else N8
    raw = raw_keys(kt, n, seed=91)
    want = oracle.sort(kt, raw, True)
    src = to_dev(cuda, raw)
    out = cuda.zeros_like(src)
    tb = gb.temp_bytes(kt, n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    gb.sort_copy(src, out, n, kt, ws, tb, descending=True)
    cuda.cuda.synchronize()
    assert gb.workspace_status(kt, n, ws) == gb.OK
    assert _eq(from_dev(out, raw), want)
    assert _eq(from_dev(src, raw), raw)  # the input is untouched
    k0, k1 = to_dev(cuda, raw), cuda.zeros_like(src)
    dbb = gb.double_buffer_bytes(kt, n)
    dws = cuda.empty(dbb, dtype=cuda.uint8, device="cuda")
    sel = gb.sort_double_buffer(k0, k1, n, kt, dws, dbb, descending=True)
    cuda.cuda.synchronize()
    assert gb.double_buffer_status(kt, n, dws) == gb.OK
    assert _eq(from_dev(k1 if sel else k0, raw), want)


def _top16_prefixes(kt, raw, prefixes, seed):
    """The keys' top 16 bits replaced by one of `prefixes` (so their groups
    outgrow a local sort)."""
    out = raw.copy()
    rng = np.random.default_rng(seed)
    pick = np.asarray(prefixes, dtype=np.uint64)[rng.integers(0, len(prefixes), raw.shape[0])]
    if KEY_BYTES[kt] == 16:
        h = out.view(np.uint64).reshape(-1, 2)  # little-endian: column 1 holds the top bytes
        h[:, 1] = (h[:, 1] & np.uint64(0x0000FFFFFFFFFFFF)) | (pick << np.uint64(48))
    else:
        out[:] = (out & np.uint64(0x0000FFFFFFFFFFFF)) | (pick << np.uint64(48))
    return out


@pytest.mark.parametrize("kt", ["u64", "u128"])
@pytest.mark.parametrize("prefixes", [[0x1234], [0x0001, 0x8000, 0xFFFE]])
def test_big_groups_fall_back_to_the_digit_passes(gb, cuda, oracle, msd_on, kt, prefixes):
    n = N16 if KEY_BYTES[kt] == 16 else N8
    raw = _top16_prefixes(kt, raw_keys(kt, n, seed=17), prefixes, seed=3)
    on, off = _both(gb, cuda, kt, raw, False)
    assert _eq(on, oracle.sort(kt, raw, False))
    assert _eq(on, off)


def _crowd_one_sub_bucket(kt, raw, count, seed):
    """`count` keys get the same top 28 bits: their group still fits a local
    sort, but one of its sub-buckets holds far more keys than the comparison
    rank takes, so that group's local sort gives up and the digit passes sort
    the whole array from what the local sorts left."""
    out = raw.copy()
    rng = np.random.default_rng(seed)
    idx = rng.choice(raw.shape[0], count, replace=False)
    top = np.uint64(0xABCDEF1) << np.uint64(36)
    low = np.uint64((1 << 36) - 1)
    if KEY_BYTES[kt] == 16:
        h = out.view(np.uint64).reshape(-1, 2)  # little-endian: column 1 holds the top bytes
        h[idx, 1] = (h[idx, 1] & low) | top
    else:
        out[idx] = (out[idx] & low) | top
    return out


@pytest.mark.parametrize("kt", ["f128", "i64", "u128", "f64"])
def test_a_local_sort_that_gives_up(gb, cuda, oracle, msd_on, kt):
    n = N16 if KEY_BYTES[kt] == 16 else N8
    raw = _crowd_one_sub_bucket(kt, raw_keys(kt, n, seed=61), 200, seed=62)
    on, off = _both(gb, cuda, kt, raw, True)
    assert _eq(on, oracle.sort(kt, raw, True))
    assert _eq(on, off)
    # the input-preserving form sorts from its untouched input
    src = to_dev(cuda, raw)
    out = cuda.zeros_like(src)
    tb = gb.temp_bytes(kt, n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    gb.sort_copy(src, out, n, kt, ws, tb, descending=True)
    cuda.cuda.synchronize()
    assert _eq(from_dev(out, raw), on)


@pytest.mark.parametrize("kt,distinct", [("u64", 1 << 20), ("u64", 1 << 13), ("u128", 1 << 19)])
def test_repeated_keys(gb, cuda, oracle, msd_on, kt, distinct):
    n = N16 if KEY_BYTES[kt] == 16 else N8
    raw = raw_keys(kt, n, seed=23)
    rng = np.random.default_rng(distinct)
    raw = np.ascontiguousarray(raw[:distinct][rng.integers(0, distinct, n)])
    on, off = _both(gb, cuda, kt, raw, True)
    assert _eq(on, oracle.sort(kt, raw, True))
    assert _eq(on, off)


def test_timed_entries(gb, cuda, msd_on):
    kt, n = "u128", N16
    raw = raw_keys(kt, n, seed=2)
    d = to_dev(cuda, raw)
    tb = gb.temp_bytes(kt, n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    ms = gb.sort_timed(d, n, kt, ws, tb)
    info = gb.plan(kt, n)
    assert info.msd_stages == 6
    # histogram, 5 MSD kernels, the other digits' histogram, 16 passes (these two exit at once), fix-up
    assert len(ms) == info.kernel_launches
    assert all(t >= 0 for t in ms)


@pytest.mark.parametrize("kt", ["u128", "i64"])
def test_host_memory_sort(gb, cuda, oracle, msd_on, kt):
    """gbsort_sort_host of a keys-only array in the MSD range: copy, sort
    most significant digit first, copy back (instead of the split path)."""
    n = N16 if KEY_BYTES[kt] == 16 else N8
    raw = raw_keys(kt, n, seed=71)
    hk = cuda.from_numpy(np.ascontiguousarray(raw).view(np.uint8).reshape(-1).copy()).pin_memory()
    hb = gb.host_buffer_bytes(kt, n)
    dbuf = cuda.empty(hb, dtype=cuda.uint8, device="cuda")
    gb.sort_host(hk.data_ptr(), n, kt, dbuf, hb, descending=True)
    assert _eq(hk.numpy().view(raw.dtype).reshape(raw.shape), oracle.sort(kt, raw, True))


@pytest.mark.parametrize("kt", ["u128", "f128"])
def test_lower_end_of_the_range(gb, cuda, oracle, msd_on, kt):
    """16-byte keys just above the one-launch sort's range: the MSD path,
    with the short tile shape for its fallback passes; equal to the oracle
    and to those passes, also when a group is too big."""
    n = (3 << 19) + 7
    assert gb.plan(kt, n).msd_stages == 6
    raw = raw_keys(kt, n, seed=81)
    on, off = _both(gb, cuda, kt, raw, True)
    assert _eq(on, oracle.sort(kt, raw, True))
    assert _eq(on, off)
    raw = _top16_prefixes(kt, raw, [0x4321], seed=4)
    on, off = _both(gb, cuda, kt, raw, False)
    assert _eq(on, oracle.sort(kt, raw, False))
    assert _eq(on, off)
