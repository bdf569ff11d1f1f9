"""Sorting host buffers (gbsort_sort_host): pinned and pageable keys and
values go through a caller-provided device buffer and come back sorted,
bit-identical to the oracle."""

import numpy as np
import pytest

from _oracle import raw_keys, raw_values

pytestmark = pytest.mark.gpu


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("kt,vb,desc", [("u32", 0, False), ("f32", 4, True), ("i64", 8, False), ("u128", 16, True)])
def test_sort_host_matches_oracle(gb, cuda, oracle, kt, vb, desc, pinned):
    n = 123457
    raw = raw_keys(kt, n, seed=7, dist=4)
    vals = raw_values(vb, n, seed=8)
    kflat = np.ascontiguousarray(raw).view(np.uint8).reshape(-1).copy()
    vflat = None if vals is None else np.ascontiguousarray(vals).view(np.uint8).reshape(-1).copy()
    if pinned:
        hk = cuda.from_numpy(kflat).pin_memory()
        hv = None if vflat is None else cuda.from_numpy(vflat).pin_memory()
        kp, vp = hk.data_ptr(), (None if hv is None else hv.data_ptr())
        read_k = lambda: hk.numpy()  # noqa: E731
        read_v = lambda: hv.numpy()  # noqa: E731
    else:
        kp, vp = kflat.ctypes.data, (None if vflat is None else vflat.ctypes.data)
        read_k = lambda: kflat  # noqa: E731
        read_v = lambda: vflat  # noqa: E731
    hb = gb.host_buffer_bytes(kt, n, vb)
    dbuf = cuda.empty(hb, dtype=cuda.uint8, device="cuda")
    gb.sort_host(kp, n, kt, dbuf, hb, h_values=vp, value_bytes=vb, descending=desc)
    k = read_k().view(raw.dtype).reshape(raw.shape)
    if vals is None:
        assert _eq(k, oracle.sort(kt, raw, desc))
    else:
        ek, ev = oracle.sort(kt, raw, desc, vals)
        assert _eq(k, ek) and _eq(read_v().view(vals.dtype).reshape(vals.shape), ev)
    with pytest.raises(gb.GbsortError):  # a buffer one byte short is refused
        gb.sort_host(kp, n, kt, dbuf, hb - 1, h_values=vp, value_bytes=vb)


def test_graph_cache_switch(gb):
    assert gb.get_graph_cache()
    gb.set_graph_cache(False)
    try:
        assert not gb.get_graph_cache()
    finally:
        gb.set_graph_cache(True)
    assert gb.get_graph_cache()


# ---- the split path: partition by the top digit, groups copied back while
# later groups sort.  GBSORT_HOST_SPLIT_MIN (read on every call) brings it
# down to sizes the oracle checks in a moment.

@pytest.fixture
def split_env(monkeypatch):
    def setup(min_keys=1000, groups=8):
        monkeypatch.setenv("GBSORT_HOST_SPLIT_MIN", str(min_keys))
        monkeypatch.setenv("GBSORT_HOST_SPLIT_GROUPS", str(groups))
    return setup


def _host_sort_check(gb, cuda, oracle, kt, raw, vals, desc, pinned=True):
    n = raw.shape[0]
    vb = 0 if vals is None else vals.dtype.itemsize * (vals.shape[1] if vals.ndim == 2 else 1)
    kflat = np.ascontiguousarray(raw).view(np.uint8).reshape(-1).copy()
    vflat = None if vals is None else np.ascontiguousarray(vals).view(np.uint8).reshape(-1).copy()
    if pinned:
        hk = cuda.from_numpy(kflat).pin_memory()
        hv = None if vflat is None else cuda.from_numpy(vflat).pin_memory()
        kp, vp = hk.data_ptr(), (None if hv is None else hv.data_ptr())
        read_k, read_v = (lambda: hk.numpy()), (lambda: hv.numpy())
    else:
        kp, vp = kflat.ctypes.data, (None if vflat is None else vflat.ctypes.data)
        read_k, read_v = (lambda: kflat), (lambda: vflat)
    hb = gb.host_buffer_bytes(kt, n, vb)
    dbuf = cuda.empty(hb, dtype=cuda.uint8, device="cuda")
    gb.sort_host(kp, n, kt, dbuf, hb, h_values=vp, value_bytes=vb, descending=desc)
    k = read_k().view(raw.dtype).reshape(raw.shape)
    if vals is None:
        assert _eq(k, oracle.sort(kt, raw, desc))
    else:
        ek, ev = oracle.sort(kt, raw, desc, vals)
        assert _eq(k, ek)
        assert _eq(read_v().view(vals.dtype).reshape(vals.shape), ev)


@pytest.mark.parametrize("groups", [1, 3, 8, 256])
@pytest.mark.parametrize("kt,dist,vb,desc", [("u32", 4, 0, False), ("u32", 4, 4, True), ("f32", 1, 4, True),
                                             ("u16", 0, 8, False), ("i64", 0, 8, True), ("u64", 2, 4, False),
                                             ("u128", 0, 16, True), ("f64", 0, 0, False)])
def test_split_matches_oracle(gb, cuda, oracle, split_env, kt, dist, vb, desc, groups):
    split_env(groups=groups)
    n = 200003
    raw = raw_keys(kt, n, seed=groups, dist=dist)
    _host_sort_check(gb, cuda, oracle, kt, raw, raw_values(vb, n, seed=3), desc, pinned=(groups != 3))


def _u32_with_top(n, seed, top_share):
    """u32 keys, `top_share` of them with top byte 0x5A (one big bucket)."""
    rng = np.random.default_rng(seed)
    k = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    big = rng.random(n) < top_share
    k[big] = (k[big] & np.uint32(0x00FFFFFF)) | np.uint32(0x5A000000)
    return k


@pytest.mark.parametrize("case", ["skewed", "near_half", "uniform_top", "low_uniform", "all_equal", "no_skip"])
def test_split_unusual_digits(gb, cuda, oracle, split_env, case):
    """A bucket with most keys (no partition), a uniform top digit, uniform
    low digits (skipped in every group), all keys equal, pass skip off."""
    split_env(groups=8)
    n = 150001
    vals = np.arange(n, dtype=np.uint32)
    kt = "u32"
    if case == "skewed":
        raw = _u32_with_top(n, 1, 0.7)
    elif case == "near_half":
        raw = _u32_with_top(n, 2, 0.45)
    elif case == "uniform_top":
        raw = (_u32_with_top(n, 3, 0.0) & np.uint32(0x00FFFFFF)) | np.uint32(0x11000000)
    elif case == "low_uniform":
        kt = "u64"
        raw = (raw_keys("u64", n, seed=4) & np.uint64(0xFFFF000000000000)) | np.uint64(0x0000000000ABCD00)
    elif case == "all_equal":
        raw = np.full(n, 0xDEADBEEF, dtype=np.uint32)
    else:
        raw = _u32_with_top(n, 5, 0.2)
    if case == "no_skip":
        gb.set_pass_skip(False)
    try:
        _host_sort_check(gb, cuda, oracle, kt, raw, vals, desc=False)
        _host_sort_check(gb, cuda, oracle, kt, raw, None, desc=True, pinned=False)
    finally:
        gb.set_pass_skip(True)


def test_split_at_default_threshold(gb, cuda, oracle):
    """2^25 + 4097 u32 keys with index values: the split path as shipped
    (two groups)."""
    n = (1 << 25) + 4097
    raw = raw_keys("u32", n, seed=11, dist=4)
    _host_sort_check(gb, cuda, oracle, "u32", raw, np.arange(n, dtype=np.uint32), desc=False)
