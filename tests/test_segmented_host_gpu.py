"""Batched sort of host-resident segments (gbsort_segmented_sort_host):
groups of segments copied in, sorted and copied back on overlapping
streams; every segment bit-identical to the oracle, for any group count,
pinned and pageable memory, offsets not starting at 0."""

import numpy as np
import pytest

from _oracle import KEY_BYTES, raw_keys, raw_values

pytestmark = pytest.mark.gpu


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


def _offsets(seed, segments, max_log2=14, start=0):
    rng = np.random.default_rng(seed)
    sizes = np.exp2(rng.uniform(0, max_log2, segments)).astype(np.int64)
    sizes[rng.random(segments) < 0.05] = 0  # empty segments
    return np.concatenate([[start], start + np.cumsum(sizes)]).astype(np.uint64)


def _run(gb, cuda, oracle, kt, vb, desc, off, pinned, seed=1):
    n_all = int(off[-1])
    raw = raw_keys(kt, n_all, seed=seed, dist=4)
    vals = raw_values(vb, n_all, seed=seed + 1)
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
    hb = gb.segmented_host_buffer_bytes(kt, off, vb)
    dbuf = cuda.empty(hb, dtype=cuda.uint8, device="cuda").random_(0, 256)
    gb.segmented_sort_host(kp, kt, off, dbuf, hb, h_values=vp, value_bytes=vb, descending=desc)
    k = read_k().view(raw.dtype).reshape(raw.shape)
    v = None if vals is None else read_v().view(vals.dtype).reshape(vals.shape)
    o0 = int(off[0])
    assert _eq(k[:o0], raw[:o0])  # before the first segment: untouched
    if vals is not None:
        assert _eq(v[:o0], vals[:o0])
    for i in range(len(off) - 1):
        a, b = int(off[i]), int(off[i + 1])
        if vals is None:
            assert _eq(k[a:b], oracle.sort(kt, raw[a:b], desc)), i
        else:
            ek, ev = oracle.sort(kt, raw[a:b], desc, vals[a:b])
            assert _eq(k[a:b], ek) and _eq(v[a:b], ev), i


@pytest.mark.parametrize("groups", [1, 3, 16])
@pytest.mark.parametrize("kt,vb,desc", [("u32", 4, False), ("f64", 0, True), ("u128", 16, False), ("i16", 8, True),
                                        ("u8", 1, False)])
def test_matches_oracle(gb, cuda, oracle, monkeypatch, kt, vb, desc, groups):
    monkeypatch.setenv("GBSORT_HOST_SPLIT_GROUPS", str(groups))
    off = _offsets(groups, 150)
    _run(gb, cuda, oracle, kt, vb, desc, off, pinned=(groups != 3))


def test_large_segments_and_offset_start(gb, cuda, oracle, monkeypatch):
    """Segments big enough for the onesweep path, one bigger than a group's
    share, and a first offset past 0."""
    monkeypatch.setenv("GBSORT_HOST_SPLIT_GROUPS", "8")
    sizes = [300000, 5, 0, 1 << 20, 70000, 4096, 1, 250000]
    off = np.concatenate([[1000], 1000 + np.cumsum(sizes)]).astype(np.uint64)
    _run(gb, cuda, oracle, "u32", 4, False, off, pinned=True, seed=9)


def test_refusals(gb, cuda):
    off = np.array([0, 10, 5], dtype=np.uint64)  # decreasing
    assert gb.segmented_host_buffer_bytes("u32", off) == 0
    with pytest.raises(gb.GbsortError):
        gb.segmented_sort_host(np.zeros(16, np.uint32).ctypes.data, "u32", off, None, 0)
    off = np.array([0, 100, 300], dtype=np.uint64)
    hb = gb.segmented_host_buffer_bytes("u32", off)
    d = cuda.empty(hb, dtype=cuda.uint8, device="cuda")
    keys = np.zeros(300, np.uint32)
    with pytest.raises(gb.GbsortError):  # one byte short
        gb.segmented_sort_host(keys.ctypes.data, "u32", off, d, hb - 1)
