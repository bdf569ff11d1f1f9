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
