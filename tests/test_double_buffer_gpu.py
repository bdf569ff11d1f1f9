"""DoubleBuffer sort (gbsort_sort_keys/pairs_double_buffer), the form of
cub::DoubleBuffer in the reference's CUB comparator: the result lands in
the buffer the returned selector names, bit-identical to the oracle, for
both starting selectors, odd pass counts (1-byte keys), and uniform digits
that leave the executed passes' parity off the pass count's (the fix-up
copy then runs in either direction)."""

import numpy as np
import pytest

from _oracle import KEY_BYTES, raw_keys, raw_values
from gpu_util import from_dev, to_dev, value_bytes_of

pytestmark = pytest.mark.gpu


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


def _db_sort(gb, cuda, kt, raw, vals, desc, sel, stream=None, ws=None):
    n = raw.shape[0]
    vb = value_bytes_of(vals)
    kb = KEY_BYTES[kt]
    bufs = [cuda.empty(max(1, n * kb), dtype=cuda.uint8, device="cuda").random_(0, 256) for _ in range(2)]
    vbufs = [cuda.empty(max(1, n * vb), dtype=cuda.uint8, device="cuda").random_(0, 256) for _ in range(2)] \
        if vb else [None, None]
    if n:
        bufs[sel].copy_(to_dev(cuda, raw))
        if vb:
            vbufs[sel].copy_(to_dev(cuda, vals))
    tb = gb.double_buffer_bytes(kt, n, vb)
    if ws is None:
        ws = cuda.empty(max(tb, 16), dtype=cuda.uint8, device="cuda").random_(0, 256)
    out = gb.sort_double_buffer(bufs[0], bufs[1], n, kt, ws, tb, selector=sel, values0=vbufs[0], values1=vbufs[1],
                                value_bytes=vb, descending=desc, stream=stream)
    cuda.cuda.synchronize()
    assert gb.double_buffer_status(kt, n, ws, vb) == gb.OK
    k = from_dev(bufs[out], raw) if n else raw.copy()
    v = None if vals is None else (from_dev(vbufs[out], vals) if n else vals.copy())
    return out, k, v


def _check(oracle, kt, raw, vals, desc, k, v):
    if vals is None:
        assert _eq(k, oracle.sort(kt, raw, desc))
    else:
        ek, ev = oracle.sort(kt, raw, desc, vals)
        assert _eq(k, ek) and _eq(v, ev)


@pytest.mark.parametrize("kt", ["u8", "i16", "u32", "f32", "i64", "f64", "u128", "f128"])
@pytest.mark.parametrize("vb,desc", [(0, False), (4, True), (8, False), (16, True)])
@pytest.mark.parametrize("sel", [0, 1])
def test_matches_oracle(gb, cuda, oracle, kt, vb, desc, sel):
    for n in (0, 1, 7, 9216, 100003):
        raw = raw_keys(kt, n, seed=n + sel, dist=4)
        vals = raw_values(vb, n, seed=5)
        out, k, v = _db_sort(gb, cuda, kt, raw, vals, desc, sel)
        assert out == (sel ^ (KEY_BYTES[kt] & 1) if n else sel), n
        _check(oracle, kt, raw, vals, desc, k, v)


@pytest.mark.parametrize("skip", [True, False])
@pytest.mark.parametrize("case", ["u8_equal", "u16_high_uniform", "u32_one_uniform", "u32_two_uniform",
                                  "u64_all_uniform"])
def test_uniform_digits(gb, cuda, oracle, case, skip):
    """Executed-pass parity different from the pass count's: the result is
    copied to the buffer the selector names (or nothing is skipped)."""
    n = 40001
    rng = np.random.default_rng(3)
    kt = {"u8_equal": "u8", "u16_high_uniform": "u16", "u32_one_uniform": "u32", "u32_two_uniform": "u32",
          "u64_all_uniform": "u64"}[case]
    if case == "u8_equal":
        raw = np.full(n, 0x5A, dtype=np.uint8)  # P = 1, E = 0
    elif case == "u16_high_uniform":
        raw = (rng.integers(0, 256, n, dtype=np.uint64).astype(np.uint16) | np.uint16(0x3300))  # P = 2, E = 1
    elif case == "u32_one_uniform":
        raw = rng.integers(0, 1 << 24, n, dtype=np.uint64).astype(np.uint32)  # P = 4, E = 3
    elif case == "u32_two_uniform":
        raw = rng.integers(0, 1 << 16, n, dtype=np.uint64).astype(np.uint32)  # P = 4, E = 2
    else:
        raw = np.full(n, 0x0123456789ABCDEF, dtype=np.uint64)  # P = 8, E = 0
    vals = np.arange(n, dtype=np.uint32)
    try:
        gb.set_pass_skip(skip)
        for sel in (0, 1):
            out, k, v = _db_sort(gb, cuda, kt, raw, vals, False, sel)
            assert out == sel ^ (KEY_BYTES[kt] & 1)
            _check(oracle, kt, raw, vals, False, k, v)
    finally:
        gb.set_pass_skip(True)


def test_graph_replay_and_workspace_size(gb, cuda, oracle):
    """Repeated identical calls (captured, then replayed) stay exact with new
    data; the workspace is far smaller than the in-place form's."""
    n = 1 << 20
    assert gb.double_buffer_bytes("u32", n) == gb.temp_bytes("u32", n) - n * 4  # no alternate buffer
    s = cuda.cuda.Stream()
    b0 = cuda.empty(n * 4, dtype=cuda.uint8, device="cuda")
    b1 = cuda.empty(n * 4, dtype=cuda.uint8, device="cuda")
    tb = gb.double_buffer_bytes("u32", n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    st0 = gb.graph_cache_stats()
    for rep in range(4):
        raw = raw_keys("u32", n, seed=50 + rep)
        b0.copy_(to_dev(cuda, raw))
        cuda.cuda.synchronize()
        out = gb.sort_double_buffer(b0, b1, n, "u32", ws, tb, selector=0, stream=s)
        s.synchronize()
        assert out == 0
        assert _eq(from_dev(b0, raw), oracle.sort("u32", raw)), rep
    st1 = gb.graph_cache_stats()
    assert st1["captures"] >= st0["captures"] + 1 and st1["replays"] >= st0["replays"] + 3


def test_refuses_overlap_and_bad_selector(gb, cuda):
    n = 1000
    buf = cuda.empty(n * 8, dtype=cuda.uint8, device="cuda")
    tb = gb.double_buffer_bytes("u32", n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    with pytest.raises(gb.GbsortError):
        gb.sort_double_buffer(buf, buf.data_ptr() + 400, n, "u32", ws, tb)  # the two buffers overlap
    with pytest.raises(gb.GbsortError):
        gb.sort_double_buffer(buf, buf.data_ptr() + 4 * n, n, "u32", ws, tb, selector=2)
    with pytest.raises(gb.GbsortError):
        gb.sort_double_buffer(buf, buf.data_ptr() + 4 * n, n, "u32", ws, tb - 1)  # workspace too small
