"""Graph replay of repeated identical sort calls: replays stay bit-exact when
the data in the same buffers changes, a changed setting (order, pass skip)
never reuses a stale graph, a sort inside the caller's own stream capture
still works, and clearing the cache is safe."""

import numpy as np
import pytest

from _oracle import raw_keys
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


# (u32 2^20: the one-launch sort; u128 2^22 + 33 keys only: most significant
# digit first across launches, whose state and counters the replayed graph
# clears again every time)
@pytest.mark.parametrize("kt,vb,n", [("u32", 0, 1 << 20), ("f64", 4, 100003), ("u128", 8, 30001),
                                     ("u128", 0, (1 << 22) + 33)])
def test_replays_exact_with_fresh_data(gb, cuda, oracle, kt, vb, n):
    assert gb.get_graph_cache()
    s = cuda.cuda.Stream()
    first = raw_keys(kt, n, seed=1)
    dk = to_dev(cuda, first)
    dv = to_dev(cuda, np.arange(n, dtype=np.uint32 if vb == 4 else np.uint64)) if vb else None
    tb = gb.temp_bytes(kt, n, vb)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    for rep in range(5):  # direct, capture, replay, replay, replay
        raw = raw_keys(kt, n, seed=10 + rep)
        vals = np.arange(n, dtype=np.uint32 if vb == 4 else np.uint64)[::-1].copy() if vb else None
        with cuda.cuda.stream(s):
            dk.copy_(to_dev(cuda, raw))
            if vb:
                dv.copy_(to_dev(cuda, vals))
        desc = rep == 3  # one call with another order: a different graph
        gb.sort(dk, n, kt, ws, tb, values=dv, value_bytes=vb, descending=desc, stream=s)
        s.synchronize()
        assert gb.workspace_status(kt, n, ws, vb) == gb.OK
        if vb:
            ek, ev = oracle.sort(kt, raw, desc, vals)
            assert _eq(from_dev(dk, raw), ek) and _eq(from_dev(dv, vals), ev), rep
        else:
            assert _eq(from_dev(dk, raw), oracle.sort(kt, raw, desc)), rep


def test_setting_change_and_clear(gb, cuda, oracle):
    n = 50000
    s = cuda.cuda.Stream()
    rng = np.random.default_rng(2)
    dk = cuda.empty(n * 4, dtype=cuda.uint8, device="cuda")
    tb = gb.temp_bytes("u32", n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    try:
        for rep in range(6):
            gb.set_pass_skip(rep % 2 == 0)
            raw = rng.integers(0, 1 << 16, n, dtype=np.uint64).astype(np.uint32)  # 2 uniform digits
            with cuda.cuda.stream(s):
                dk.copy_(to_dev(cuda, raw))
            gb.sort(dk, n, "u32", ws, tb, stream=s)
            s.synchronize()
            assert _eq(from_dev(dk, raw), oracle.sort("u32", raw)), rep
    finally:
        gb.set_pass_skip(True)
    gb.graph_cache_clear()
    gb.sort(dk, n, "u32", ws, tb, stream=s)  # still fine afterwards
    s.synchronize()
    assert gb.check_order(dk, n, "u32") == 0


def test_inside_callers_capture(gb, cuda, oracle):
    n = 1 << 18
    s = cuda.cuda.Stream()
    dk = cuda.empty(n * 4, dtype=cuda.uint8, device="cuda")
    src = cuda.empty_like(dk)
    tb = gb.temp_bytes("u32", n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    gb.generate(0, 4, src, n, 3)
    with cuda.cuda.stream(s):
        dk.copy_(src)
        gb.sort(dk, n, "u32", ws, tb, stream=s)  # warm: kernels prepared outside the capture
    s.synchronize()
    g = cuda.cuda.CUDAGraph()
    with cuda.cuda.graph(g, stream=s):
        dk.copy_(src)
        gb.sort(dk, n, "u32", ws, tb, stream=s)
    for seed in (4, 5):
        gb.generate(0, 4, src, n, seed)
        cuda.cuda.synchronize()
        g.replay()
        cuda.cuda.synchronize()
        raw = src.cpu().numpy().view(np.uint32)
        assert _eq(dk.cpu().numpy().view(np.uint32), oracle.sort("u32", raw))


def test_least_recently_used_call_is_replaced(gb, cuda):
    """Once 32 calls are tracked, a new call replaces the least recently used
    one, so a call repeated after many distinct ones still gets its graph."""
    s = cuda.cuda.Stream()
    nmax = 8000
    dk = cuda.empty(nmax * 4, dtype=cuda.uint8, device="cuda")
    tb = gb.temp_bytes("u32", nmax)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    gb.generate(0, 4, dk, nmax, 9)
    cuda.cuda.synchronize()
    gb.graph_cache_clear()
    for i in range(40):  # 40 distinct calls, each once
        gb.sort(dk, 1000 + i, "u32", ws, tb, stream=s)
    s.synchronize()
    st0 = gb.graph_cache_stats()
    assert st0["calls"] == 32 and st0["graphs"] == 0
    for rep in range(3):  # tracked, captured + launched, replayed
        gb.generate(0, 4, dk, nmax, 20 + rep)
        cuda.cuda.synchronize()
        gb.sort(dk, 5000, "u32", ws, tb, stream=s)
        s.synchronize()
        assert gb.check_order(dk, 5000, "u32") == 0, rep
    st1 = gb.graph_cache_stats()
    assert st1["calls"] == 32 and st1["graphs"] == 1
    assert st1["captures"] == st0["captures"] + 1 and st1["replays"] == st0["replays"] + 2
    gb.graph_cache_clear()
    assert gb.graph_cache_stats()["calls"] == 0
