"""Sort server parity: every request's result, after it went through a mixed
coalesced batch, must be bit-identical to the same request sorted alone by
the plain sort and to the oracle; admission by bytes, rejection, in-place
device requests, empty requests and concurrent submitters."""

import threading

import numpy as np
import pytest

from _oracle import KEY_BYTES, raw_keys, raw_values
from gpu_util import gpu_sort, to_dev

pytestmark = pytest.mark.gpu

MEMS = ("pinned", "pageable", "device", "device_inplace")


def _host_buf(cuda, arr: np.ndarray, mem: str):
    """(input, output, reader) for a raw-bit array in the given memory."""
    flat = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
    if mem == "pageable":
        src = flat.copy()
        dst = np.zeros_like(src)
        return src.ctypes.data, dst.ctypes.data, (src, dst), lambda: dst.view(arr.dtype).reshape(arr.shape)
    if mem == "pinned":
        src = cuda.from_numpy(flat.copy()).pin_memory()
        dst = cuda.zeros(flat.shape[0], dtype=cuda.uint8).pin_memory()
        return src.data_ptr(), dst.data_ptr(), (src, dst), \
            lambda: dst.numpy().view(arr.dtype).reshape(arr.shape)
    src = to_dev(cuda, arr)
    if mem == "device_inplace":
        return src.data_ptr(), src.data_ptr(), (src,), lambda: src.cpu().numpy().view(arr.dtype).reshape(arr.shape)
    dst = cuda.zeros_like(src)
    return src.data_ptr(), dst.data_ptr(), (src, dst), lambda: dst.cpu().numpy().view(arr.dtype).reshape(arr.shape)


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


def _make_requests(rng, count):
    types = ("u32", "u64", "f32", "i16", "u128", "f64")
    sizes = (0, 1, 2, 7, 1000, 4097, 20000, 70001, 300000)
    out = []
    for i in range(count):
        kt = types[i % len(types)]
        vb = (0, 4, 8)[int(rng.integers(3))]
        desc = bool(rng.integers(2))
        n = int(sizes[int(rng.integers(len(sizes)))])
        mem = MEMS[i % len(MEMS)]
        out.append((kt, vb, desc, n, mem, int(rng.integers(1 << 30))))
    return out


def test_mixed_batch_equals_alone_and_oracle(gb, cuda, oracle):
    rng = np.random.default_rng(77)
    reqs = _make_requests(rng, 96)
    with gb.Server(pool_bytes=512 << 20, streams=3, paused=True) as srv:
        live = []
        for kt, vb, desc, n, mem, seed in reqs:
            raw = raw_keys(kt, n, seed=seed, dist=4 if seed % 2 else 0)
            if n > 8:
                raw[n // 2:] = raw[: n - n // 2]  # duplicates: stability shows
            vals = raw_values(vb, n, seed=seed + 1)
            kin, kout, hold_k, read_k = _host_buf(cuda, raw, mem)
            vin = vout = read_v = None
            hold_v = ()
            if vals is not None:
                vin, vout, hold_v, read_v = _host_buf(cuda, vals, mem)
            t = srv.submit(kt, n, kin, kout, vin, vout, value_bytes=vb, descending=desc)
            live.append((t, kt, vb, desc, raw, vals, read_k, read_v, hold_k, hold_v))
        srv.resume()
        assert srv.drain(120.0) == gb.OK
        for t, kt, vb, desc, raw, vals, read_k, read_v, _, _ in live:
            assert srv.poll(t) == gb.OK
            k = read_k()
            v = None if read_v is None else read_v()
            # alone: the plain sort of the same input
            if vals is None:
                alone_k, alone_v = gpu_sort(gb, cuda, kt, raw, desc), None
                ek, ev = oracle.sort(kt, raw, desc), None
            else:
                alone_k, alone_v = gpu_sort(gb, cuda, kt, raw, desc, vals)
                ek, ev = oracle.sort(kt, raw, desc, vals)
            assert _eq(k, alone_k) and _eq(k, ek), (kt, vb, desc, raw.shape[0])
            if vals is not None:
                assert _eq(v, alone_v) and _eq(v, ev), (kt, vb, desc, raw.shape[0])
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        # paused while everything queued: classes were coalesced
        assert st["batches"] < sum(1 for r in reqs if r[3] > 0)
        assert st["max_batch_requests"] > 1
        assert st["pool_peak_bytes"] <= 512 << 20
        assert st["latency_p99_us"] >= st["latency_p50_us"] > 0


def test_admission_by_bytes_and_rejection(gb, cuda, oracle):
    pool = 24 << 20
    with gb.Server(pool_bytes=pool, streams=2, paused=True) as srv:
        big = 4 << 20  # u32 + u32 values: ~32 MiB staged + workspace > pool
        k = cuda.zeros(big * 4, dtype=cuda.uint8, device="cuda")
        st, t = srv.try_submit("u32", big, k.data_ptr(), cuda.zeros_like(k).data_ptr(), k.data_ptr(),
                               cuda.zeros_like(k).data_ptr(), value_bytes=4)
        assert st == gb.ERR_BUDGET and t is None
        # each fits alone, all together need several times the pool
        items = []
        for i in range(12):
            n = 600000 + 1000 * i
            raw = raw_keys("u32", n, seed=i)
            vals = np.arange(n, dtype=np.uint32)
            dk, dv = to_dev(cuda, raw), to_dev(cuda, vals)
            ok, ov = cuda.zeros_like(dk), cuda.zeros_like(dv)
            t = srv.submit("u32", n, dk, ok, dv, ov, value_bytes=4)
            items.append((t, raw, vals, ok, ov, dk, dv))  # inputs stay alive until drained
        srv.resume()
        assert srv.drain(120.0) == gb.OK
        for t, raw, vals, ok, ov, _, _ in items:
            assert srv.poll(t) == gb.OK
            ek, ev = oracle.sort("u32", raw, False, vals)
            assert _eq(ok.cpu().numpy().view(np.uint32), ek) and _eq(ov.cpu().numpy().view(np.uint32), ev)
        s = srv.stats()
        assert s["rejected"] == 1 and s["completed"] == 12
        assert 0 < s["pool_peak_bytes"] <= pool
        assert s["batches"] >= 3  # the pool cannot hold them at once
        assert srv.poll(items[0][0]) == gb.ERR_INVALID_ARGUMENT  # retired


def test_concurrent_submitters_and_tickets(gb, cuda, oracle):
    with gb.Server(pool_bytes=256 << 20, streams=4) as srv:
        results = {}
        errors = []

        def client(cid):
            try:
                rng = np.random.default_rng(cid)
                mine = []
                for j in range(10):
                    kt = ("u32", "u64", "f32")[j % 3]
                    n = int(rng.integers(1, 50000))
                    raw = raw_keys(kt, n, seed=cid * 100 + j)
                    vals = np.arange(n, dtype=np.uint32) if j % 2 else None
                    kin = cuda.from_numpy(raw.view(np.uint8).reshape(-1).copy()).pin_memory()
                    vin = None if vals is None else cuda.from_numpy(vals.view(np.uint8).copy()).pin_memory()
                    t = srv.submit(kt, n, kin, values_in=vin, value_bytes=4 if vals is not None else 0)
                    mine.append((t, kt, raw, vals, kin, vin))
                for t, kt, raw, vals, kin, vin in mine:
                    assert srv.wait(t, 60.0) == gb.OK
                    results[(cid, t)] = (kt, raw, vals, kin, vin)
            except Exception as e:  # surfaced below
                errors.append(e)

        th = [threading.Thread(target=client, args=(c,)) for c in range(4)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        assert not errors, errors
        assert len(results) == 40
        for kt, raw, vals, kin, vin in results.values():
            k = kin.numpy().view(raw.dtype)
            if vals is None:
                assert _eq(k, oracle.sort(kt, raw, False))
            else:
                ek, ev = oracle.sort(kt, raw, False, vals)
                assert _eq(k, ek) and _eq(vin.numpy().view(np.uint32), ev)


def test_workspace_reset(gb, cuda):
    n = 5000
    tb = gb.temp_bytes("u32", n)
    ws = cuda.full((tb,), 0xFF, dtype=cuda.uint8, device="cuda")
    assert gb.workspace_status("u32", n, ws) != gb.OK  # garbage error word
    gb.workspace_reset("u32", n, ws)
    assert gb.workspace_status("u32", n, ws) == gb.OK
