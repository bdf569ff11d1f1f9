"""Batched (segmented) sort parity: every segment must equal the oracle's
stable sort of that segment alone, bit for bit, for every path (CTA-sized
segments, onesweep segments), key widths (incl. odd pass counts), value
sizes and both orders; graph replay and forced paths give the same result."""

import numpy as np
import pytest

from _oracle import KEY_BYTES, raw_keys, raw_values
from gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


def _layout(rng, count, lo_log2, hi_log2, extras=()):
    sizes = np.floor(np.exp2(rng.uniform(lo_log2, hi_log2, count))).astype(np.int64)
    sizes = np.concatenate([sizes, np.array(extras, dtype=np.int64)])
    rng.shuffle(sizes)
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)


def _expected(oracle, kt, raw, vals, off, desc):
    k = raw.copy()
    v = None if vals is None else vals.copy()
    for s in range(len(off) - 1):
        b, e = int(off[s]), int(off[s + 1])
        if e - b <= 1:
            continue
        if v is None:
            k[b:e] = oracle.sort(kt, raw[b:e], desc)
        else:
            k[b:e], v[b:e] = oracle.sort(kt, raw[b:e], desc, vals[b:e])
    return k, v


def _run(gb, cuda, kt, raw, vals, off, desc, use_graph=True, reps=1, regen=None):
    vb = 0 if vals is None else vals.dtype.itemsize * (vals.shape[1] if vals.ndim == 2 else 1)
    plan = gb.SegmentedPlan(kt, off, vb, desc)
    ws = cuda.empty(max(1, plan.workspace_bytes), dtype=cuda.uint8, device="cuda")
    dk = to_dev(cuda, raw)
    dv = None if vals is None else to_dev(cuda, vals)
    s = cuda.cuda.Stream()
    plan.bind(dk, ws, plan.workspace_bytes, values=dv, stream=s)
    out = []
    for r in range(reps):
        if r > 0 and regen is not None:
            raw, vals = regen(r)
            dk.copy_(to_dev(cuda, raw))
            if dv is not None:
                dv.copy_(to_dev(cuda, vals))
            cuda.cuda.synchronize()
        plan.run(stream=s, use_graph=use_graph)
        assert plan.status(stream=s) == gb.OK
        out.append((raw, vals, from_dev(dk, raw), None if dv is None else from_dev(dv, vals)))
    info = plan.info()
    plan.close()
    return out, info


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("kt,vb,desc", [("u32", 4, False), ("f32", 0, False), ("u64", 8, True), ("i16", 2, True),
                                        ("u8", 4, False), ("u128", 0, True), ("f64", 16, False), ("i32", 1, True)])
def test_segmented_matches_per_segment_oracle(gb, cuda, oracle, kt, vb, desc):
    rng = np.random.default_rng(hash((kt, vb, desc)) & 0xFFFF)
    off = _layout(rng, 120, 0, 17, extras=(0, 1, 2, 2047, 2048, 2049, 8192, 8193, 5120, 5121, 200000))
    n = int(off[-1])
    raw = raw_keys(kt, n, seed=n, dist=4)
    raw[n // 2:] = raw[: n - n // 2]  # duplicates across and within segments
    vals = raw_values(vb, n, seed=3)
    (r0, v0, k, v), = _run(gb, cuda, kt, raw, vals, off, desc)[0]
    ek, ev = _expected(oracle, kt, raw, vals, off, desc)
    assert _eq(k, ek)
    if vals is not None:
        assert _eq(v, ev)


def test_graph_replay_and_paths_agree(gb, cuda, oracle):
    rng = np.random.default_rng(5)
    off = _layout(rng, 300, 6, 16)
    n = int(off[-1])

    def regen(r):
        return raw_keys("u32", n, seed=100 + r), np.arange(n, dtype=np.uint32)

    raw, vals = regen(0)
    results, info = _run(gb, cuda, "u32", raw, vals, off, False, use_graph=True, reps=3, regen=regen)
    assert info["cta_small_segments"] and info["cta_large_segments"] and info["onesweep_segments"]
    for r_raw, r_vals, k, v in results:
        ek, ev = _expected(oracle, "u32", r_raw, r_vals, off, False)
        assert _eq(k, ek) and _eq(v, ev)
    # every bucket forced through onesweep, then through the CTA paths
    try:
        for path in (gb.PATH_ONESWEEP, gb.PATH_CTA_S):
            gb.set_segmented_path("u32", 4, -1, path)
            (r_raw, r_vals, k, v), = _run(gb, cuda, "u32", raw, vals, off, False)[0]
            ek, ev = _expected(oracle, "u32", raw, vals, off, False)
            assert _eq(k, ek) and _eq(v, ev)
    finally:
        gb.set_segmented_path("u32", 4, -1, -1)


def test_one_shot_segmented_sort(gb, cuda, oracle):
    rng = np.random.default_rng(9)
    off = _layout(rng, 50, 4, 15)
    n = int(off[-1])
    raw = raw_keys("i64", n, seed=1)
    tb = gb.segmented_sort(None, "i64", off)
    ws = cuda.empty(max(1, tb), dtype=cuda.uint8, device="cuda")
    dk = to_dev(cuda, raw)
    gb.segmented_sort(dk, "i64", off, ws, tb)
    ek, _ = _expected(oracle, "i64", raw, None, off, False)
    assert _eq(from_dev(dk, raw), ek)


def test_segments_at_unaligned_offsets(gb, cuda, oracle):
    """Segments starting anywhere: onesweep tiles begin off the 16-byte grid."""
    sizes = [13, 7001, 3, 40001, 5121, 9999, 1, 65537]
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    n = int(off[-1])
    raw = raw_keys("u16", n, seed=4)
    vals = raw_values(8, n, seed=4)
    try:
        gb.set_segmented_path("u16", 8, -1, gb.PATH_ONESWEEP)
        (r, v0, k, v), = _run(gb, cuda, "u16", raw, vals, off, False)[0]
    finally:
        gb.set_segmented_path("u16", 8, -1, -1)
    ek, ev = _expected(oracle, "u16", raw, vals, off, False)
    assert _eq(k, ek) and _eq(v, ev)


def test_autotuner_installs_paths_and_stays_exact(gb, cuda, oracle):
    scratch_bytes = 160 << 20
    scratch = cuda.empty(scratch_bytes, dtype=cuda.uint8, device="cuda")
    try:
        report = gb.autotune_segmented("u32", 4, scratch, scratch_bytes, 4, 12)
        lines = [ln for ln in report.splitlines() if ln.startswith("bucket")]
        assert len(lines) == 9 and all("->" in ln for ln in lines)
        chosen = {b: gb.get_segmented_path("u32", 4, b) for b in range(4, 13)}
        assert all(v in (gb.PATH_CTA_S, gb.PATH_CTA_S4, gb.PATH_CTA_L, gb.PATH_ONESWEEP) for v in chosen.values())
        text = gb.segmented_tuning_text()
        assert len([ln for ln in text.splitlines() if ln.startswith("2 4 ")]) >= 1
        rng = np.random.default_rng(21)
        off = _layout(rng, 200, 4, 13)
        n = int(off[-1])
        raw = raw_keys("u32", n, seed=8)
        vals = np.arange(n, dtype=np.uint32)
        (r, v0, k, v), = _run(gb, cuda, "u32", raw, vals, off, False)[0]
        ek, ev = _expected(oracle, "u32", raw, vals, off, False)
        assert _eq(k, ek) and _eq(v, ev)
        gb.segmented_tuning_load(text)  # round trip
    finally:
        gb.set_segmented_path("u32", 4, -1, -1)


@pytest.mark.parametrize("skip", [True, False])
@pytest.mark.parametrize("path", ["PATH_CTA_S", "PATH_CTA_S4", "PATH_CTA_L", "PATH_ONESWEEP"])
@pytest.mark.parametrize("kt,mask", [("u32", 0x00000FFF), ("u64", 0x0000FF00FF0000FF), ("i16", 0x00FF)])
def test_uniform_digits_per_segment(gb, cuda, oracle, path, kt, mask, skip):
    """Keys whose masked-out bytes are constant: those digit passes are
    uniform inside every segment.  The CTA sort short-circuits them; the
    onesweep path skips them (u32: 2 of 4 run; u64: 3 of 8 run, ending with
    the copy home; i16: 1 of 2 runs, copy home), or runs them all with
    skipping off."""
    rng = np.random.default_rng(31)
    off = _layout(rng, 150, 2, 12, extras=(0, 1, 4095, 4096))
    n = int(off[-1])
    raw = raw_keys(kt, n, seed=17)
    dt = raw.dtype
    raw = ((raw.astype(np.uint64) & np.uint64(mask)) | np.uint64(0x0101010101010101 & ~mask)).astype(dt)
    vals = np.arange(n, dtype=np.uint32)
    vb = 4
    try:
        gb.set_pass_skip(skip)
        gb.set_segmented_path(kt, vb, -1, getattr(gb, path))
        (r, v0, k, v), = _run(gb, cuda, kt, raw, vals, off, False)[0]
    finally:
        gb.set_segmented_path(kt, vb, -1, -1)
        gb.set_pass_skip(True)
    ek, ev = _expected(oracle, kt, raw, vals, off, False)
    assert _eq(k, ek) and _eq(v, ev)
