"""Full-size parity: the benchmark configurations at their real sizes, checked
on the device against an independent stable sort.

The CPU oracle would take minutes at these sizes, so the checker here is
torch's stable sort of the twiddled keys (a device-side restatement of the
reference's twiddle, include/rsort/detail/tuning.cuh:352-384, in int64
arithmetic).  A stable sort of the twiddled keys is exactly the reference's
result, so keys and values must match bit for bit; that also proves the
output is a permutation (size-independent property) and that equal keys kept
their input order (stability).
"""

import pytest

pytestmark = pytest.mark.gpu

U32_MASK = 0xFFFFFFFF
SIGN64 = -(1 << 63)


def _sort(gb, torch, kt, keys, n, vals=None, vb=0, desc=False):
    tb = gb.temp_bytes(kt, n, vb)
    ws = torch.empty(tb, dtype=torch.uint8, device="cuda")
    gb.sort(keys, n, kt, ws, tb, values=vals, value_bytes=vb, descending=desc)
    torch.cuda.synchronize()
    assert gb.workspace_status(kt, n, ws, vb) == gb.OK
    del ws


def test_u32_keys_2p28(gb, cuda):
    torch = cuda
    n = 1 << 28
    keys = torch.empty(n, dtype=torch.int32, device="cuda")
    gb.generate(0, 4, keys, n, 2028)
    expect = torch.sort(keys.to(torch.int64) & U32_MASK).values
    _sort(gb, torch, "u32", keys, n)
    got = keys.to(torch.int64) & U32_MASK
    assert torch.equal(got, expect)


def test_f32_pairs_2p28_specials_stable(gb, cuda):
    torch = cuda
    n = 1 << 28
    keys = torch.empty(n, dtype=torch.int32, device="cuda")
    gb.generate(1, 4, keys, n, 77)
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    bits = keys.to(torch.int64) & U32_MASK
    neg = (bits >> 31) == 1
    tw = torch.where(neg, (~bits) & U32_MASK, bits | 0x80000000)  # twiddle_in for floats
    del neg, bits
    perm = torch.sort(tw, stable=True).indices
    del tw
    expect_keys = keys[perm]
    _sort(gb, torch, "f32", keys, n, vals, 4)
    assert torch.equal(vals.to(torch.int64), perm)
    assert torch.equal(keys, expect_keys)


def test_u64_pairs_2p27_dup_prefix_desc(gb, cuda):
    torch = cuda
    n = 1 << 27
    keys = torch.empty(n, dtype=torch.int64, device="cuda")
    gb.generate(2, 8, keys, n, 31)
    vals = torch.arange(n, dtype=torch.int64, device="cuda")
    order_key = (~keys) ^ SIGN64  # descending twiddle, then unsigned -> signed order
    perm = torch.sort(order_key, stable=True).indices
    del order_key
    expect_keys = keys[perm]
    _sort(gb, torch, "u64", keys, n, vals, 8, desc=True)
    assert torch.equal(vals, perm)
    assert torch.equal(keys, expect_keys)


def test_u128_keys_2p26_desc(gb, cuda):
    torch = cuda
    n = 1 << 26
    keys = torch.empty((n, 2), dtype=torch.int64, device="cuda")  # [lo, hi] little-endian halves
    gb.generate(0, 16, keys, n, 5)
    lo = (~keys[:, 0]) ^ SIGN64
    hi = (~keys[:, 1]) ^ SIGN64
    p1 = torch.sort(lo, stable=True).indices          # LSD over two 64-bit digits
    p2 = torch.sort(hi[p1], stable=True).indices
    perm = p1[p2]
    del lo, hi, p1, p2
    expect = keys[perm]
    _sort(gb, torch, "u128", keys, n, desc=True)
    assert torch.equal(keys, expect)


@pytest.mark.parametrize("kt,kb,n,vb", [
    ("u16", 2, (1 << 29) + 12345, 0),   # 2 passes: 64-bit status words past 2^29
    ("i32", 4, (1 << 28) + 4097, 4),    # 4 passes: past 2^28, with index values
    ("f64", 8, (1 << 27) + 777, 8),     # 8 passes: past 2^27, with index values
    ("u128", 16, (1 << 26) + 5, 0),     # 16 passes: past 2^26
])
def test_wide_status_words(gb, cuda, kt, kb, n, vb):
    """Sizes just past each key width's 32-bit status-word limit
    (n > 2^(30 - log2 passes)) run the 64-bit status instantiations; checked
    on the device: sorted order, the same multiset of keys, and (with index
    values) every value pointing at an input key equal to its output key."""
    torch = cuda
    plan = gb.plan(kt, n, vb)
    assert plan.status_word_bytes == 8
    keys = torch.empty(n * kb, dtype=torch.uint8, device="cuda")
    gb.generate(4, kb, keys, n, 99)  # the reference's random mode (duplicates for u16)
    src = keys.clone()
    vals = None
    if vb:
        vals = torch.empty(n * vb, dtype=torch.uint8, device="cuda")
        gb.generate(3, vb, vals, n, 0)  # original index
    for desc in (False, True):
        keys.copy_(src)
        if vb:
            gb.generate(3, vb, vals, n, 0)
        _sort(gb, torch, kt, keys, n, vals, vb, desc)
        assert gb.check_order(keys, n, kt, desc) == 0
        assert gb.checksum(keys, n, kt) == gb.checksum(src, n, kt)
        if vb:
            assert gb.check_pairs(src, keys, vals, vb, n, kt) == 0


@pytest.mark.parametrize("kt,vb", [("u32", 0), ("f32", 4), ("u64", 8)])
def test_short_array_shape_boundary(gb, cuda, oracle, kt, vb):
    """n <= 2^22 takes the short-array pass shape, larger n the default one:
    both sides of the switch against the oracle."""
    import os

    import numpy as np

    from _oracle import raw_keys, raw_values
    from gpu_util import gpu_sort

    threads = max(1, min(16, os.cpu_count() or 1))
    for n in ((1 << 22) - 1, 1 << 22, (1 << 22) + 1):
        raw = raw_keys(kt, n, seed=n, dist=4)
        vals = raw_values(vb, n, seed=1)
        got = gpu_sort(gb, cuda, kt, raw, False, vals)
        ref = oracle.sort(kt, raw, False, vals, threads=threads)
        if vals is None:
            assert np.array_equal(got.view(np.uint8), ref.view(np.uint8)), n
        else:
            assert np.array_equal(got[0].view(np.uint8), ref[0].view(np.uint8)), n
            assert np.array_equal(got[1].view(np.uint8), ref[1].view(np.uint8)), n
