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
