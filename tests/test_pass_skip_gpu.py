"""Uniform-digit pass skipping: passes whose digit is the same for every key
are skipped on the device.  Results must equal the oracle and the sort with
skipping off, for even and odd numbers of executed passes (the odd case ends
with the fix-up copy), no executed pass at all, values, descending order,
signed and float keys, partial tiles; skipped passes must cost ~nothing."""

import numpy as np
import pytest

from _oracle import raw_keys, raw_values
from gpu_util import gpu_sort

pytestmark = pytest.mark.gpu


def _case(kind, n, seed):
    rng = np.random.default_rng(seed)
    if kind == "u32_low16":          # passes 2, 3 uniform: 2 executed
        return "u32", rng.integers(0, 1 << 16, n, dtype=np.uint64).astype(np.uint32)
    if kind == "u32_byte1":          # only byte 1 varies: 1 executed -> fix-up copy
        return "u32", ((rng.integers(0, 256, n, dtype=np.uint64) << 8) | 0x5A).astype(np.uint32)
    if kind == "u32_const":          # every pass uniform: nothing runs
        return "u32", np.full(n, 0xDEADBEEF, dtype=np.uint32)
    if kind == "u64_low32":          # 4 of 8 executed
        return "u64", rng.integers(0, 1 << 32, n, dtype=np.uint64)
    if kind == "u64_mid":            # bytes 2 and 5 vary: 2 executed
        a = rng.integers(0, 256, n, dtype=np.uint64)
        b = rng.integers(0, 256, n, dtype=np.uint64)
        return "u64", (a << np.uint64(16)) | (b << np.uint64(40)) | np.uint64(0x0101000001010101)
    if kind == "i32_small":          # small signed: the twiddled top bytes differ by sign
        return "i32", rng.integers(-300, 300, n).astype(np.int32).view(np.uint32)
    if kind == "f32_few":            # few distinct floats
        return "f32", rng.choice(np.array([1.0, 2.0, 3.0, -0.5], dtype=np.float32), n).view(np.uint32)
    if kind == "u16_hi_const":       # 2 passes, byte 1 constant: 1 executed -> fix-up
        return "u16", (rng.integers(0, 256, n, dtype=np.uint64) | 0x3300).astype(np.uint16)
    if kind == "u8_const":           # 1 pass, uniform
        return "u8", np.full(n, 7, dtype=np.uint8)
    if kind == "u128_low2":          # 16 passes, 2 executed
        k = np.zeros((n, 16), dtype=np.uint8)
        k[:, 0] = rng.integers(0, 256, n)
        k[:, 1] = rng.integers(0, 256, n)
        k[:, 9] = 0x42
        return "u128", k
    raise ValueError(kind)


KINDS = ["u32_low16", "u32_byte1", "u32_const", "u64_low32", "u64_mid", "i32_small", "f32_few", "u16_hi_const",
         "u8_const", "u128_low2"]


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("vb,desc,n", [(0, False, 100003), (4, True, 70001), (8, False, 5000)])
def test_skip_matches_oracle_and_no_skip(gb, cuda, oracle, kind, vb, desc, n):
    kt, raw = _case(kind, n, seed=n + vb)
    vals = raw_values(vb, n, seed=9)
    assert gb.get_pass_skip()
    got = gpu_sort(gb, cuda, kt, raw, desc, vals)
    ref = oracle.sort(kt, raw, desc, vals)
    try:
        gb.set_pass_skip(False)
        plain = gpu_sort(gb, cuda, kt, raw, desc, vals)
    finally:
        gb.set_pass_skip(True)
    if vals is None:
        assert _eq(got, ref) and _eq(got, plain)
    else:
        assert _eq(got[0], ref[0]) and _eq(got[1], ref[1])
        assert _eq(got[0], plain[0]) and _eq(got[1], plain[1])


def test_skipped_passes_cost_nothing(gb, cuda):
    n = 1 << 24  # a pass takes ~60 us: a launch that exits at once is well under a quarter of it
    rng = np.random.default_rng(3)
    keys = cuda.from_numpy(rng.integers(0, 1 << 16, n, dtype=np.uint64).astype(np.uint32).view(np.int32)).cuda()
    tb = gb.temp_bytes("u32", n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    ms = None
    for _ in range(3):
        k = keys.clone()
        ms = gb.sort_timed(k, n, "u32", ws, tb)
    # [upsweep, pass 0..3, fix-up]: passes 2 and 3 exit at once
    assert len(ms) == 6
    assert ms[3] < 0.25 * ms[1] and ms[4] < 0.25 * ms[1], ms
    assert ms[5] < 0.25 * ms[1], ms  # two passes ran: the fix-up copies nothing
    k = k.cpu().numpy().view(np.uint32)
    assert (k[1:] >= k[:-1]).all()
