"""Input-preserving (DoubleBuffer-style) sort: the input stays untouched and
the output equals the oracle, for every key width, with and without values,
both orders, partial tiles, and inputs whose uniform digits make the sort run
an odd, even or zero number of passes (with pass skipping on and off)."""

import numpy as np
import pytest

from _oracle import raw_keys, raw_values
from gpu_util import from_dev, to_dev
from test_pass_skip_gpu import KINDS, _case

pytestmark = pytest.mark.gpu


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


def _run(gb, cuda, kt, raw, desc, vals):
    n = raw.shape[0]
    vb = 0 if vals is None else vals.dtype.itemsize * (vals.shape[1] if vals.ndim == 2 else 1)
    kin = to_dev(cuda, raw)
    kout = cuda.full_like(kin, 0x5A)
    vin = None if vals is None else to_dev(cuda, vals)
    vout = None if vals is None else cuda.full_like(vin, 0xA5)
    tb = gb.temp_bytes(kt, n, vb)
    ws = cuda.empty(max(1, tb), dtype=cuda.uint8, device="cuda")
    gb.sort_copy(kin, kout, n, kt, ws, tb, values_in=vin, values_out=vout, value_bytes=vb, descending=desc)
    cuda.cuda.synchronize()
    assert gb.workspace_status(kt, n, ws, vb) == gb.OK
    assert _eq(from_dev(kin, raw), raw)  # input preserved
    if vals is not None:
        assert _eq(from_dev(vin, vals), vals)
    k = from_dev(kout, raw)
    return k if vals is None else (k, from_dev(vout, vals))


@pytest.mark.parametrize("kt", ["u8", "u16", "u32", "i64", "f32", "f64", "u128", "f128"])
@pytest.mark.parametrize("vb,desc", [(0, False), (4, True), (8, False), (16, True)])
def test_copy_matches_oracle_input_kept(gb, cuda, oracle, kt, vb, desc):
    for n in (1, 7, 9216, 100003):
        raw = raw_keys(kt, n, seed=n, dist=4)
        vals = raw_values(vb, n, seed=2)
        got = _run(gb, cuda, kt, raw, desc, vals)
        ref = oracle.sort(kt, raw, desc, vals)
        if vals is None:
            assert _eq(got, ref), n
        else:
            assert _eq(got[0], ref[0]) and _eq(got[1], ref[1]), n


@pytest.mark.parametrize("skip", [True, False])
@pytest.mark.parametrize("kind", KINDS)
def test_copy_with_uniform_digits(gb, cuda, oracle, kind, skip):
    kt, raw = _case(kind, 50001, seed=11)
    vals = raw_values(4, raw.shape[0], seed=1)
    try:
        gb.set_pass_skip(skip)
        got = _run(gb, cuda, kt, raw, False, vals)
    finally:
        gb.set_pass_skip(True)
    ref = oracle.sort(kt, raw, False, vals)
    assert _eq(got[0], ref[0]) and _eq(got[1], ref[1])


def test_copy_aliasing_rules(gb, cuda, oracle):
    n = 10000
    raw = raw_keys("u32", n, seed=5)
    buf = to_dev(cuda, raw)
    tb = gb.temp_bytes("u32", n)
    ws = cuda.empty(tb, dtype=cuda.uint8, device="cuda")
    gb.sort_copy(buf, buf, n, "u32", ws, tb)  # identical: in place
    cuda.cuda.synchronize()
    assert _eq(from_dev(buf, raw), oracle.sort("u32", raw))
    big = cuda.zeros(2 * n * 4, dtype=cuda.uint8, device="cuda")
    with pytest.raises(gb.GbsortError):
        gb.sort_copy(big.data_ptr(), big.data_ptr() + 4 * 100, n, "u32", ws, tb)  # partial overlap
    gb.sort_copy(None, None, 0, "u32", ws, tb)  # n = 0: nothing to do
