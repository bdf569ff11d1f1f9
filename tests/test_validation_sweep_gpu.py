"""The reference's validation sweep, against the oracle, bit for bit.

benchmark/validate_sort.cuh:20-147 validates every key type (13, incl.
__int128 and long double) x every value kind (none, u32, u8, u16, u64, u128)
x every input mode of init_keys (random, byte_skip, ascending index;
include/rsort/detail/utils.cuh:245-317) x both orders x 14 sizes: three small
(1000, 100, 10) and 11 powers of two ending at the largest that fits the GPU.
Here the powers run 2^10 .. 2^20 so the oracle checks every one of the
13 x 6 x 3 x 2 x 14 = 6552 sorts exactly (the full-size configurations are
covered by the size-independent checks of the full-size tests).  byte_skip
keys keep every other digit constant, so they also run the uniform-pass skip
with odd and even numbers of executed passes.
"""

import os

import numpy as np
import pytest

from _oracle import KEY_TYPES, raw_keys, raw_values
from gpu_util import gpu_sort

pytestmark = pytest.mark.gpu

VALUE_KINDS = [0, 4, 1, 2, 8, 16]                        # none, u32, u8, u16, u64, u128
MODES = {"random": 4, "byte_skip": 5, "asc": 3}          # gbsort.gen distributions
SIZES = [1000, 100, 10] + [1 << i for i in range(10, 21)]
THREADS = max(1, min(16, os.cpu_count() or 1))


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("desc", [False, True], ids=["asc", "desc"])
@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("vb", VALUE_KINDS)
@pytest.mark.parametrize("kt", KEY_TYPES)
def test_validation_sweep(gb, cuda, oracle, kt, vb, mode, desc):
    failed = []
    for n in SIZES:
        seed = (n * 131 + vb * 7 + len(kt)) & 0xFFFFFFFF
        raw = raw_keys(kt, n, seed=seed, dist=MODES[mode])
        vals = raw_values(vb, n, seed=seed + 1)
        got = gpu_sort(gb, cuda, kt, raw, desc, vals)
        ref = oracle.sort(kt, raw, desc, vals, threads=THREADS if n > (1 << 16) else 1)
        if vals is None:
            ok = _eq(got, ref)
        else:
            ok = _eq(got[0], ref[0]) and _eq(got[1], ref[1])
        if not ok:
            failed.append(n)
    assert not failed, f"{kt} vb={vb} {mode} {'desc' if desc else 'asc'}: sizes {failed}"
