"""Device generators reproduce the host (numpy) streams bit for bit, and the
float distribution has the configured special values."""

import numpy as np
import pytest

from gbsort import gen
from gpu_util import from_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dist,kb", [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (3, 4), (3, 16),
                                     (4, 1), (4, 2), (4, 4), (4, 8), (4, 16), (5, 4), (5, 8), (5, 16)])
def test_device_generator_matches_numpy(gb, cuda, dist, kb):
    n = 100003
    seed = 12345
    d = cuda.empty(n * kb, dtype=cuda.uint8, device="cuda")
    gb.generate(dist, kb, d, n, seed)
    cuda.cuda.synchronize()
    ref = gen.generate(dist, kb, n, seed)
    assert np.array_equal(from_dev(d, ref), ref)


def test_float_distribution_specials(gb, cuda):
    n = 1 << 22
    d = cuda.empty(n, dtype=cuda.int32, device="cuda")
    gb.generate(1, 4, d, n, 7)
    bits = d.cpu().numpy().view(np.uint32)
    negz = np.count_nonzero(bits == 0x80000000) / n
    inf = np.count_nonzero((bits == 0x7F800000) | (bits == 0xFF800000)) / n
    nan = np.count_nonzero(bits == 0x7FC00000) / n
    assert 0.009 < negz < 0.011
    assert 0.0008 < inf < 0.0012
    assert 0.00005 < nan < 0.00015
    f = bits.view(np.float32)
    finite = f[np.isfinite(f) & (bits != 0x80000000)]
    assert abs(float(finite.mean())) < 0.01 and abs(float(finite.std()) - 1.0) < 0.01
