"""Device-side result checks (order, permutation checksum, index pairs) and
the benchmark CLI built on them (reference options, statistics block,
validation sweep, plotting dump)."""

import os
import subprocess
import sys

import numpy as np
import pytest

from _oracle import raw_keys
from gpu_util import to_dev

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "cuda-fast-sort_gb300")


@pytest.mark.parametrize("kt", ["u8", "i16", "u32", "f32", "i64", "f64", "u128", "f128"])
def test_checks_accept_sorted_and_catch_faults(gb, cuda, oracle, kt):
    n = 5000
    raw = raw_keys(kt, n, seed=3, dist=4)
    for desc in (False, True):
        srt = oracle.sort(kt, raw, desc)
        d_src, d_srt = to_dev(cuda, raw), to_dev(cuda, srt)
        assert gb.check_order(d_srt, n, kt, desc) == 0
        assert gb.check_order(d_src, n, kt, desc) > 0           # random input is out of order
        assert gb.checksum(d_srt, n, kt) == gb.checksum(d_src, n, kt)
        bad = srt.copy()
        bad[10] = bad[11]                                      # not a permutation any more
        if not np.array_equal(bad.view(np.uint8), srt.view(np.uint8)):
            assert gb.checksum(to_dev(cuda, bad), n, kt) != gb.checksum(d_src, n, kt)
    # pairs: values = original index
    keys, idx = oracle.sort(kt, raw, False, np.arange(n, dtype=np.uint32))
    d_in, d_out, d_idx = to_dev(cuda, raw), to_dev(cuda, keys), to_dev(cuda, idx)
    assert gb.check_pairs(d_in, d_out, d_idx, 4, n, kt) == 0
    idx2 = idx.copy()
    idx2[[0, 1]] = idx2[[1, 0]]
    i0, i1 = int(idx2[0]), int(idx2[1])
    same = np.array_equal(raw[i0:i0 + 1].view(np.uint8), raw[i1:i1 + 1].view(np.uint8))
    assert gb.check_pairs(d_in, d_out, to_dev(cuda, idx2), 4, n, kt) == (0 if same else 2)


def _cli(*args):
    env = dict(os.environ, PYTHONPATH=PKG + os.pathsep + os.environ.get("PYTHONPATH", ""))
    return subprocess.run([sys.executable, "-m", "gbsort.cli", *args], capture_output=True, text=True, env=env,
                          timeout=900)


def test_cli_benchmark_block():
    r = _cli("--n", "1000000", "--iterations", "3", "--warmup", "1", "--warmup_ms", "0", "--type", "float",
             "--values", "uint32_t", "--descending")
    assert r.returncode == 0, r.stdout + r.stderr
    for field in ("RADIX", "N\t=\t1000000", "Type\t=\tfloat", "Time\t=", "it/s", "ps/el", "Order\t=\tDESC",
                  "Pairs\t=\tuint32_t", "Post sort checks [order, hist, pair]: [1, 1, 1]"):
        assert field in r.stdout, field


def test_cli_scaling_dump(tmp_path):
    out = tmp_path / "benchmark_data.py"
    r = _cli("--scaling", "16:18", "--dump", str(out), "--iterations", "2", "--warmup", "1", "--warmup_ms", "0")
    assert r.returncode == 0, r.stdout + r.stderr
    ns = {}
    exec(out.read_text(), ns)
    assert set(ns["scaling_avg"]["uint32_t"]) == {16, 17, 18}
    assert all(len(v) == 1 and v[0] > 0 for v in ns["scaling_avg"]["uint32_t"].values())
    assert set(ns["scaling_std"]["uint32_t"]) == {16, 17, 18}


def test_cli_validation_sweep_small():
    r = _cli("--validation", "--iterations", "1", "--warmup", "0", "--max_log2", "11")
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "Done... passed 6552/6552 tests." in r.stdout
