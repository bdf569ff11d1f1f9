"""bench.py's host-side helpers, without a GPU: the published baselines
restate the reference's own timings, each configuration names its metric,
the roofline peak comes from MEASURED_PEAKS.json, committed ncu traffic
scales to the workload, and the step statistics."""

import importlib.util
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_published_baselines_match_their_timings(bench):
    for name, (gkeys, note) in bench.PUBLISHED.items():
        ms = float(re.search(r"([0-9.]+) ms", note).group(1))
        n = bench.CONFIGS[name]["n"]
        assert gkeys == pytest.approx(n / (ms * 1e-3) / 1e9, rel=0.01), name


def test_configurations(bench):
    assert bench.CONFIGS["c2b"]["n"] == 1 << 28 and bench.CONFIGS["c2b"]["key"] == "u32"
    assert bench.CONFIGS["c1"]["n"] == 1 << 20
    assert bench.metric_of(bench.CONFIGS["c2b"]) == bench.PLAIN_METRIC
    assert bench.metric_of(bench.CONFIGS["c4"]) == bench.BATCHED_METRIC
    assert bench.metric_of(bench.CONFIGS["c5"]) == bench.SERVING_METRIC


def test_peak_is_the_measured_one(bench):
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if not os.path.exists(path):
        pytest.skip("no MEASURED_PEAKS.json")
    gbs, kind = bench.peaks()
    assert kind == "measured" and gbs > 1000


def test_committed_traffic_scales(bench):
    import json

    with open(os.path.join(REPO, "profiles", "ncu_traffic.json")) as f:
        table = json.load(f)
    for config, e in table.items():
        assert os.path.exists(os.path.join(REPO, e["summary"])), e["summary"]
        full = bench.CONFIGS[config]["n"] or 508761137  # the batched run: keys of the benchmark's segments
        traffic, src = bench.committed_traffic(config, full)
        assert traffic == int(e["dram_bytes_per_launch"] * full / e["captured_n"])
        assert e["summary"] in src
    assert bench.committed_traffic("c5", 1000) == (None, None)


def test_step_stats(bench):
    st = bench.step_stats([3.0, 1.0, 2.0])
    assert st == {"mean": 2.0, "std": round((2 / 3) ** 0.5, 4), "p50": 2.0, "p99": 3.0, "min": 1.0, "max": 3.0,
                  "n": 3}
