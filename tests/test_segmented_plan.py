"""Host-side planning of the batched sort (no GPU needed): segment
classification by size bucket, the tuning table, tile tables, workspace."""

import numpy as np
import pytest


def _plan(gb, kt, sizes, vb=0):
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    return gb.SegmentedPlan(kt, off, vb)


def test_classification_by_size(gb):
    p = _plan(gb, "u32", [0, 1, 2, 100, 2048, 2049, 8192, 8193, 100000], vb=4)
    inf = p.info()
    assert inf["num_segments"] == 9
    assert inf["cta_small_max"] == 2048 and inf["cta_large_max"] == 8192
    assert inf["cta_small_segments"] == 3      # 2, 100, 2048 (0 and 1 are already sorted)
    assert inf["cta_large_segments"] == 2      # 2049, 8192
    assert inf["onesweep_segments"] == 2       # 8193, 100000
    tile = inf["onesweep_tile"]
    assert inf["onesweep_tiles"] == -(-8193 // tile) + -(-100000 // tile)
    assert inf["keys_in_cta"] == 2 + 100 + 2048 + 2049 + 8192
    assert inf["keys_in_onesweep"] == 8193 + 100000
    assert inf["workspace_bytes"] > 0


def test_tuning_table_routes_buckets(gb):
    try:
        gb.set_segmented_path("u64", 8, -1, gb.PATH_ONESWEEP)
        assert all(gb.get_segmented_path("u64", 8, b) == gb.PATH_ONESWEEP for b in range(0, 30))
        gb.set_segmented_path("u64", 8, 10, gb.PATH_CTA_S)
        assert gb.get_segmented_path("u64", 8, 10) == gb.PATH_CTA_S
        # a path too small for the bucket falls through to a bigger one
        gb.set_segmented_path("u64", 8, 20, gb.PATH_CTA_S)
        assert gb.get_segmented_path("u64", 8, 20) == gb.PATH_ONESWEEP
        p = _plan(gb, "u64", [1000, 1500, 3000], vb=8)  # buckets 9, 10, 11
        inf = p.info()
        assert inf["cta_small_segments"] == 1 and inf["onesweep_segments"] == 2
    finally:
        gb.set_segmented_path("u64", 8, -1, -1)
    assert gb.get_segmented_path("u64", 8, 4) == gb.PATH_CTA_S


def test_invalid_offsets_rejected(gb):
    with pytest.raises(gb.GbsortError):
        gb.SegmentedPlan("u32", np.array([0, 10, 5], dtype=np.uint64))
    with pytest.raises(gb.GbsortError):
        gb.SegmentedPlan("u32", np.array([0, 1 << 33], dtype=np.uint64))


def test_workspace_query_without_device(gb):
    off = np.array([0, 1000, 50000, 51000], dtype=np.uint64)
    assert gb.segmented_sort(None, "f32", off, values=None) > 0
