"""libgbsort.so loads, exports every symbol include/gbsort.h declares, and its
host-only logic (size query, plan, argument checks) works without a GPU."""

import os
import re
import subprocess

import pytest

from _oracle import KEY_BYTES

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "gbsort.h")


def declared_functions():
    src = open(HEADER).read()
    names = set(re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(gbsort_\w+)\s*\(", src, flags=re.M))
    typed = re.findall(r"^GBSORT_DECLARE_TYPED\((\w+)\)", src, flags=re.M)
    for t in typed:
        names |= {f"gbsort_sort_{t}", f"gbsort_sort_{t}_desc", f"gbsort_sort_pairs_{t}",
                  f"gbsort_sort_pairs_{t}_desc"}
    names.discard("gbsort_sort_")
    return sorted(n for n in names if not n.endswith("_"))


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_library_exports_every_declared_symbol(gb):
    decl = declared_functions()
    assert len(decl) >= 60, decl
    missing = [d for d in decl if d not in exported_symbols(gb.LIB_PATH)]
    assert not missing, missing


def test_library_loads_and_reports_version(gb):
    assert "sm_103a" in gb.lib().gbsort_version().decode()


def test_size_query_needs_no_device(gb):
    # rsort protocol: workspace == NULL -> bytes written, no device work.
    n = 1 << 20
    tb = gb.temp_bytes("u32", n)
    assert tb >= n * 4
    assert gb.temp_bytes("u32", n, value_bytes=4) >= n * 8
    assert gb.temp_bytes("u128", n) >= n * 16
    # larger n never needs less
    for kt in gb.KEY_TYPES:
        prev = 0
        for n in (0, 1, 100, 8191, 8192, 8193, 1 << 20):
            b = gb.temp_bytes(kt, n)
            assert b >= prev
            prev = b


def test_size_query_reserves_the_msd_blocks(gb):
    """The size query holds room for the path a keys-only sort may take,
    whether or not it is switched on: the one-launch sort's top-digit regions
    (short arrays) and the MSD block of large 8- and 16-byte keys (state,
    claim counters, 65536 group sizes, claims and offsets)."""
    msd_block = 256 + 256 * 4 + 3 * 65536 * 4

    def beyond_buffers(kt, n):  # bytes past the alternate keys and the lookback status
        p = gb.plan(kt, n)
        return gb.temp_bytes(kt, n) - n * KEY_BYTES[kt] - p.num_tiles * 256 * p.status_word_bytes

    for kt, n in (("u64", 1 << 25), ("f128", 1 << 23), ("u128", 1 << 27)):
        assert beyond_buffers(kt, n) >= msd_block
    # 4-byte keys, pairs and sizes outside the range carry no MSD block
    for kt, n in (("u32", 1 << 25), ("u64", 1 << 24), ("u128", (1 << 27) + 1)):
        assert beyond_buffers(kt, n) < 64 << 10
    # short keys-only arrays: the regions hold every key with a margin
    n = 1 << 20
    assert gb.temp_bytes("u32", n) >= 2 * n * 4


def test_msd_planning_needs_no_device(gb):
    """Which keys-only sorts go most significant digit first (host logic):
    8-byte keys from 1.5 x 2^24 to 2^28, 16-byte keys from 1.5 x 2^20 to
    2^27, never pairs or narrower keys; the switch changes the plan, not the
    size query."""
    assert gb.get_msd()
    for kt, n, want in (("u64", 3 << 23, 6), ("i64", 1 << 28, 6), ("f64", (3 << 23) - 1, 0),
                        ("u64", (1 << 28) + 1, 0), ("u128", 3 << 19, 6), ("f128", 1 << 27, 6),
                        ("i128", (3 << 19) - 1, 0), ("u128", (1 << 27) + 1, 0), ("u32", 1 << 26, 0),
                        ("u16", 1 << 26, 0)):
        assert gb.plan(kt, n).msd_stages == want, (kt, n)
    assert gb.plan("u64", 1 << 26, 8).msd_stages == 0
    tb = gb.temp_bytes("u128", 1 << 24)
    gb.set_msd(False)
    try:
        assert gb.plan("u128", 1 << 24).msd_stages == 0
        assert gb.temp_bytes("u128", 1 << 24) == tb
    finally:
        gb.set_msd(True)


def test_plan_reports_geometry(gb):
    p = gb.plan("u32", 1 << 28)
    assert p.passes == 4 and p.radix_bits == 8
    assert p.num_tiles == -(-(1 << 28) // p.tile_items)
    assert p.status_word_bytes == 4  # 2^28 fits the 32-bit epoch-tagged words
    assert gb.plan("u32", (1 << 28) + 1).status_word_bytes == 8
    assert gb.plan("u128", 1 << 26).passes == 16


def test_invalid_arguments_are_rejected(gb):
    import ctypes

    tb = ctypes.c_size_t(0)
    lib = gb.lib()
    assert lib.gbsort_sort_keys(99, 0, None, ctypes.byref(tb), None, 10, None) == gb.ERR_INVALID_ARGUMENT
    assert lib.gbsort_sort_pairs(2, 0, None, None, 3, ctypes.byref(tb), None, 10, None) == gb.ERR_INVALID_ARGUMENT
    assert lib.gbsort_sort_keys(2, 0, None, None, None, 10, None) == gb.ERR_INVALID_ARGUMENT
    # workspace smaller than required is refused before any device work
    tb.value = 16
    assert lib.gbsort_sort_keys(2, 0, 4096, ctypes.byref(tb), 8192, 1000, None) == gb.ERR_WORKSPACE_TOO_SMALL
    # n == 0 is a no-op (rsort underflows there)
    tb.value = 0
    assert lib.gbsort_sort_keys(2, 0, 4096, ctypes.byref(tb), 8192, 0, None) == gb.OK


def test_no_device_fails_loudly(gb):
    """Without a GB300 a sort returns an error instead of running anywhere else."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import ctypes

    n = 1000
    tb = ctypes.c_size_t(gb.temp_bytes("u32", n))
    st = gb.lib().gbsort_sort_keys(2, 0, 4096, ctypes.byref(tb), 8192, n, None)
    assert st == gb.ERR_UNSUPPORTED


def test_status_strings(gb):
    for s in range(9):
        assert gb.status_string(s)
