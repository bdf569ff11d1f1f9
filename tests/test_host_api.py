"""Host-side parts of the C ABI that need no GPU: key sizes, the rsort
size-query protocol (workspace == NULL: bytes out, no device work), the
host-buffer sizing, status strings and argument checks."""

import ctypes

import pytest

KEY_BYTES = {"u8": 1, "u16": 2, "u32": 4, "u64": 8, "u128": 16, "i8": 1, "i16": 2, "i32": 4, "i64": 8,
             "i128": 16, "f32": 4, "f64": 8, "f128": 16}


def test_key_bytes(gb):
    l = gb.lib()
    for name, kb in KEY_BYTES.items():
        assert l.gbsort_key_bytes(gb.KEY_TYPES[name]) == kb
    assert l.gbsort_key_bytes(13) == 0 and l.gbsort_key_bytes(-1) == 0


@pytest.mark.parametrize("kt", ["u8", "u32", "u64", "u128", "f32"])
@pytest.mark.parametrize("vb", [0, 1, 4, 8, 16])
def test_size_query_protocol(gb, kt, vb):
    kb = KEY_BYTES[kt]
    prev = 0
    for n in (0, 1, 1000, 1 << 20, (1 << 22) + 1, 1 << 28):
        tb = gb.temp_bytes(kt, n, vb)
        # the workspace holds at least the alternate keys and values
        assert tb >= n * (kb + vb)
        assert tb >= prev
        prev = tb
        hb = gb.host_buffer_bytes(kt, n, vb)
        assert hb >= tb + n * (kb + vb)


def test_bad_arguments_rejected_without_device_work(gb):
    l = gb.lib()
    tb = ctypes.c_size_t(0)
    # unknown key type, bad value size, no temp_bytes pointer
    assert l.gbsort_sort_keys(99, 0, None, ctypes.byref(tb), None, 10, None) == gb.ERR_INVALID_ARGUMENT
    assert l.gbsort_sort_pairs(2, 0, None, None, 3, ctypes.byref(tb), None, 10, None) == gb.ERR_INVALID_ARGUMENT
    assert l.gbsort_sort_keys(2, 0, None, None, None, 10, None) == gb.ERR_INVALID_ARGUMENT
    # the copy forms follow the same size query
    f = l.gbsort_sort_keys_copy
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t),
                  ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    tb2 = ctypes.c_size_t(0)
    assert f(2, 0, None, None, ctypes.byref(tb2), None, 12345, None) == gb.OK
    assert tb2.value == gb.temp_bytes("u32", 12345)


def test_status_strings(gb):
    for st in range(9):
        assert gb.status_string(st) and gb.status_string(st) != "unknown status"
    assert gb.status_string(99) == "unknown status"


@pytest.mark.parametrize("kt,vb", [("u8", 0), ("u32", 0), ("u32", 4), ("u64", 8), ("u128", 16)])
def test_double_buffer_size_query(gb, kt, vb):
    """The DoubleBuffer workspace holds control words and status only."""
    kb = KEY_BYTES[kt]
    for n in (0, 1, 5000, 1 << 22, 1 << 28):
        db = gb.double_buffer_bytes(kt, n, vb)
        assert 0 < db <= gb.temp_bytes(kt, n, vb) - n * (kb + vb) + 512
        if n:
            assert db < gb.temp_bytes(kt, n, vb)
    if kt == "u32" and vb == 0:  # 2^28 keys: ~30 MB instead of ~1.1 GB
        assert gb.double_buffer_bytes(kt, 1 << 28) < 32 << 20


def test_double_buffer_rejects_bad_selector(gb):
    l = gb.lib()
    f = l.gbsort_sort_keys_double_buffer
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                  ctypes.POINTER(ctypes.c_size_t), ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    tb = ctypes.c_size_t(0)
    for bad in (2, -1):
        sel = ctypes.c_int(bad)
        assert f(2, 0, None, None, ctypes.byref(sel), ctypes.byref(tb), None, 10, None) == gb.ERR_INVALID_ARGUMENT
    assert f(2, 0, None, None, None, ctypes.byref(tb), None, 10, None) == gb.ERR_INVALID_ARGUMENT


def test_segmented_host_buffer_bytes(gb):
    """Host-memory batched sort: the keys and values once, plus one group's
    workspace; malformed offsets give 0 (and no device work)."""
    import numpy as np

    rng = np.random.default_rng(4)
    for kt, vb in (("u32", 4), ("u64", 0), ("u128", 16)):
        sizes = np.exp2(rng.uniform(8, 20, 300)).astype(np.uint64)
        off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
        n = int(off[-1])
        hb = gb.segmented_host_buffer_bytes(kt, off, vb)
        assert n * (KEY_BYTES[kt] + vb) < hb < 2 * n * (KEY_BYTES[kt] + vb)
    assert gb.segmented_host_buffer_bytes("u32", np.array([0, 10, 5], dtype=np.uint64)) == 0
    assert gb.segmented_host_buffer_bytes("u32", np.array([0], dtype=np.uint64)) > 0  # no segments


def test_buffer_addresses(gb):
    """Buffers may be raw addresses, torch tensors or contiguous numpy arrays."""
    import numpy as np

    a = np.zeros(16, np.uint32)
    assert gb._ptr(a) == a.ctypes.data
    assert gb._ptr(12345) == 12345 and gb._ptr(None) is None
    with pytest.raises(ValueError):
        gb._ptr(a[::2])
    with pytest.raises(TypeError):
        gb._ptr("not a buffer")
    torch = pytest.importorskip("torch")
    t = torch.zeros(4)
    assert gb._ptr(t) == t.data_ptr()
