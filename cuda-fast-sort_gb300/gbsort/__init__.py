"""ctypes binding of libgbsort.so (the C ABI declared in include/gbsort.h).

This is a thin host-side mirror of rsort's entry points for Python callers
(tests, benchmark): ``sort`` / ``sort_descending`` / ``sort_pairs`` /
``sort_pairs_descending`` with rsort's size-query + workspace protocol
(reference include/rsort/rsort.cuh:13-92).  Device memory is handed in as raw
pointers (``int``) or as torch tensors (only their ``data_ptr()`` is used).

There is no fallback: if libgbsort.so is missing, importing the binding
raises ``GbsortUnavailable``; build it with ``python cuda-fast-sort_gb300/build.py``.
"""

from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# GBSORT_LIB selects another build of the same library (e.g. a tuning variant).
LIB_PATH = os.environ.get("GBSORT_LIB") or os.path.join(PKG_DIR, "lib", "libgbsort.so")

KEY_TYPES = {
    "u8": 0, "u16": 1, "u32": 2, "u64": 3, "u128": 4,
    "i8": 5, "i16": 6, "i32": 7, "i64": 8, "i128": 9,
    "f32": 10, "f64": 11, "f128": 12,
}
KEY_BYTES = {"u8": 1, "u16": 2, "u32": 4, "u64": 8, "u128": 16, "i8": 1, "i16": 2, "i32": 4,
             "i64": 8, "i128": 16, "f32": 4, "f64": 8, "f128": 16}
TYPED_NAMES = list(KEY_TYPES)

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_WORKSPACE_TOO_SMALL = 2
ERR_CUDA = 3
ERR_TIMEOUT = 4
ERR_UNSUPPORTED = 5
ERR_BUDGET = 6
ERR_NOT_READY = 7


class GbsortUnavailable(RuntimeError):
    pass


class GbsortError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = f"{what}: " if what else ""
        super().__init__(f"{msg}gbsort status {status} ({status_string(status)}) {last_error()}".strip())


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("passes", ctypes.c_uint32), ("radix_bits", ctypes.c_uint32), ("tile_items", ctypes.c_uint32),
        ("threads", ctypes.c_uint32), ("items_per_thread", ctypes.c_uint32), ("num_tiles", ctypes.c_uint32),
        ("pass_ctas", ctypes.c_uint32), ("hist_ctas", ctypes.c_uint32), ("status_word_bytes", ctypes.c_uint32),
        ("kernel_launches", ctypes.c_uint32), ("workspace_bytes", ctypes.c_uint64),
        ("msd_region_keys", ctypes.c_uint32), ("msd_stages", ctypes.c_uint32),
    ]


class SegmentedInfo(ctypes.Structure):
    _fields_ = [
        ("num_segments", ctypes.c_uint64), ("cta_small_segments", ctypes.c_uint64),
        ("cta_large_segments", ctypes.c_uint64), ("onesweep_segments", ctypes.c_uint64),
        ("onesweep_tiles", ctypes.c_uint64), ("keys_in_cta", ctypes.c_uint64),
        ("keys_in_onesweep", ctypes.c_uint64), ("cta_small_max", ctypes.c_uint32),
        ("cta_large_max", ctypes.c_uint32), ("onesweep_tile", ctypes.c_uint32), ("pad", ctypes.c_uint32),
        ("cta_small4_segments", ctypes.c_uint64), ("workspace_bytes", ctypes.c_uint64),
        ("kernel_launches", ctypes.c_uint64),
    ]


PATH_CTA_S, PATH_CTA_L, PATH_ONESWEEP, PATH_CTA_S4 = 0, 1, 2, 3

_lib = None


def _declare(lib: ctypes.CDLL) -> None:
    vp, sz, i, u64 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint64
    psz = ctypes.POINTER(ctypes.c_size_t)
    sig = {
        "gbsort_key_bytes": (sz, [i]),
        "gbsort_status_string": (ctypes.c_char_p, [i]),
        "gbsort_version": (ctypes.c_char_p, []),
        "gbsort_last_error": (ctypes.c_char_p, []),
        "gbsort_sort_keys": (i, [i, i, vp, psz, vp, sz, vp]),
        "gbsort_sort_pairs": (i, [i, i, vp, vp, sz, psz, vp, sz, vp]),
        "gbsort_host_buffer_bytes": (sz, [i, sz, sz]),
        "gbsort_sort_host": (i, [i, i, vp, vp, sz, sz, vp, sz, vp]),
        "gbsort_workspace_status": (i, [i, sz, sz, vp, vp]),
        "gbsort_set_wait_limit_ns": (None, [u64]),
        "gbsort_get_wait_limit_ns": (u64, []),
        "gbsort_probe_wait_timeout": (i, [vp, u64, vp]),
        "gbsort_probe_barrier_timeout": (i, [vp, u64, vp]),
        "gbsort_plan": (i, [i, sz, sz, ctypes.POINTER(PlanInfo)]),
        "gbsort_sort_timed": (i, [i, i, vp, vp, sz, vp, sz, sz, vp, ctypes.POINTER(ctypes.c_float), i,
                                  ctypes.POINTER(ctypes.c_int)]),
        "gbsort_generate": (i, [i, sz, vp, sz, u64, vp]),
        "gbsort_device_sm_count": (i, []),
    }
    pplan = ctypes.POINTER(ctypes.c_void_p)
    sig.update({
        "gbsort_segmented_plan_create": (i, [i, sz, i, ctypes.POINTER(ctypes.c_uint64), sz, pplan]),
        "gbsort_segmented_plan_destroy": (None, [vp]),
        "gbsort_segmented_plan_info": (i, [vp, ctypes.POINTER(SegmentedInfo)]),
        "gbsort_segmented_bind": (i, [vp, vp, vp, vp, sz, vp]),
        "gbsort_segmented_run": (i, [vp, i, vp]),
        "gbsort_segmented_status": (i, [vp, vp]),
        "gbsort_segmented_sort": (i, [i, i, vp, vp, sz, ctypes.POINTER(ctypes.c_uint64), sz, psz, vp, vp]),
        "gbsort_segmented_host_buffer_bytes": (sz, [i, sz, ctypes.POINTER(ctypes.c_uint64), sz]),
        "gbsort_segmented_sort_host": (i, [i, i, vp, vp, sz, ctypes.POINTER(ctypes.c_uint64), sz, vp, sz, vp]),
        "gbsort_set_segmented_path": (i, [i, sz, i, i]),
        "gbsort_get_segmented_path": (i, [i, sz, i]),
    })
    for name in TYPED_NAMES:
        sig[f"gbsort_sort_{name}"] = (i, [vp, psz, vp, sz, vp])
        sig[f"gbsort_sort_{name}_desc"] = (i, [vp, psz, vp, sz, vp])
        sig[f"gbsort_sort_pairs_{name}"] = (i, [vp, vp, sz, psz, vp, sz, vp])
        sig[f"gbsort_sort_pairs_{name}_desc"] = (i, [vp, vp, sz, psz, vp, sz, vp])
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args


def lib() -> ctypes.CDLL:
    """Loads libgbsort.so (once); raises GbsortUnavailable if it is not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise GbsortUnavailable(f"{LIB_PATH} is not built (run cuda-fast-sort_gb300/build.py)")
        l = ctypes.CDLL(LIB_PATH)
        _declare(l)
        _lib = l
    return _lib


def status_string(status: int) -> str:
    return lib().gbsort_status_string(status).decode()


def last_error() -> str:
    return lib().gbsort_last_error().decode()


def _ptr(x) -> int | None:
    """Address of a raw pointer (int), a torch tensor, or a C-contiguous
    numpy array (host memory for the host-buffer sorts)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if hasattr(x, "ctypes") and hasattr(x, "flags"):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("numpy arrays passed as buffers must be C-contiguous")
        return int(x.ctypes.data)
    raise TypeError(f"cannot take the address of {type(x).__name__}")


def _stream(s) -> int | None:
    if s is None:
        return None
    if isinstance(s, int):
        return s
    return int(s.cuda_stream)


def _check(status: int, what: str) -> None:
    if status != OK:
        raise GbsortError(status, what)


def key_type_id(key_type) -> int:
    return KEY_TYPES[key_type] if isinstance(key_type, str) else int(key_type)


def temp_bytes(key_type, n: int, value_bytes: int = 0) -> int:
    """rsort's size query: workspace bytes for (key type, value size, n)."""
    tb = ctypes.c_size_t(0)
    kt = key_type_id(key_type)
    if value_bytes:
        st = lib().gbsort_sort_pairs(kt, 0, None, None, value_bytes, ctypes.byref(tb), None, n, None)
    else:
        st = lib().gbsort_sort_keys(kt, 0, None, ctypes.byref(tb), None, n, None)
    _check(st, "size query")
    return tb.value


def sort(keys, n: int, key_type, workspace, workspace_bytes: int, *, values=None, value_bytes: int = 0,
         descending: bool = False, stream=None) -> None:
    """In-place device sort (keys-only if values is None).  Raises GbsortError."""
    kt = key_type_id(key_type)
    tb = ctypes.c_size_t(workspace_bytes)
    if values is None:
        st = lib().gbsort_sort_keys(kt, int(descending), _ptr(keys), ctypes.byref(tb), _ptr(workspace), n,
                                    _stream(stream))
    else:
        st = lib().gbsort_sort_pairs(kt, int(descending), _ptr(keys), _ptr(values), value_bytes, ctypes.byref(tb),
                                     _ptr(workspace), n, _stream(stream))
    _check(st, "sort")


def sort_timed(keys, n: int, key_type, workspace, workspace_bytes: int, *, values=None, value_bytes: int = 0,
               descending: bool = False, stream=None) -> list[float]:
    """Sort with a CUDA event around every kernel; returns per-kernel ms
    ([upsweep, pass 0, ..., pass P-1]).  Synchronizes the stream."""
    kt = key_type_id(key_type)
    ms = (ctypes.c_float * 32)()
    cnt = ctypes.c_int(0)
    st = lib().gbsort_sort_timed(kt, int(descending), _ptr(keys), _ptr(values), value_bytes if values is not None
                                 else 0, _ptr(workspace), workspace_bytes, n, _stream(stream), ms, 32,
                                 ctypes.byref(cnt))
    _check(st, "timed sort")
    return [ms[i] for i in range(cnt.value)]


def workspace_status(key_type, n: int, workspace, value_bytes: int = 0, stream=None) -> int:
    return lib().gbsort_workspace_status(key_type_id(key_type), value_bytes, n, _ptr(workspace), _stream(stream))


@dataclass
class Plan:
    passes: int
    radix_bits: int
    tile_items: int
    threads: int
    items_per_thread: int
    num_tiles: int
    pass_ctas: int
    hist_ctas: int
    status_word_bytes: int
    kernel_launches: int
    workspace_bytes: int
    msd_region_keys: int
    msd_stages: int


def plan(key_type, n: int, value_bytes: int = 0) -> Plan:
    info = PlanInfo()
    _check(lib().gbsort_plan(key_type_id(key_type), value_bytes, n, ctypes.byref(info)), "plan")
    return Plan(*(getattr(info, f) for f, _ in PlanInfo._fields_))


def generate(dist: int, key_bytes: int, out, n: int, seed: int, stream=None) -> None:
    _check(lib().gbsort_generate(dist, key_bytes, _ptr(out), n, seed, _stream(stream)), "generate")


def host_buffer_bytes(key_type, n: int, value_bytes: int = 0) -> int:
    return lib().gbsort_host_buffer_bytes(key_type_id(key_type), value_bytes, n)


def sort_host(h_keys, n: int, key_type, d_buffer, buffer_bytes: int, *, h_values=None, value_bytes: int = 0,
              descending: bool = False, stream=None) -> None:
    """Sorts host buffers (pointers or pinned torch tensors) through d_buffer."""
    st = lib().gbsort_sort_host(key_type_id(key_type), int(descending), _ptr(h_keys), _ptr(h_values),
                                value_bytes if h_values is not None else 0, n, _ptr(d_buffer), buffer_bytes,
                                _stream(stream))
    _check(st, "host sort")


def set_wait_limit_ns(ns: int) -> None:
    lib().gbsort_set_wait_limit_ns(ns)


def get_wait_limit_ns() -> int:
    return lib().gbsort_get_wait_limit_ns()


def probe_wait_timeout(scratch, limit_ns: int, stream=None) -> int:
    return lib().gbsort_probe_wait_timeout(_ptr(scratch), limit_ns, _stream(stream))


def probe_barrier_timeout(scratch, limit_ns: int, stream=None) -> int:
    return lib().gbsort_probe_barrier_timeout(_ptr(scratch), limit_ns, _stream(stream))


def sm_count() -> int:
    return lib().gbsort_device_sm_count()


# ---- batched (segmented) sort ---------------------------------------------

def _offsets_array(offsets):
    import numpy as np

    off = np.ascontiguousarray(np.asarray(offsets, dtype=np.uint64))
    return off, off.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))


class SegmentedPlan:
    """A batched sort of many independent segments (offsets on the host).
    bind() device buffers + workspace once, run() as often as needed (the
    first graph run captures a CUDA graph that later runs replay)."""

    def __init__(self, key_type, offsets, value_bytes: int = 0, descending: bool = False):
        self._off, ptr = _offsets_array(offsets)
        h = ctypes.c_void_p()
        _check(lib().gbsort_segmented_plan_create(key_type_id(key_type), value_bytes, int(descending), ptr,
                                                  len(self._off) - 1, ctypes.byref(h)), "segmented plan")
        self.handle = h
        self.key_type = key_type
        self.value_bytes = value_bytes

    def info(self) -> dict:
        inf = SegmentedInfo()
        _check(lib().gbsort_segmented_plan_info(self.handle, ctypes.byref(inf)), "segmented info")
        return {f: getattr(inf, f) for f, _ in SegmentedInfo._fields_ if f != "pad"}

    @property
    def workspace_bytes(self) -> int:
        return self.info()["workspace_bytes"]

    def bind(self, keys, workspace, workspace_bytes: int, values=None, stream=None) -> None:
        _check(lib().gbsort_segmented_bind(self.handle, _ptr(keys), _ptr(values), _ptr(workspace), workspace_bytes,
                                           _stream(stream)), "segmented bind")

    def run(self, stream=None, use_graph: bool = True) -> None:
        _check(lib().gbsort_segmented_run(self.handle, int(use_graph), _stream(stream)), "segmented run")

    def status(self, stream=None) -> int:
        return lib().gbsort_segmented_status(self.handle, _stream(stream))

    def close(self) -> None:
        if self.handle:
            lib().gbsort_segmented_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def segmented_sort(keys, key_type, offsets, workspace=None, workspace_bytes: int = 0, values=None,
                   value_bytes: int = 0, descending: bool = False, stream=None) -> int:
    """One-shot batched sort (rsort-style size query when workspace is None:
    returns the bytes needed)."""
    off, ptr = _offsets_array(offsets)
    tb = ctypes.c_size_t(workspace_bytes)
    st = lib().gbsort_segmented_sort(key_type_id(key_type), int(descending), _ptr(keys), _ptr(values), value_bytes,
                                     ptr, len(off) - 1, ctypes.byref(tb), _ptr(workspace), _stream(stream))
    _check(st, "segmented sort")
    return tb.value


def segmented_host_buffer_bytes(key_type, offsets, value_bytes: int = 0) -> int:
    off, ptr = _offsets_array(offsets)
    return lib().gbsort_segmented_host_buffer_bytes(key_type_id(key_type), value_bytes, ptr, len(off) - 1)


def segmented_sort_host(h_keys, key_type, offsets, d_buffer, buffer_bytes: int, *, h_values=None,
                        value_bytes: int = 0, descending: bool = False, stream=None) -> None:
    """Batched sort of host-resident segments (pointers or pinned tensors),
    copies overlapped with the sorting, through d_buffer."""
    off, ptr = _offsets_array(offsets)
    st = lib().gbsort_segmented_sort_host(key_type_id(key_type), int(descending), _ptr(h_keys), _ptr(h_values),
                                          value_bytes if h_values is not None else 0, ptr, len(off) - 1,
                                          _ptr(d_buffer), buffer_bytes, _stream(stream))
    _check(st, "batched host sort")


def set_segmented_path(key_type, value_bytes: int, size_log2: int, path: int) -> None:
    _check(lib().gbsort_set_segmented_path(key_type_id(key_type), value_bytes, size_log2, path), "tuning")


def get_segmented_path(key_type, value_bytes: int, size_log2: int) -> int:
    return lib().gbsort_get_segmented_path(key_type_id(key_type), value_bytes, size_log2)


def autotune_segmented(key_type, value_bytes: int, scratch, scratch_bytes: int, min_log2: int = 4,
                       max_log2: int = 20, descending: bool = False, stream=None) -> str:
    """Runs the batched sort's autotuner (installs the winners) and returns
    its per-bucket report."""
    f = lib().gbsort_autotune_segmented
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_size_t, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    buf = ctypes.create_string_buffer(1 << 16)
    _check(f(key_type_id(key_type), value_bytes, int(descending), min_log2, max_log2, _ptr(scratch), scratch_bytes,
             _stream(stream), buf, len(buf)), "autotune")
    return buf.value.decode()


def segmented_tuning_text() -> str:
    f = lib().gbsort_segmented_tuning_text
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
    buf = ctypes.create_string_buffer(1 << 16)
    f(buf, len(buf))
    return buf.value.decode()


def segmented_tuning_load(text: str) -> None:
    f = lib().gbsort_segmented_tuning_load
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p]
    _check(f(text.encode()), "tuning load")


# ---- sort server (continuous batching) --------------------------------------

class ServerConfig(ctypes.Structure):
    _fields_ = [("pool_bytes", ctypes.c_uint64), ("streams", ctypes.c_uint32), ("paused", ctypes.c_uint32),
                ("max_batch_keys", ctypes.c_uint64), ("max_batch_requests", ctypes.c_uint64)]


class Request(ctypes.Structure):
    _fields_ = [("key_type", ctypes.c_int), ("descending", ctypes.c_int), ("value_bytes", ctypes.c_size_t),
                ("n", ctypes.c_size_t), ("keys_in", ctypes.c_void_p), ("values_in", ctypes.c_void_p),
                ("keys_out", ctypes.c_void_p), ("values_out", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [(f, ctypes.c_uint64) for f in ("submitted", "completed", "failed", "rejected", "batches",
                                               "max_batch_requests", "keys_sorted", "bytes_sorted", "pool_bytes",
                                               "pool_peak_bytes", "kernel_launches")] + \
               [(f, ctypes.c_double) for f in ("latency_p50_us", "latency_p99_us", "latency_mean_us",
                                               "latency_max_us", "queue_p50_us", "queue_p99_us",
                                               "mean_batch_requests", "active_seconds", "host_plan_seconds",
                                               "host_launch_seconds", "batch_seconds", "h2d_seconds",
                                               "sort_seconds", "d2h_seconds")]


def _declare_server(l) -> None:
    vp, i, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64
    sig = {
        "gbsort_server_create": (i, [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]),
        "gbsort_server_destroy": (None, [vp]),
        "gbsort_server_submit": (i, [vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
        "gbsort_server_poll": (i, [vp, u64]),
        "gbsort_server_wait": (i, [vp, u64, u64]),
        "gbsort_server_drain": (i, [vp, u64]),
        "gbsort_server_pause": (i, [vp]),
        "gbsort_server_resume": (i, [vp]),
        "gbsort_server_stats_get": (i, [vp, ctypes.POINTER(ServerStats)]),
        "gbsort_server_stats_reset": (i, [vp]),
        "gbsort_workspace_reset": (i, [i, ctypes.c_size_t, ctypes.c_size_t, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(l, name)
        f.restype = res
        f.argtypes = args


class Server:
    """Continuous-batching sort server (gbsort_server_*): submit requests
    from host or device buffers, poll/wait per ticket; queued requests of one
    class are coalesced into batched sorts, admitted by bytes against a
    pooled device allocation, with several batches in flight."""

    def __init__(self, pool_bytes: int = 0, streams: int = 0, paused: bool = False, max_batch_keys: int = 0,
                 max_batch_requests: int = 0):
        _declare_server(lib())
        cfg = ServerConfig(pool_bytes, streams, int(paused), max_batch_keys, max_batch_requests)
        h = ctypes.c_void_p()
        _check(lib().gbsort_server_create(ctypes.byref(cfg), ctypes.byref(h)), "server create")
        self.handle = h

    def submit(self, key_type, n: int, keys_in, keys_out=None, values_in=None, values_out=None,
               value_bytes: int = 0, descending: bool = False) -> int:
        """Pointers are ints or tensors (host or device); keys_out defaults
        to keys_in (in place).  Returns the ticket."""
        keys_out = keys_in if keys_out is None else keys_out
        values_out = values_in if values_out is None else values_out
        r = Request(key_type_id(key_type), int(descending), value_bytes, n, _ptr(keys_in), _ptr(values_in),
                    _ptr(keys_out), _ptr(values_out))
        t = ctypes.c_uint64()
        _check(lib().gbsort_server_submit(self.handle, ctypes.byref(r), ctypes.byref(t)), "server submit")
        return t.value

    def try_submit(self, *args, **kw):
        """As submit, but returns (status, ticket) instead of raising."""
        try:
            return OK, self.submit(*args, **kw)
        except GbsortError as e:
            return e.status, None

    def poll(self, ticket: int) -> int:
        return lib().gbsort_server_poll(self.handle, ticket)

    def wait(self, ticket: int, timeout_s: float = 60.0) -> int:
        return lib().gbsort_server_wait(self.handle, ticket, int(timeout_s * 1e9))

    def drain(self, timeout_s: float = 600.0) -> int:
        return lib().gbsort_server_drain(self.handle, int(timeout_s * 1e9))

    def pause(self) -> None:
        _check(lib().gbsort_server_pause(self.handle), "server pause")

    def resume(self) -> None:
        _check(lib().gbsort_server_resume(self.handle), "server resume")

    def stats(self) -> dict:
        s = ServerStats()
        _check(lib().gbsort_server_stats_get(self.handle, ctypes.byref(s)), "server stats")
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}

    def reset_stats(self) -> None:
        _check(lib().gbsort_server_stats_reset(self.handle), "server stats reset")

    def close(self) -> None:
        if self.handle:
            lib().gbsort_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def workspace_reset(key_type, n: int, workspace, value_bytes: int = 0, stream=None) -> None:
    _declare_server(lib())
    _check(lib().gbsort_workspace_reset(key_type_id(key_type), value_bytes, n, _ptr(workspace), _stream(stream)),
           "workspace reset")


# ---- multi-GPU sharding (host only) -----------------------------------------

def partition_weights(weights, world: int):
    """Bytes-balanced owner rank of every item (gbsort_partition_weights);
    returns (owner int32 array, per-rank load uint64 array)."""
    import numpy as np

    w = np.ascontiguousarray(np.asarray(weights, dtype=np.uint64))
    owner = np.empty(len(w), dtype=np.int32)
    load = np.zeros(max(1, world), dtype=np.uint64)
    f = lib().gbsort_partition_weights
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    _check(f(w.ctypes.data, len(w), world, owner.ctypes.data, load.ctypes.data), "partition")
    return owner, load[:world]


def partition_segments(offsets, world: int, key_bytes: int, value_bytes: int = 0):
    """Owner rank of every segment of a batched sort, balanced by bytes."""
    import numpy as np

    off, _ = _offsets_array(offsets)
    owner = np.empty(max(0, len(off) - 1), dtype=np.int32)
    load = np.zeros(max(1, world), dtype=np.uint64)
    f = lib().gbsort_partition_segments
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t,
                  ctypes.c_void_p, ctypes.c_void_p]
    _check(f(off.ctypes.data, len(owner), world, key_bytes, value_bytes, owner.ctypes.data, load.ctypes.data),
           "partition")
    return owner, load[:world]


def shard_offsets(offsets, owner, rank: int):
    """Offsets of the compacted batch holding only `rank`'s segments (in
    their original order) and the indices of those segments."""
    import numpy as np

    off = np.asarray(offsets, dtype=np.uint64)
    mine = np.nonzero(np.asarray(owner) == rank)[0]
    sizes = (off[1:] - off[:-1])[mine]
    return np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64), mine


def set_pass_skip(enable: bool) -> None:
    """Uniform-digit pass skipping on or off (process-wide; default on)."""
    f = lib().gbsort_set_pass_skip
    f.restype = None
    f.argtypes = [ctypes.c_int]
    f(int(enable))


def get_pass_skip() -> bool:
    f = lib().gbsort_get_pass_skip
    f.restype = ctypes.c_int
    return bool(f())


def set_short_fused(enable: bool) -> None:
    """One-launch sort of short keys-only arrays on (default) or off."""
    f = lib().gbsort_set_short_fused
    f.restype = None
    f.argtypes = [ctypes.c_int]
    f(int(enable))


def get_short_fused() -> bool:
    f = lib().gbsort_get_short_fused
    f.restype = ctypes.c_int
    return bool(f())


def set_short_msd(enable: bool) -> None:
    """MSD partition + per-CTA bucket sorts inside the one-launch short sort."""
    f = lib().gbsort_set_short_msd
    f.restype = None
    f.argtypes = [ctypes.c_int]
    f(int(enable))


def get_short_msd() -> bool:
    f = lib().gbsort_get_short_msd
    f.restype = ctypes.c_int
    return bool(f())


def set_msd(enable: bool) -> None:
    """Most-significant-digit-first path of large keys-only sorts of 8- and
    16-byte keys on (default) or off."""
    f = lib().gbsort_set_msd
    f.restype = None
    f.argtypes = [ctypes.c_int]
    f(int(enable))


def get_msd() -> bool:
    f = lib().gbsort_get_msd
    f.restype = ctypes.c_int
    return bool(f())


def sort_copy(keys_in, keys_out, n: int, key_type, workspace, workspace_bytes: int, *, values_in=None,
              values_out=None, value_bytes: int = 0, descending: bool = False, stream=None) -> None:
    """Input-preserving sort (gbsort_sort_keys_copy / gbsort_sort_pairs_copy):
    reads keys_in (values_in), writes the sorted result to keys_out
    (values_out)."""
    l = lib()
    vp, sz, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    tb = ctypes.c_size_t(workspace_bytes)
    kt = key_type_id(key_type)
    if value_bytes:
        f = l.gbsort_sort_pairs_copy
        f.restype = i
        f.argtypes = [i, i, vp, vp, vp, vp, sz, ctypes.POINTER(ctypes.c_size_t), vp, sz, vp]
        st = f(kt, int(descending), _ptr(keys_in), _ptr(keys_out), _ptr(values_in), _ptr(values_out), value_bytes,
               ctypes.byref(tb), _ptr(workspace), n, _stream(stream))
    else:
        f = l.gbsort_sort_keys_copy
        f.restype = i
        f.argtypes = [i, i, vp, vp, ctypes.POINTER(ctypes.c_size_t), vp, sz, vp]
        st = f(kt, int(descending), _ptr(keys_in), _ptr(keys_out), ctypes.byref(tb), _ptr(workspace), n,
               _stream(stream))
    _check(st, "sort copy")


def _double_buffer_fn(value_bytes: int):
    l = lib()
    vp, sz, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
    ip, tp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_size_t)
    if value_bytes:
        f = l.gbsort_sort_pairs_double_buffer
        f.argtypes = [i, i, vp, vp, vp, vp, sz, ip, tp, vp, sz, vp]
    else:
        f = l.gbsort_sort_keys_double_buffer
        f.argtypes = [i, i, vp, vp, ip, tp, vp, sz, vp]
    f.restype = i
    return f


def double_buffer_bytes(key_type, n: int, value_bytes: int = 0) -> int:
    """Workspace bytes of the DoubleBuffer form (control words and status only)."""
    f = _double_buffer_fn(value_bytes)
    tb = ctypes.c_size_t(0)
    sel = ctypes.c_int(0)
    args = [key_type_id(key_type), 0, None, None] + ([None, None, value_bytes] if value_bytes else [])
    _check(f(*args, ctypes.byref(sel), ctypes.byref(tb), None, n, None), "size query")
    return tb.value


def sort_double_buffer(keys0, keys1, n: int, key_type, workspace, workspace_bytes: int, *, selector: int = 0,
                       values0=None, values1=None, value_bytes: int = 0, descending: bool = False,
                       stream=None) -> int:
    """DoubleBuffer sort (gbsort_sort_keys/pairs_double_buffer): the input is
    in buffer `selector` (0: keys0/values0, 1: keys1/values1); returns the
    selector of the buffer holding the result."""
    f = _double_buffer_fn(value_bytes)
    tb = ctypes.c_size_t(workspace_bytes)
    sel = ctypes.c_int(selector)
    vals = [_ptr(values0), _ptr(values1), value_bytes] if value_bytes else []
    st = f(key_type_id(key_type), int(descending), _ptr(keys0), _ptr(keys1), *vals, ctypes.byref(sel),
           ctypes.byref(tb), _ptr(workspace), n, _stream(stream))
    _check(st, "double-buffer sort")
    return sel.value


def double_buffer_status(key_type, n: int, workspace, value_bytes: int = 0, stream=None) -> int:
    """gbsort_double_buffer_status: syncs `stream`, returns the last DoubleBuffer sort's status."""
    f = lib().gbsort_double_buffer_status
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    return f(key_type_id(key_type), value_bytes, n, _ptr(workspace), _stream(stream))


# ---- device-side result checks ------------------------------------------------

def check_order(keys, n: int, key_type, descending: bool = False, stream=None) -> int:
    """Adjacent pairs out of order (0 for a sorted array)."""
    f = lib().gbsort_check_order
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_uint64)]
    out = ctypes.c_uint64(0)
    _check(f(key_type_id(key_type), int(descending), _ptr(keys), n, _stream(stream), ctypes.byref(out)), "order")
    return out.value


def checksum(keys, n: int, key_type, stream=None) -> int:
    """Order-independent checksum of the keys (equal for any permutation)."""
    f = lib().gbsort_checksum
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
    out = ctypes.c_uint64(0)
    _check(f(key_type_id(key_type), _ptr(keys), n, _stream(stream), ctypes.byref(out)), "checksum")
    return out.value


def check_pairs(keys_in, keys_out, index_values, value_bytes: int, n: int, key_type, stream=None) -> int:
    """Output positions whose index value does not point at an equal input key."""
    f = lib().gbsort_check_pairs
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                  ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
    out = ctypes.c_uint64(0)
    _check(f(key_type_id(key_type), _ptr(keys_in), _ptr(keys_out), _ptr(index_values), value_bytes, n,
             _stream(stream), ctypes.byref(out)), "pairs")
    return out.value


def set_graph_cache(enable: bool) -> None:
    """Graph replay of repeated identical calls on/off (default on)."""
    f = lib().gbsort_set_graph_cache
    f.restype = None
    f.argtypes = [ctypes.c_int]
    f(int(enable))


def get_graph_cache() -> bool:
    f = lib().gbsort_get_graph_cache
    f.restype = ctypes.c_int
    return bool(f())


def graph_cache_clear() -> None:
    f = lib().gbsort_graph_cache_clear
    f.restype = ctypes.c_int
    _check(f(), "graph cache clear")


def graph_cache_stats() -> dict:
    """Tracked calls, those holding a graph, graphs captured and replays since load."""
    f = lib().gbsort_graph_cache_stats
    f.restype = None
    f.argtypes = [ctypes.POINTER(ctypes.c_uint64)] * 4
    v = [ctypes.c_uint64(0) for _ in range(4)]
    f(*[ctypes.byref(x) for x in v])
    return dict(zip(("calls", "graphs", "captures", "replays"), (x.value for x in v)))
