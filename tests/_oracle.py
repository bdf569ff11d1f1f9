"""ctypes binding of the CPU oracle (oracle/liboracle.so) for the tests.

Test infrastructure: the oracle is the checker, never the thing measured.
Keys are passed as raw-bit numpy arrays: uint8/16/32/64 for 1..8-byte keys,
(n, 16) uint8 for 16-byte keys.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
ORACLE_DIR = os.path.join(REPO, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")

KEY_TYPES = ["u8", "u16", "u32", "u64", "u128", "i8", "i16", "i32", "i64", "i128", "f32", "f64", "f128"]
KEY_ID = {k: i for i, k in enumerate(KEY_TYPES)}
KEY_BYTES = {"u8": 1, "u16": 2, "u32": 4, "u64": 8, "u128": 16, "i8": 1, "i16": 2, "i32": 4, "i64": 8,
             "i128": 16, "f32": 4, "f64": 8, "f128": 16}
RAW_DTYPE = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


class Oracle:
    def __init__(self, lib: ctypes.CDLL):
        self.lib = lib
        vp, sz, i = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
        lib.oracle_twiddle_in.argtypes = [i, i, vp, vp, sz]
        lib.oracle_twiddle_out.argtypes = [i, i, vp, vp, sz]
        lib.oracle_sort.argtypes = [i, i, vp, vp, sz, sz]
        lib.oracle_sort_parallel.argtypes = [i, i, vp, vp, sz, sz, i]
        lib.oracle_lsd_sort.argtypes = [i, i, vp, vp, sz, sz]
        lib.oracle_histogram.argtypes = [i, i, vp, sz, vp]
        for f in ("oracle_twiddle_in", "oracle_twiddle_out", "oracle_sort", "oracle_sort_parallel",
                  "oracle_lsd_sort", "oracle_histogram", "oracle_max_threads"):
            getattr(lib, f).restype = ctypes.c_int

    @staticmethod
    def _n(raw: np.ndarray) -> int:
        return raw.shape[0]

    def twiddle_in(self, kt: str, raw: np.ndarray, desc: bool) -> np.ndarray:
        out = np.empty_like(raw)
        assert self.lib.oracle_twiddle_in(KEY_ID[kt], int(desc), raw.ctypes.data, out.ctypes.data, self._n(raw)) == 0
        return out

    def twiddle_out(self, kt: str, bits: np.ndarray, desc: bool) -> np.ndarray:
        out = np.empty_like(bits)
        assert self.lib.oracle_twiddle_out(KEY_ID[kt], int(desc), bits.ctypes.data, out.ctypes.data,
                                           self._n(bits)) == 0
        return out

    def sort(self, kt: str, raw: np.ndarray, desc: bool = False, vals: np.ndarray | None = None,
             threads: int = 1, lsd: bool = False):
        k = np.ascontiguousarray(raw).copy()
        v = None if vals is None else np.ascontiguousarray(vals).copy()
        vb = 0 if v is None else v.dtype.itemsize * (v.shape[1] if v.ndim == 2 else 1)
        vptr = None if v is None else v.ctypes.data
        if lsd:
            rc = self.lib.oracle_lsd_sort(KEY_ID[kt], int(desc), k.ctypes.data, vptr, vb, self._n(k))
        elif threads > 1:
            rc = self.lib.oracle_sort_parallel(KEY_ID[kt], int(desc), k.ctypes.data, vptr, vb, self._n(k), threads)
        else:
            rc = self.lib.oracle_sort(KEY_ID[kt], int(desc), k.ctypes.data, vptr, vb, self._n(k))
        assert rc == 0
        return k if v is None else (k, v)

    def histogram(self, kt: str, raw: np.ndarray, desc: bool = False) -> np.ndarray:
        out = np.zeros(KEY_BYTES[kt] * 256, dtype=np.uint64)
        assert self.lib.oracle_histogram(KEY_ID[kt], int(desc), raw.ctypes.data, self._n(raw), out.ctypes.data) == 0
        return out.reshape(KEY_BYTES[kt], 256)

    def max_threads(self) -> int:
        return self.lib.oracle_max_threads()


_oracle = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "all"], check=True)
    return ORACLE_LIB


def load() -> Oracle:
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < os.path.getmtime(
                os.path.join(ORACLE_DIR, "oracle.cpp")):
            build()
        _oracle = Oracle(ctypes.CDLL(ORACLE_LIB))
    return _oracle


def raw_keys(kt: str, n: int, seed: int, dist: int = 0) -> np.ndarray:
    """Raw key bits of type kt from the shared generators."""
    from gbsort import gen

    return gen.generate(dist, KEY_BYTES[kt], n, seed)


def raw_values(value_bytes: int, n: int, seed: int) -> np.ndarray | None:
    """Values: index for 4/8-byte values (checks stability), random bits otherwise."""
    if value_bytes == 0:
        return None
    if value_bytes == 4:
        return np.arange(n, dtype=np.uint32)
    if value_bytes == 8:
        return np.arange(n, dtype=np.uint64)
    from gbsort import gen

    if value_bytes == 16:
        s = gen.splitmix64(seed ^ 0x77, 0, 2 * n)
        out = np.empty((n, 2), dtype=np.uint64)
        out[:, 0] = np.arange(n, dtype=np.uint64)
        out[:, 1] = s[1::2]
        return out.view(np.uint8).reshape(n, 16)
    return gen.splitmix64(seed ^ 0x77, 0, n).astype(RAW_DTYPE[value_bytes])
