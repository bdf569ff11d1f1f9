"""Seeded synthetic key generators (host side, numpy).

The same streams are produced on the device by ``gbsort_generate`` (see
``csrc/generate.cu``); tests check the two agree bit for bit for the integer
distributions.

Distributions (ids match ``gbsort_generate``):
  0  splitmix64 stream, full-range bits of the key width (16-byte keys take
     two consecutive stream values: low half = 2i, high half = 2i+1)
  1  float32 N(0,1) (Box-Muller) with 1% -0.0, 0.1% +/-inf, 0.01% quiet NaN
  2  uint64 keys whose upper 32 bits come from 256 distinct values and whose
     lower 32 bits are uniform (heavy duplicate prefixes)
  3  ascending: key i = i (truncated to the key width)
  4  rsort ``init_keys`` random mode: mix32 of (i ^ seed) per 32-bit word
     (include/rsort/detail/utils.cuh:245-290 of the reference)
  5  rsort ``init_keys`` byte_skip mode (utils.cuh:292-309)
"""

from __future__ import annotations

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)
DIST_SALT = np.uint64(0xD1B54A32D192ED03)
TABLE_SALT = np.uint64(0x5BD1E9955BD1E995)

DIST_SPLITMIX = 0
DIST_NORMAL_F32 = 1
DIST_DUP_PREFIX_U64 = 2
DIST_ASCENDING = 3
DIST_RSORT_RANDOM = 4
DIST_RSORT_BYTE_SKIP = 5

_WIDTH_DTYPE = {1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}


def _mix64(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * M1
    z = (z ^ (z >> np.uint64(27))) * M2
    return z ^ (z >> np.uint64(31))


def splitmix64(seed: int, start: int, count: int) -> np.ndarray:
    """Values start .. start+count-1 of the splitmix64 stream seeded with seed."""
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + count + 1, dtype=np.uint64)
        return _mix64(np.uint64(seed) + i * GOLDEN)


def mix32(x: np.ndarray) -> np.ndarray:
    """The reference's mix32 avalanche hash (utils.cuh:228-242)."""
    x = np.asarray(x, dtype=np.uint32).copy()
    with np.errstate(over="ignore"):
        x ^= x >> np.uint32(16)
        x *= np.uint32(0x7FEB352D)
        x ^= x >> np.uint32(15)
        x *= np.uint32(0x846CA68B)
        x ^= x >> np.uint32(16)
    return x


def _as_width(words64: np.ndarray, width: int) -> np.ndarray:
    if width == 16:
        raise ValueError("use _as_u128")
    return words64.astype(_WIDTH_DTYPE[width])


def _u128_from_halves(lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
    """16-byte little-endian keys as an (n, 16) uint8 array."""
    out = np.empty((lo.size, 2), dtype=np.uint64)
    out[:, 0] = lo
    out[:, 1] = hi
    return out.view(np.uint8).reshape(lo.size, 16)


def generate(dist: int, key_bytes: int, n: int, seed: int) -> np.ndarray:
    """Returns raw key bits: a uint{8,16,32,64} array, or (n,16) uint8 for 16 B."""
    if dist == DIST_SPLITMIX:
        if key_bytes == 16:
            s = splitmix64(seed, 0, 2 * n)
            return _u128_from_halves(s[0::2], s[1::2])
        return _as_width(splitmix64(seed, 0, n), key_bytes)
    if dist == DIST_NORMAL_F32:
        if key_bytes != 4:
            raise ValueError("normal_f32 is a 4-byte distribution")
        return normal_f32_bits(n, seed)
    if dist == DIST_DUP_PREFIX_U64:
        if key_bytes != 8:
            raise ValueError("dup_prefix_u64 is an 8-byte distribution")
        u = splitmix64(seed, 0, n)
        table = splitmix64(int(np.uint64(seed) ^ TABLE_SALT), 0, 256) & np.uint64(0xFFFFFFFF)
        upper = table[(u >> np.uint64(56)).astype(np.int64)]
        return (upper << np.uint64(32)) | (u & np.uint64(0xFFFFFFFF))
    if dist == DIST_ASCENDING:
        i = np.arange(n, dtype=np.uint64)
        if key_bytes == 16:
            return _u128_from_halves(i, np.zeros(n, dtype=np.uint64))
        return _as_width(i, key_bytes)
    if dist in (DIST_RSORT_RANDOM, DIST_RSORT_BYTE_SKIP):
        return rsort_init_keys(key_bytes, n, seed, byte_skip=(dist == DIST_RSORT_BYTE_SKIP))
    raise ValueError(f"unknown distribution {dist}")


def normal_f32_bits(n: int, seed: int) -> np.ndarray:
    u = splitmix64(seed, 0, n)
    r1 = ((u >> np.uint64(40)).astype(np.float64) + 1.0) / float(1 << 24)
    r2 = (u & np.uint64(0xFFFFFF)).astype(np.float64) / float(1 << 24)
    z = (np.sqrt(-2.0 * np.log(r1)) * np.cos(2.0 * np.pi * r2)).astype(np.float32)
    bits = z.view(np.uint32).copy()
    sel = splitmix64(int(np.uint64(seed) ^ DIST_SALT), 0, n) % np.uint64(10000)
    bits[sel < 100] = np.uint32(0x80000000)                       # 1% -0.0
    inf = (sel >= 100) & (sel < 110)                              # 0.1% +/-inf
    bits[inf & (sel % np.uint64(2) == 0)] = np.uint32(0x7F800000)
    bits[inf & (sel % np.uint64(2) == 1)] = np.uint32(0xFF800000)
    bits[(sel >= 110) & (sel < 111)] = np.uint32(0x7FC00000)      # 0.01% NaN
    return bits


def rsort_init_keys(key_bytes: int, n: int, seed: int, byte_skip: bool = False) -> np.ndarray:
    """Restates the reference's init_keys kernel (utils.cuh:245-317) per element."""
    i64 = np.arange(n, dtype=np.uint64)
    s = np.uint32(seed & 0xFFFFFFFF)
    with np.errstate(over="ignore"):
        if key_bytes <= 4:
            x = mix32((i64 ^ np.uint64(seed)).astype(np.uint32)).astype(np.uint64)
        elif key_bytes == 8:
            hi = (mix32((i64 + np.uint64(0x00000000)).astype(np.uint32)) ^ s).astype(np.uint64)
            lo = (mix32((i64 + np.uint64(0x9E3779B9)).astype(np.uint32)) ^ s).astype(np.uint64)
            x = (hi << np.uint64(32)) | lo
        else:
            w = [
                (mix32((i64 + np.uint64(c)).astype(np.uint32)) ^ s).astype(np.uint64)
                for c in (0x00000000, 0x9E3779B9, 0x3C6EF372, 0xDAA66D2B)
            ]
            hi = (w[0] << np.uint64(32)) | w[1]
            lo = (w[2] << np.uint64(32)) | w[3]
            if byte_skip:
                hi = (hi & np.uint64(0xFF00FF00FF00FF00)) | np.uint64(0x0055005500550055)
                lo = (lo & np.uint64(0xFF00FF00FF00FF00)) | np.uint64(0x0055005500550055)
            return _u128_from_halves(lo, hi)
        if byte_skip:
            x = (x & np.uint64(0xFF00FF00FF00FF00)) | np.uint64(0x0055005500550055)
    return _as_width(x, key_bytes)


def log_uniform_sizes(count: int, lo_log2: float, hi_log2: float, seed: int) -> np.ndarray:
    """Segment / request sizes drawn log-uniform in [2^lo, 2^hi] (seeded)."""
    u = splitmix64(seed, 0, count)
    f = (u >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    return np.floor(np.exp2(lo_log2 + f * (hi_log2 - lo_log2))).astype(np.int64)
