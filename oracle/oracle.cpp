/*
 * oracle.cpp — CPU oracle for the onesweep LSD radix sort.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load this library, and only to check or to
 * time the CPU side.  The product path (libgbsort.so) never links, loads or
 * calls it.
 *
 * What it restates (AwardOfSky/CUDA-Fast-Sort "rsort" v0.4.0):
 *   - key twiddle in/out: include/rsort/detail/tuning.cuh:352-384
 *     floats (and long double, sign at bit 127): neg ? ~b : b ^ sign;
 *     signed integers: b ^ sign; descending: ~b after that.
 *   - tail filler / digit extraction: tuning.cuh:388-396 (digit = (u >> 8p) & 0xFF)
 *   - long double handled as a raw unsigned __int128: radix_kernel.cuh:351-356
 *   - the sort itself: an LSD radix sort with one stable counting pass per
 *     byte (radix_kernel.cuh:412-465 pass loop, ping-pong buffers), whose
 *     result equals a stable sort of the twiddled keys; both forms are here
 *     (oracle_lsd_sort_* and oracle_sort_*) and the tests check they agree.
 *   - the global digit histogram: detail/histogram.cuh:88-211 (counts per pass)
 *
 * Parity is pinned against the reference itself: oracle/ref_probe.cpp
 * compiles the reference's own radix_traits::twiddle_in/out and mix32 on the
 * host, and tests/golden/ holds the vectors it printed.
 */
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#include <parallel/algorithm>
#endif

namespace {

using u128 = unsigned __int128;

enum KeyType {
    U8 = 0, U16, U32, U64, U128,
    I8, I16, I32, I64, I128,
    F32, F64, F128, KEY_COUNT
};

enum Kind { UNSIGNED = 0, SIGNED = 1, FLOAT = 2 };

int key_bytes(int kt) {
    static const int b[KEY_COUNT] = {1, 2, 4, 8, 16, 1, 2, 4, 8, 16, 4, 8, 16};
    return (kt >= 0 && kt < KEY_COUNT) ? b[kt] : 0;
}

int key_kind(int kt) {
    if (kt >= F32) return FLOAT;
    if (kt >= I8) return SIGNED;
    return UNSIGNED;
}

template <class U>
U sign_bit() { return U(U(1) << (8 * sizeof(U) - 1)); }

// tuning.cuh:352-367
template <class U>
U twiddle_in(U b, int kind, bool desc) {
    const U s = sign_bit<U>();
    if (kind == FLOAT) b = (b & s) ? U(~b) : U(b ^ s);
    else if (kind == SIGNED) b = U(b ^ s);
    return desc ? U(~b) : b;
}

// tuning.cuh:370-384
template <class U>
U twiddle_out(U b, int kind, bool desc) {
    const U s = sign_bit<U>();
    if (desc) b = U(~b);
    if (kind == FLOAT) return (b & s) ? U(b ^ s) : U(~b);
    if (kind == SIGNED) return U(b ^ s);
    return b;
}

template <class U>
void load_bits(const void* src, size_t i, U* out) {
    std::memcpy(out, static_cast<const uint8_t*>(src) + i * sizeof(U), sizeof(U));
}

template <class U>
void store_bits(void* dst, size_t i, U v) {
    std::memcpy(static_cast<uint8_t*>(dst) + i * sizeof(U), &v, sizeof(U));
}

template <class U>
void twiddle_in_n(int kind, bool desc, const void* keys, void* bits, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        U b; load_bits(keys, i, &b);
        store_bits(bits, i, twiddle_in<U>(b, kind, desc));
    }
}

template <class U>
void twiddle_out_n(int kind, bool desc, const void* bits, void* keys, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        U b; load_bits(bits, i, &b);
        store_bits(keys, i, twiddle_out<U>(b, kind, desc));
    }
}

// Stable sort by twiddled bits.  Keys and (optional) values are permuted in
// place.  `threads` > 1 uses libstdc++ parallel mode (OpenMP).
template <class U>
void stable_sort_by_bits(int kind, bool desc, void* keys, void* vals,
                         size_t vbytes, size_t n, int threads) {
    if (n == 0) return;
    if (vals == nullptr || vbytes == 0) {
        std::vector<U> bits(n);
        for (size_t i = 0; i < n; ++i) {
            U b; load_bits(keys, i, &b);
            bits[i] = twiddle_in<U>(b, kind, desc);
        }
#ifdef _OPENMP
        if (threads > 1) {
            omp_set_num_threads(threads);
            __gnu_parallel::stable_sort(bits.begin(), bits.end());
        } else
#endif
        {
            (void)threads;
            std::stable_sort(bits.begin(), bits.end());
        }
        for (size_t i = 0; i < n; ++i) store_bits(keys, i, twiddle_out<U>(bits[i], kind, desc));
        return;
    }
    struct Item { U bits; uint64_t idx; };
    std::vector<Item> items(n);
    for (size_t i = 0; i < n; ++i) {
        U b; load_bits(keys, i, &b);
        items[i].bits = twiddle_in<U>(b, kind, desc);
        items[i].idx = i;
    }
    auto less = [](const Item& a, const Item& b) { return a.bits < b.bits; };
#ifdef _OPENMP
    if (threads > 1) {
        omp_set_num_threads(threads);
        __gnu_parallel::stable_sort(items.begin(), items.end(), less);
    } else
#endif
    {
        std::stable_sort(items.begin(), items.end(), less);
    }
    std::vector<uint8_t> vcopy(n * vbytes);
    std::memcpy(vcopy.data(), vals, n * vbytes);
    uint8_t* vout = static_cast<uint8_t*>(vals);
    for (size_t i = 0; i < n; ++i) {
        store_bits(keys, i, twiddle_out<U>(items[i].bits, kind, desc));
        std::memcpy(vout + i * vbytes, vcopy.data() + items[i].idx * vbytes, vbytes);
    }
}

// Restatement of the reference's pass loop (radix_kernel.cuh:412-465): one
// stable counting pass per 8-bit digit, least significant first, ping-pong
// between two buffers; the digit histogram of each pass comes first
// (histogram.cuh:88-211) and its exclusive scan gives the output bases.
template <class U>
void lsd_sort(int kind, bool desc, void* keys, void* vals, size_t vbytes, size_t n) {
    if (n == 0) return;
    std::vector<U> a(n), b(n);
    for (size_t i = 0; i < n; ++i) {
        U k; load_bits(keys, i, &k);
        a[i] = twiddle_in<U>(k, kind, desc);
    }
    const bool pairs = vals != nullptr && vbytes != 0;
    std::vector<uint8_t> va, vb;
    if (pairs) {
        va.assign(static_cast<uint8_t*>(vals), static_cast<uint8_t*>(vals) + n * vbytes);
        vb.resize(n * vbytes);
    }
    for (unsigned p = 0; p < sizeof(U); ++p) {
        size_t count[256] = {0};
        for (size_t i = 0; i < n; ++i) ++count[unsigned(a[i] >> (8 * p)) & 0xFFu];
        size_t base[256];
        size_t run = 0;
        for (int d = 0; d < 256; ++d) { base[d] = run; run += count[d]; }
        for (size_t i = 0; i < n; ++i) {
            const unsigned d = unsigned(a[i] >> (8 * p)) & 0xFFu;
            const size_t o = base[d]++;
            b[o] = a[i];
            if (pairs) std::memcpy(&vb[o * vbytes], &va[i * vbytes], vbytes);
        }
        a.swap(b);
        if (pairs) va.swap(vb);
    }
    for (size_t i = 0; i < n; ++i) store_bits(keys, i, twiddle_out<U>(a[i], kind, desc));
    if (pairs) std::memcpy(vals, va.data(), n * vbytes);
}

template <class U>
void histogram(int kind, bool desc, const void* keys, size_t n, uint64_t* counts) {
    std::memset(counts, 0, sizeof(uint64_t) * 256 * sizeof(U));
    for (size_t i = 0; i < n; ++i) {
        U k; load_bits(keys, i, &k);
        const U t = twiddle_in<U>(k, kind, desc);
        for (unsigned p = 0; p < sizeof(U); ++p) ++counts[p * 256 + (unsigned(t >> (8 * p)) & 0xFFu)];
    }
}

#define DISPATCH_WIDTH(kt, CALL)                  \
    switch (key_bytes(kt)) {                      \
        case 1: { using U = uint8_t; CALL; } break;  \
        case 2: { using U = uint16_t; CALL; } break; \
        case 4: { using U = uint32_t; CALL; } break; \
        case 8: { using U = uint64_t; CALL; } break; \
        case 16: { using U = u128; CALL; } break;    \
        default: return -1;                       \
    }

}  // namespace

extern "C" {

int oracle_key_bytes(int kt) { return key_bytes(kt); }

int oracle_twiddle_in(int kt, int desc, const void* keys, void* bits, size_t n) {
    DISPATCH_WIDTH(kt, twiddle_in_n<U>(key_kind(kt), desc != 0, keys, bits, n));
    return 0;
}

int oracle_twiddle_out(int kt, int desc, const void* bits, void* keys, size_t n) {
    DISPATCH_WIDTH(kt, twiddle_out_n<U>(key_kind(kt), desc != 0, bits, keys, n));
    return 0;
}

// std::stable_sort on twiddled keys (single thread): the correctness oracle.
int oracle_sort(int kt, int desc, void* keys, void* vals, size_t vbytes, size_t n) {
    DISPATCH_WIDTH(kt, stable_sort_by_bits<U>(key_kind(kt), desc != 0, keys, vals, vbytes, n, 1));
    return 0;
}

// Same result, libstdc++ parallel-mode stable sort on `threads` host threads:
// the timed CPU baseline.
int oracle_sort_parallel(int kt, int desc, void* keys, void* vals, size_t vbytes,
                         size_t n, int threads) {
    DISPATCH_WIDTH(kt, stable_sort_by_bits<U>(key_kind(kt), desc != 0, keys, vals, vbytes, n, threads));
    return 0;
}

// Literal LSD restatement of the reference's pass loop.
int oracle_lsd_sort(int kt, int desc, void* keys, void* vals, size_t vbytes, size_t n) {
    DISPATCH_WIDTH(kt, lsd_sort<U>(key_kind(kt), desc != 0, keys, vals, vbytes, n));
    return 0;
}

// Digit counts of every pass: counts[p * 256 + d], p < key bytes.
int oracle_histogram(int kt, int desc, const void* keys, size_t n, uint64_t* counts) {
    DISPATCH_WIDTH(kt, histogram<U>(key_kind(kt), desc != 0, keys, n, counts));
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
