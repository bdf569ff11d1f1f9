// shapes.h — CTA geometry of the onesweep pass per (key bytes, value bytes).
//
// Chosen for GB300: items per thread sized so two CTAs fit in an SM's 228 KB
// of shared memory where possible (two double-buffered key tiles, one value
// tile, per-warp counters and match words per CTA) and the register file
// holds keys, values and ranks without spilling.
#pragma once

#include <cmath>

#include <cstdint>

namespace gbsort {

// Threads of the upsweep (global histogram) kernel.
constexpr int HIST_THREADS = 1024;

// Measured on a GB300 (pass kernel, bench.py configurations):
//   4-byte keys only, 2^28:      384 x 24, 2 CTAs/SM  (67 Gkeys/s)
//   f32 keys + u32 values, 2^28: 256 x 26, 2 CTAs/SM  (49 Gkeys/s)
//   u64 keys + u64 values, 2^27: 256 x 14, 2 CTAs/SM  (15.0 Gkeys/s)
//   u128 keys only, 2^26:        384 x 16, 1 CTA/SM   (7.45 Gkeys/s)
// Tile bytes per key are 2K + V (only keys are double-buffered), so with
// values the tile grows with 2(K + V) / (2K + V) over a layout that double
// buffers both; other widths follow by bytes per item in the same budget.
struct ShapeRow {
    int threads, ipt, min_ctas;
};
constexpr ShapeRow pass_shape_row(int kb, int vb) {
    if (kb <= 4) {
        if (vb == 0) return {384, 24, 2};
        if (vb <= 4) return {256, 26, 2};
        if (vb == 8) return {256, 22, 2};
        return {256, 13, 2};
    }
    if (kb == 8) {
        if (vb == 0) return {256, 22, 2};
        if (vb <= 4) return {256, 17, 2};
        if (vb == 8) return {256, 14, 2};
        return {256, 10, 2};
    }
    if (vb == 0) return {384, 16, 1};
    if (vb <= 8) return {256, 8, 2};
    return {256, 6, 2};
}

// Small inputs (n <= 2^22, the reference's "short" range): tiles of about half
// the size at 256 threads and two CTAs per SM, so a short array still spreads
// over the SMs (2^20 u32 keys: 114 tiles of 9216 keys leave SMs idle; 256 of
// 4096 keys took 12.8 -> 14.2 Gkeys/s on GB300).
constexpr ShapeRow pass_shape_small_row(int kb, int vb) {
    if (kb <= 4) return {256, vb == 0 ? 16 : vb <= 4 ? 13 : vb == 8 ? 11 : 7, 2};
    if (kb == 8) return {256, vb == 0 ? 11 : vb <= 4 ? 9 : vb == 8 ? 7 : 5, 2};
    return {256, vb == 0 ? 8 : vb <= 8 ? 4 : 3, 2};
}
constexpr uint64_t SMALL_N_MAX = uint64_t(1) << 22;

// Arrays sorted in one launch when keys-only (fused_short.cuh): up to 2^21
// keys (2^20 for 16-byte keys, whose buckets outgrow a CTA sooner and whose
// 16 passes then run slower inside one launch: 2^21 u128 610 vs 567 us).
// With every digit taking a pass inside the launch, u32 measured (CUDA
// events) 2^16 40.8 vs 59.0 us, 2^20 56-58 vs 76.6, 2^22 164.8 vs 157.4;
// with the MSD partition + bucket sorts, 2^17 28.6 vs 62.5, 2^20 36.6 vs
// 76.6, 2^21 98 vs 111.
constexpr uint64_t FUSED_N_MAX = uint64_t(1) << 21;
constexpr uint64_t fused_n_max(int kb) { return kb == 16 ? FUSED_N_MAX / 2 : FUSED_N_MAX; }

// The one-launch short sort: the short shape's tile, ranked by 512 threads
// where it divides (half the columns per warp: a shorter dependent chain in
// the rank, which bounds a short sort's passes).
template <int KB>
struct FusedShape {
    static constexpr int TILE = pass_shape_small_row(KB, 0).threads * pass_shape_small_row(KB, 0).ipt;
    static constexpr int THREADS = TILE % 512 == 0 ? 512 : pass_shape_small_row(KB, 0).threads;
    static constexpr int IPT = TILE / THREADS;
    static constexpr int MIN_CTAS = pass_shape_small_row(KB, 0).min_ctas;
    // keys per thread of the bucket sort after the MSD partition: buckets of
    // up to THREADS * LIPT keys (2 and 4-byte keys 8192, 8-byte 7168, 16-byte
    // 3072), sized so that two CTAs still fit an SM
    static constexpr int LIPT = KB == 1 ? IPT : KB <= 4 ? 2 * IPT : KB == 8 ? 28 : 6;
};

// Keys per bucket the one-launch sort's CTA sorts in shared memory.
constexpr int fused_local_tile(int kb) {
    return kb == 1    ? FusedShape<1>::THREADS * FusedShape<1>::LIPT
           : kb == 2  ? FusedShape<2>::THREADS * FusedShape<2>::LIPT
           : kb == 4  ? FusedShape<4>::THREADS * FusedShape<4>::LIPT
           : kb == 8  ? FusedShape<8>::THREADS * FusedShape<8>::LIPT
                      : FusedShape<16>::THREADS * FusedShape<16>::LIPT;
}

// Keys-only sorts of 8- and 16-byte keys, most significant digit first
// (msd.cuh): the two splits' tiles (THREADS x IPT keys; 8-byte keys 2^27:
// 2.95 ms with 24 keys per thread, 3.06 with 16, 3.03 with 32) and the local
// sorts' CTAs (groups of up to C_THREADS x C_LIPT keys), for n in
// [msd_n_min, msd_n_max] (groups of ~24 to ~2048 / ~384 to ~4096 keys;
// outside, the digit passes).  Measured against the digit passes, CUDA
// events, descending: 16-byte keys 2^22 0.58 vs 0.82 ms, 2^24 0.89 vs 2.46,
// 2^26 2.11 vs 9.24; 8-byte keys 2^24 0.86 vs 0.82, 2^25 1.18 vs 1.52, 2^27
// 2.95 vs 5.71.
// Two local-sort shapes per width: L = 0 for groups of up to ~1024
// (16-byte) / ~2048 (8-byte) keys on average, more CTAs per SM; L = 1 for
// the larger groups up to msd_n_max.
template <int KB>
struct MsdShape {
    static constexpr int THREADS = 256;
    static constexpr int IPT = KB == 16 ? 12 : 24;
    static constexpr int MIN_CTAS = 2;
    static constexpr int C_THREADS = 256;
    // 16-byte keys up to 2^26 (groups of up to ~1024 keys on average): 6 keys
    // a thread, 4 CTAs an SM (2^26: local sorts 0.655 ms against 0.703 with
    // 8 keys a thread and 3 CTAs; 1024 sub-buckets 0.694)
    static constexpr int C_LIPT[2] = {KB == 16 ? 6 : 12, KB == 16 ? 12 : 24};
    static constexpr int C_MIN_CTAS[2] = {KB == 16 ? 4 : 3, 2};
    static constexpr int C_SPLIT_WORDS[2] = {KB == 16 ? 2048 : 4096, 4096};
};
// (4-byte keys measured slower this way: 2^28 u32 5.12 vs 4.11 ms, 2^25
// 1.01 vs 0.58 — groups of 4096 keys with 16 bits left cost their local sort
// more than the two digit passes it replaces.)
constexpr bool msd_key_bytes(int kb) { return kb == 8 || kb == 16; }
// (16-byte keys, descending, against the digit passes of the short shape:
// 2^20 0.40 vs 0.32 ms, 1.5 x 2^20 0.488 vs 0.491, 2^21 0.50 vs 0.56, 3 x 2^20
// 0.52 vs 0.74.)
constexpr uint64_t msd_n_min(int kb) { return kb == 16 ? uint64_t(3) << 19 : uint64_t(3) << 23; }
constexpr uint64_t msd_n_max(int kb) { return kb == 16 ? uint64_t(1) << 27 : uint64_t(1) << 28; }
// the local-sort shape for n keys (groups of n / 65536 on average)
constexpr int msd_local_shape(int kb, uint64_t n) { return n <= (msd_n_max(kb) >> 1) ? 0 : 1; }
constexpr uint32_t msd_group_cap(int kb, int shape) {
    return kb == 16 ? uint32_t(MsdShape<16>::C_THREADS * MsdShape<16>::C_LIPT[shape])
                    : uint32_t(MsdShape<8>::C_THREADS * MsdShape<8>::C_LIPT[shape]);
}

// Keys per MSD region of the one-launch sort (one region per top digit):
// the mean bucket n/256 plus four of its standard deviations plus 64,
// rounded up to 32 (uniform top digits overflow a region about once in
// 10^4 sorts at 2^20 keys, and then the sort takes the per-digit passes);
// 0 where that exceeds a CTA's local sort.
inline uint32_t msd_region_cap(int kb, uint64_t n) {
    const double mean = double((n + 255) / 256);
    const uint64_t cap = (uint64_t(mean + 4.0 * std::sqrt(mean) + 64.0) + 31) & ~uint64_t(31);
    return cap <= uint64_t(fused_local_tile(kb)) ? uint32_t(cap) : 0u;
}

// Predecessor tiles per lookback round trip for short arrays: all their tiles
// are in flight at once, so the known-prefix frontier moves a window per L2
// round trip (2^20 u32: 4 -> 8 took 14.0 -> 14.35 Gkeys/s; 16 and 32 slower).
#ifndef GBSORT_SMALL_WINDOW
#define GBSORT_SMALL_WINDOW 8
#endif

template <int KB, int VB>
struct PassShapeSmall {
    static constexpr int THREADS = pass_shape_small_row(KB, VB).threads;
    static constexpr int IPT = pass_shape_small_row(KB, VB).ipt;
    static constexpr int MIN_CTAS = pass_shape_small_row(KB, VB).min_ctas;
    static constexpr int LOOKBACK_WINDOW = GBSORT_SMALL_WINDOW;
};

template <int KB, int VB>
struct PassShape {
    static constexpr int THREADS = pass_shape_row(KB, VB).threads;
    static constexpr int IPT = pass_shape_row(KB, VB).ipt;
    // Resident CTAs per SM the register allocation must allow.
    static constexpr int MIN_CTAS = pass_shape_row(KB, VB).min_ctas;
    // Predecessor tiles read per lookback round trip.
    static constexpr int LOOKBACK_WINDOW = 4;
};

// Build-time override of one (key bytes, value bytes) shape, for tuning
// sweeps: -DGBSORT_SHAPE_KB=.. -DGBSORT_SHAPE_VB=.. -DGBSORT_SHAPE_THREADS=..
// -DGBSORT_SHAPE_IPT=.. -DGBSORT_SHAPE_MIN_CTAS=..
#if defined(GBSORT_SHAPE_KB)
#ifndef GBSORT_SHAPE_WINDOW
#define GBSORT_SHAPE_WINDOW 4
#endif
template <>
struct PassShape<GBSORT_SHAPE_KB, GBSORT_SHAPE_VB> {
    static constexpr int THREADS = GBSORT_SHAPE_THREADS;
    static constexpr int IPT = GBSORT_SHAPE_IPT;
    static constexpr int MIN_CTAS = GBSORT_SHAPE_MIN_CTAS;
    static constexpr int LOOKBACK_WINDOW = GBSORT_SHAPE_WINDOW;
};
#endif

// Older form of the override for the 4-byte keys-only shape.
#if defined(GBSORT_SHAPE_K4V0_THREADS)
template <>
struct PassShape<4, 0> {
    static constexpr int THREADS = GBSORT_SHAPE_K4V0_THREADS;
    static constexpr int IPT = GBSORT_SHAPE_K4V0_IPT;
    static constexpr int MIN_CTAS = GBSORT_SHAPE_K4V0_MIN_CTAS;
    static constexpr int LOOKBACK_WINDOW = GBSORT_SHAPE_K4V0_WINDOW;
};
#endif

// Value-size index used by the dispatch tables: 0,1,2,4,8,16 bytes -> 0..5.
inline int value_index(int vb) {
    switch (vb) {
        case 0: return 0;
        case 1: return 1;
        case 2: return 2;
        case 4: return 3;
        case 8: return 4;
        case 16: return 5;
        default: return -1;
    }
}

struct KernelEntry {
    const void* fn;
    int threads;
    int ipt;
    int tile;
    unsigned long smem;
};

// Defined in inst_k{1,2,4,8,16}.cu: entries[value_index][wide_status].
const KernelEntry* pass_entries(int kb);
const KernelEntry* upsweep_entry(int kb);

}  // namespace gbsort
