// shapes.h — CTA geometry of the onesweep pass per (key bytes, value bytes).
//
// Chosen for GB300: 512 threads (16 warps; the first 256 threads own one
// digit bin each), items per thread sized so two CTAs (two double-buffered
// tiles each) fit in an SM's 228 KB of shared memory where possible and the
// register file holds keys, values and ranks without spilling.
#pragma once

namespace gbsort {

// Threads of the upsweep (global histogram) kernel.
constexpr int HIST_THREADS = 1024;

template <int KB, int VB>
struct PassShape {
    static constexpr int THREADS = (KB <= 4 && VB == 0) ? 384 : 512;
    static constexpr int IPT =
        KB <= 4 ? (VB == 0 ? 24 : VB <= 4 ? 10 : VB == 8 ? 8 : 6)
      : KB == 8 ? (VB == 0 ? 10 : VB <= 4 ? 8 : VB == 8 ? 6 : 4)
      :           (VB == 0 ? 6 : 4);
    // Resident CTAs per SM the register allocation must allow.
    static constexpr int MIN_CTAS = 2;
    // Predecessor tiles read per lookback round trip.
    static constexpr int LOOKBACK_WINDOW = 8;
};

// Build-time override of the 4-byte keys-only shape, for tuning sweeps
// (-DGBSORT_SHAPE_K4V0_THREADS=.. -DGBSORT_SHAPE_K4V0_IPT=.. -DGBSORT_SHAPE_K4V0_MIN_CTAS=..).
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
