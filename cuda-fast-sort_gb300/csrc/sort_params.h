// sort_params.h — launch parameter blocks shared by host and device code.
#pragma once

#include <cstdint>

namespace gbsort {

// Outcome of the most-significant-digit-first path of a keys-only sort
// (msd.cuh): 0 undecided, MSD_OK the MSD kernels sort, MSD_OFF the digit
// passes sort.
constexpr uint32_t MSD_OK = 1u, MSD_OFF = 2u;

// Global-histogram upsweep (one launch per sort).
struct HistParams {
    const void* keys;           // user keys (raw bits)
    uint64_t n;
    int kind;                   // KeyKind
    int desc;                   // descending
    unsigned long long* gp_counts;  // [passes][256] digit counts, zeroed before launch
    void* status;               // lookback status array to clear
    uint64_t status_bytes;      // multiple of 16
    // Odd pass counts (1-byte keys) end in the alternate buffer; the upsweep
    // then also mirrors keys/values there so the single pass lands in place.
    void* mirror_keys;          // nullptr: no mirroring
    const void* vals;
    void* mirror_vals;
    uint64_t val_bytes_total;   // n * value bytes
    // digits counted: [digit_lo, digit_hi), every digit when digit_hi == 0
    int digit_lo, digit_hi;
    // non-null: a histogram of the remaining digits for the digit passes of
    // a keys-only sort whose MSD path may already have sorted: exits when it
    // did (MSD_OK), waits for its predecessor kernel first
    const uint32_t* msd_state;
};

// Batched mode: one entry per global tile, built on the host.
struct alignas(16) TileRec {
    unsigned long long base;  // index of the tile's first element in the key array
    uint32_t cnt;             // elements in the tile
    uint32_t seg_flags;       // segment << 2 | last << 1 | first
};

// One onesweep digit pass (one persistent launch per digit).
struct PassParams {
    const void* keys_in;
    void* keys_out;
    const void* vals_in;
    void* vals_out;
    uint64_t n;
    uint32_t num_tiles;
    int pass;                   // digit index, 0 = least significant byte
    int kind;
    int desc;
    int twiddle_load;           // first pass: map raw keys to ordered bits
    int twiddle_store;          // last pass: map ordered bits back to keys
    int tma_keys;               // keys_in 16-byte aligned: tiles arrive by bulk copy
    int tma_vals;
    const unsigned long long* gp_counts;  // this pass's row [256]
    void* status;               // [num_tiles][256] status words
    uint32_t* tile_counter;     // this pass's dynamic tile counter (zeroed)
    uint32_t* err;              // workspace error word
    uint64_t wait_limit_ns;
    // batched mode only
    const TileRec* tiles;       // [num_tiles]
    const uint32_t* seg_gofs;   // [segments][256] absolute output base of each digit, this pass
    // Uniform-digit pass skipping (plain sort).  skip != 0: a pass whose digit
    // is the same for all n keys is a no-op and exits; the kernel derives its
    // buffers and twiddles from every pass's digit counts instead of taking
    // keys_in/out, vals_in/out and twiddle_load/store from the host.
    int skip;
    int passes;
    int start_alt;              // the data starts in the alternate buffer (mirrored)
    const unsigned long long* gp_all;  // [passes][256]
    void* keys_a;               // the caller's buffers
    void* vals_a;
    void* keys_b;               // the workspace's alternate buffers
    void* vals_b;
    // Input-preserving sort: the first executed pass reads these, passes then
    // alternate between the caller's output (keys_a/vals_a) and the alternate
    // buffers so that the last one lands in the output.  nullptr: in place.
    const void* copy_keys_in;
    const void* copy_vals_in;
    // batched mode: bit q set when pass q's digit varies inside some segment
    const uint32_t* nonuniform_mask;
    // plain mode with skipping: receives bit 31 | number of executed passes
    uint32_t* executed;
    // keys-only sorts with the MSD path: the pass exits when it sorted (MSD_OK)
    const uint32_t* msd_state;
};

// The copy home after uniform-pass skipping left an odd number of executed
// passes (the result then sits in the alternate buffer).
struct FixupParams {
    const uint32_t* executed;  // bit 31 | executed passes, 0 when none ran
    int passes;
    void* keys_b;
    void* keys_a;
    uint64_t key_bytes_total;
    void* vals_b;
    void* vals_a;
    uint64_t val_bytes_total;
    // parity of executed passes that leaves the result where it belongs:
    // 0 in place (in a), 1 in b (DoubleBuffer form of an odd pass count);
    // otherwise the result is copied across
    int want_odd;
    // input-preserving sort: when no pass ran, copy these to the output
    const void* copy_keys_in;
    const void* copy_vals_in;
    // keys-only sorts with the MSD path: nothing to do when it sorted
    const uint32_t* msd_state;
};

// One-launch sort of a short array (cooperative launch, every CTA resident):
// digit counts of all passes, then every pass, then the parity fix-up, with a
// grid barrier between the phases.
struct FusedParams {
    HistParams hist;        // phase 0 (status clear, mirror for odd pass counts)
    PassParams pass;        // pass 0; the kernel derives each later pass from it
    FixupParams fix;
    int fixup;              // run the fix-up phase
    uint32_t* barrier;      // grid barrier counter and generation, zeroed before the launch
    uint32_t* barrier_gen;
    int msd;                // MSD partition into the regions + bucket sorts (needs regions)
    void* regions;          // 256 regions of region_cap keys (workspace), one per top digit
    uint32_t region_cap;
    uint32_t* fill;         // [256] keys claimed in each region, zeroed before the launch
    uint32_t* overflow;     // nonzero: a region overflowed (zeroed before the launch)
};

// Batched upsweep: one work item per chunk of one segment.
struct SegItem {
    unsigned long long begin, end;  // element range (within one segment)
    uint32_t seg;                   // onesweep segment index
    uint32_t pad;
};

struct SegUpsweepParams {
    const void* keys;
    int kind;
    int desc;
    const SegItem* items;
    uint32_t num_items;
    uint32_t* item_counter;     // zeroed
    uint32_t* seg_counts;       // [segments][passes][256], zeroed
    void* status;               // lookback status array to clear
    uint64_t status_bytes;
    // odd pass counts: mirror each item's keys/values into the alternate buffer
    void* mirror_keys;
    const void* vals;
    void* mirror_vals;
    uint32_t val_bytes;
};

// Batched: digit counts -> absolute digit bases, one CTA per (segment, pass).
struct SegScanParams {
    const uint32_t* seg_counts;           // [segments][passes][256]
    const unsigned long long* seg_begin;  // [segments]
    uint32_t* seg_gofs;                   // [passes][segments][256]
    uint32_t segments;
    uint32_t passes;
    uint32_t* nonuniform;                 // bit q: pass q's digit varies inside some segment
};

// Batched pass skipping: copies the onesweep segments' tiles home when an
// odd number of passes ran.
struct SegFixupParams {
    const TileRec* tiles;
    uint32_t num_tiles;
    int passes;
    const uint32_t* nonuniform;
    uint32_t key_bytes, val_bytes;
    const void* keys_b;
    void* keys_a;
    const void* vals_b;
    void* vals_a;
};

// Small segments sorted whole inside one CTA's shared memory.
struct CtaSortParams {
    void* keys;
    void* vals;
    const SegItem* segs;        // [num_segs] (begin, end)
    uint32_t num_segs;
    uint32_t* seg_counter;      // zeroed
    int kind;
    int desc;
};

}  // namespace gbsort
