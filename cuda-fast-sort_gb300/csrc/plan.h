// plan.h — host-side planning of one sort: geometry, workspace layout and
// launch sizes.  Shared by the plain sort (sort_api.cu) and the batched path.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "shapes.h"

namespace gbsort {

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Control block at the start of the workspace's control region:
//   [gp_counts: passes*256 u64][tile_counters: 16 u32][err: u32][executed: u32][barrier: u32][pad]
//   [barrier generation: u32, own 128-byte line][pad]
// executed: written by the pass kernels that run (bit 31 | passes executed)
// when uniform passes are skipped; 0 when none ran.
struct CtlLayout {
    size_t gp_off = 0;
    size_t counters_off = 0;
    size_t err_off = 0;
    size_t exec_off = 0;
    size_t barrier_off = 0;      // grid barrier counter of the one-launch short sort
    size_t barrier_gen_off = 0;  // its generation word (another 128-byte line)
    size_t fill_off = 0;         // [256] fill counts of its MSD regions
    size_t overflow_off = 0;     // its region overflow flag
    size_t bytes = 0;
    static CtlLayout make(int passes) {
        CtlLayout c;
        c.gp_off = 0;
        c.counters_off = size_t(passes) * 256 * 8;
        c.err_off = c.counters_off + 16 * 4;
        c.exec_off = c.err_off + 4;
        c.barrier_off = c.exec_off + 4;
        c.barrier_gen_off = align_up(c.barrier_off + 4, 128);
        c.fill_off = align_up(c.barrier_gen_off + 4, 128);
        c.overflow_off = c.fill_off + 256 * 4;
        c.bytes = align_up(c.overflow_off + 4, 256);
        return c;
    }
};

// The MSD block of a keys-only sort of 8- or 16-byte keys (offsets from
// Plan::msd_off; msd.cuh).
struct MsdLayout {
    static constexpr size_t STATE = 0;
    static constexpr size_t CURSOR1 = 256;
    static constexpr size_t JOINT = CURSOR1 + 256 * 4;
    static constexpr size_t CURSOR2 = JOINT + 65536 * 4;
    static constexpr size_t ZERO_BYTES = CURSOR2 + 65536 * 4;  // cleared by the upsweep
    static constexpr size_t OFFS2 = ZERO_BYTES;
    static constexpr size_t BYTES = OFFS2 + 65536 * 4;
};

struct Plan {
    int key_type = 0;
    int kb = 0;            // key bytes
    int vb = 0;            // value bytes (0: keys only)
    int kind = 0;          // KeyKind
    int passes = 0;
    bool wide_status = false;
    KernelEntry pass{};
    KernelEntry upsweep{};
    // One-launch path (short keys-only arrays): upsweep, passes and fix-up in
    // one cooperative kernel of pass's shape.  fused.fn == nullptr: not used.
    KernelEntry fused{};
    uint64_t n = 0;
    uint32_t num_tiles = 0;
    // workspace layout (offsets from the workspace base)
    size_t alt_keys_off = 0;
    size_t alt_vals_off = 0;
    size_t ctl_off = 0;
    size_t status_off = 0;
    size_t status_bytes = 0;
    // the one-launch sort's MSD regions: 256 x msd_cap keys (msd_cap 0: none)
    size_t regions_off = 0;
    uint32_t msd_cap = 0;
    // keys-only sorts of 8- and 16-byte keys, most significant digit first
    // (msd.cuh): kernels (top split, pair count, scan, second split, local
    // sorts), group capacity, and the block at msd_off: state word (256 B),
    // cursors [256], group sizes [65536], group cursors [65536] — zeroed by
    // the upsweep — then group offsets [65536]
    bool msd = false;
    KernelEntry msd_k[5]{};
    KernelEntry msd_hist{};  // its first kernel: the top digit's histogram
    uint32_t msd_group_cap = 0;
    size_t msd_off = 0;
    size_t total_bytes = 0;
    CtlLayout ctl{};
};

// Fills *plan; returns a gbsort_status code.
int make_plan(int key_type, size_t value_bytes, uint64_t n, Plan* plan);

// DoubleBuffer form: the caller's second key (and value) buffer replaces
// the workspace's alternate buffers, and the workspace holds only the
// control block and the lookback status (double_buffer_bytes).  The result
// lands in the second buffer when the pass count is odd, else in the first.
struct AltBuffers {
    void* keys_b;
    void* vals_b;
};
size_t double_buffer_bytes(const Plan& plan);

// Enqueues one sort on `stream`.  `ms` (optional) receives per-kernel event
// times after a stream sync: [upsweep, pass 0 .. pass P-1].
// keys_src != nullptr: input-preserving sort, reads keys_src (and vals_src)
// and leaves the result in d_keys (and d_values).
int enqueue_sort(const Plan& plan, int descending, void* d_keys, void* d_values, void* d_workspace,
                 cudaStream_t stream, float* ms, int ms_cap, int* n_ms, const void* keys_src = nullptr,
                 const void* vals_src = nullptr, const AltBuffers* alt = nullptr);

// Device facts (cached per device).
int device_sm_count();
int device_is_sm103();
int resident_ctas(const KernelEntry& e);  // per SM, after opting in to the smem
int prepare_kernel(const KernelEntry& e); // cudaFuncSetAttribute once per device
uint32_t upsweep_ctas(uint64_t n, int kb);  // grid of the plain upsweep

uint64_t wait_limit_ns();
int status_from_error_word(uint32_t err);  // workspace error word -> gbsort_status
void set_last_error(const char* what, cudaError_t err);
void set_last_error_text(const char* text);

}  // namespace gbsort
