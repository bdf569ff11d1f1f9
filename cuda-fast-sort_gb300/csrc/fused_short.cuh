// fused_short.cuh — the whole sort of a short keys-only array in one
// cooperative launch (sm_103a).
//
// A short array (n <= 2^22, the reference's short mode,
// include/rsort/detail/radix_kernel.cuh:525-559) sorted by separate launches
// spends most of its time outside the work: every launch ramps up and drains,
// the upsweep's CTAs each end on global atomics, and each pass starts by
// fetching its digit offsets.  Here one cooperative launch (every CTA
// resident at once, or the launch fails) runs
//   phase 0: the digit counts of every pass from one read of the keys (plus
//            the lookback status clear and, for odd pass counts, the mirror);
//   one phase per digit pass: the onesweep pass body of the multi-launch
//            path, unchanged (persistent tiles, bulk copies, lookback);
//   the parity fix-up when uniform passes were skipped;
// separated by a grid barrier whose wait is bounded like the lookback's
// (GBSORT_ERR_TIMEOUT, then every CTA leaves).
#pragma once

#include "onesweep.cuh"

namespace gbsort {

// Phase 0: every digit count of the whole array into p.gp_counts, using the
// CTA's tile buffers (smem_bytes of them) for shared counters.
template <int KB, int THREADS>
__device__ __forceinline__ void fused_counts(const HistParams& h, uint8_t* smem, size_t smem_bytes) {
    using U = typename KeyBits<KB>::U;
    constexpr int P = KB;
    constexpr int NB = P * 256;
    constexpr int WARPS = THREADS / 32;
    // lane groups (by warp) with counters of their own: fewer same-word atomics
    int copies = 1;
    while (copies * 2 <= WARPS && size_t(copies * 2) * NB * 4 <= smem_bytes) copies *= 2;
    uint32_t* cnt = reinterpret_cast<uint32_t*>(smem);
    const int tid = threadIdx.x;
    for (int i = tid; i < copies * NB; i += THREADS) cnt[i] = 0u;
    {
        const uint64_t nv = h.status_bytes >> 4;
        uint4* s = static_cast<uint4*>(h.status);
        const uint64_t stride = uint64_t(gridDim.x) * THREADS;
        for (uint64_t i = uint64_t(blockIdx.x) * THREADS + tid; i < nv; i += stride) s[i] = make_uint4(0, 0, 0, 0);
        if (h.mirror_keys) grid_copy_bytes(h.mirror_keys, h.keys, h.n * KB);
    }
    __syncthreads();
    uint32_t* mine = cnt + ((tid >> 5) & (copies - 1)) * NB;
    const U* keys = static_cast<const U*>(h.keys);
    const uint64_t stride = uint64_t(gridDim.x) * THREADS;
    for (uint64_t i = uint64_t(blockIdx.x) * THREADS + tid; i < h.n; i += stride) {
        const U t = twiddle_in<U>(keys[i], h.kind, h.desc);
#pragma unroll
        for (int d = 0; d < P; ++d) atomicAdd(&mine[d * 256 + digit_of(t, d)], 1u);
    }
    __syncthreads();
    for (int b = tid; b < NB; b += THREADS) {
        uint32_t s = 0;
        for (int c = 0; c < copies; ++c) s += cnt[c * NB + b];
        if (s) atomicAdd(&h.gp_counts[b], static_cast<unsigned long long>(s));
    }
}

template <int KB, class W, int THREADS, int IPT, int MIN_CTAS, int LBW>
__global__ void __launch_bounds__(THREADS, MIN_CTAS) fused_short_kernel(FusedParams f) {
    using G = PassGeom<KB, 0, THREADS, IPT>;
    extern __shared__ __align__(128) uint8_t smem[];
    const uint64_t limit = f.pass.wait_limit_ns;
    uint32_t* err = f.pass.err;
    uint32_t phase = 0;

    fused_counts<KB, THREADS>(f.hist, smem, 2 * G::BUF_BYTES);
    if (!grid_barrier(f.barrier, ++phase, limit, err)) return;

    const int passes = f.pass.passes;
    for (int q = 0; q < passes; ++q) {
        PassParams pp = f.pass;
        pp.pass = q;
        pp.gp_counts = f.pass.gp_all + size_t(q) * 256;
        pp.tile_counter = f.pass.tile_counter + q;
        // the host's ping-pong (used when neither skipping nor an input
        // copy lets the pass derive its own buffers)
        const bool from_a = ((q + f.pass.start_alt) & 1) == 0;
        pp.keys_in = from_a ? f.pass.keys_a : f.pass.keys_b;
        pp.keys_out = from_a ? f.pass.keys_b : f.pass.keys_a;
        pp.twiddle_load = q == 0;
        pp.twiddle_store = q == passes - 1;
        onesweep_pass_body<KB, 0, W, THREADS, IPT, false, LBW, true>(pp, smem);
        if (!grid_barrier(f.barrier, ++phase, limit, err)) return;
        if (ld_relaxed(err) != 0u) return;  // a failed wait or bounds check: every CTA leaves
    }
    if (f.fixup) fixup_body(f.fix);
}

}  // namespace gbsort
