// segmented.cuh — kernels of the batched (segmented) sort: thousands of
// independent sorts of uneven sizes in a handful of persistent launches.
//
//   seg_upsweep_kernel  per-segment digit counts of the segments that go
//                       through onesweep; work items = (segment, chunk)
//                       pulled from a device counter; also clears the
//                       lookback status array and mirrors keys for odd
//                       pass counts
//   seg_scan_kernel     (segmented_api.cu) counts -> absolute digit bases,
//                       one CTA per (segment, pass)
//   cta_sort_kernel     small segments sorted whole in one CTA's shared
//                       memory: all digit passes back to back, one read and
//                       one write of global memory; segments pulled from a
//                       device counter
// The onesweep passes themselves are onesweep_pass_kernel<..., SEG = true>.
// No reference counterpart: rsort sorts one array per call.
#pragma once

#include "onesweep.cuh"

namespace gbsort {

constexpr int SEG_UP_THREADS = 1024;

// CTA-wide copy of `bytes` bytes (16-byte vectors when both sides allow).
__device__ __forceinline__ void block_copy(uint8_t* dst, const uint8_t* src, uint64_t bytes) {
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
        const uint64_t nv = bytes >> 4;
        for (uint64_t i = threadIdx.x; i < nv; i += blockDim.x)
            reinterpret_cast<uint4*>(dst)[i] = reinterpret_cast<const uint4*>(src)[i];
        for (uint64_t i = (nv << 4) + threadIdx.x; i < bytes; i += blockDim.x) dst[i] = src[i];
    } else {
        for (uint64_t i = threadIdx.x; i < bytes; i += blockDim.x) dst[i] = src[i];
    }
}

// Counters [bin][copy], copy = lane % COPIES.  With 32 copies (keys up to 4
// bytes, 32-128 KB) every lane of a warp owns a bank and the atomics never
// conflict; wider keys keep 32 KB with 4 or 2 copies.
template <int KB>
struct SegHistGeom {
    static constexpr int P = KB;
    static constexpr int COPIES = P <= 4 ? 32 : (P == 8 ? 4 : 2);
    static constexpr int NBINS = P * 256;
    static constexpr size_t SMEM_BYTES = size_t(NBINS) * COPIES * 4;
};

template <int KB>
__global__ void __launch_bounds__(SEG_UP_THREADS) seg_upsweep_kernel(SegUpsweepParams p) {
    using U = typename KeyBits<KB>::U;
    using G = SegHistGeom<KB>;
    extern __shared__ __align__(16) uint32_t cnt[];
    __shared__ uint32_t s_item;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int copy = lane & (G::COPIES - 1);
    {
        const uint64_t nv = p.status_bytes >> 4;
        uint4* s = static_cast<uint4*>(p.status);
        const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
        for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + tid; i < nv; i += stride) s[i] = make_uint4(0, 0, 0, 0);
    }
    const U* keys = static_cast<const U*>(p.keys);
    const int kind = p.kind, desc = p.desc;
    auto count = [&](U k) {
        const U t = twiddle_in<U>(k, kind, desc);
#pragma unroll
        for (int d = 0; d < G::P; ++d) atomicAdd(&cnt[(d * 256 + digit_of(t, d)) * G::COPIES + copy], 1u);
    };
    for (;;) {
        if (tid == 0) s_item = atomicAdd(p.item_counter, 1u);
        for (int i = tid; i < G::NBINS * G::COPIES / 4; i += SEG_UP_THREADS)
            reinterpret_cast<uint4*>(cnt)[i] = make_uint4(0, 0, 0, 0);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= p.num_items) break;
        const SegItem w = p.items[item];
        if (p.mirror_keys)
            block_copy(static_cast<uint8_t*>(p.mirror_keys) + w.begin * KB,
                       static_cast<const uint8_t*>(p.keys) + w.begin * KB, (w.end - w.begin) * KB);
        if (p.mirror_vals)
            block_copy(static_cast<uint8_t*>(p.mirror_vals) + w.begin * p.val_bytes,
                       static_cast<const uint8_t*>(p.vals) + w.begin * p.val_bytes, (w.end - w.begin) * p.val_bytes);
        // aligned 16-byte body, scalar head and tail
        const U* k0 = keys + w.begin;
        const uint64_t m = w.end - w.begin;
        uint64_t head = ((16u - (reinterpret_cast<uintptr_t>(k0) & 15u)) & 15u) / KB;
        if (head > m) head = m;
        constexpr int PER_VEC = 16 / KB;
        const uint64_t nvec = (m - head) / PER_VEC;
        if (uint64_t(tid) < head) count(k0[tid]);
        const uint4* vec = reinterpret_cast<const uint4*>(k0 + head);
        // four 16-byte loads in flight per thread before their counts
        constexpr int UNROLL = 4;
        uint64_t i = tid;
        for (; i + (UNROLL - 1) * SEG_UP_THREADS < nvec; i += UNROLL * SEG_UP_THREADS) {
            uint4 v[UNROLL];
#pragma unroll
            for (int r = 0; r < UNROLL; ++r) v[r] = __ldcs(vec + i + r * SEG_UP_THREADS);
#pragma unroll
            for (int r = 0; r < UNROLL; ++r) {
                union { uint4 q; U k[PER_VEC]; } u;
                u.q = v[r];
#pragma unroll
                for (int e = 0; e < PER_VEC; ++e) count(u.k[e]);
            }
        }
        for (; i < nvec; i += SEG_UP_THREADS) {
            union { uint4 q; U k[PER_VEC]; } u;
            u.q = __ldcs(vec + i);
#pragma unroll
            for (int e = 0; e < PER_VEC; ++e) count(u.k[e]);
        }
        for (uint64_t j = head + nvec * PER_VEC + tid; j < m; j += SEG_UP_THREADS) count(k0[j]);
        __syncthreads();
        uint32_t* out = p.seg_counts + size_t(w.seg) * G::NBINS;
        for (int bin = warp; bin < G::NBINS; bin += SEG_UP_THREADS / 32) {
            uint32_t s = (lane < G::COPIES) ? cnt[bin * G::COPIES + lane] : 0u;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0 && s) atomicAdd(&out[bin], s);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Small segments: whole-segment LSD sort inside one CTA's shared memory.
// RBITS = bits per digit: 8 (256 bins, shared-memory OR match) or 4 (16
// bins, twice the passes but tiny scans, 4-ballot match) — the batched
// sort's tuning picks per size bucket.  Warp-columns holding only filler
// positions (past the segment's end) are skipped entirely.
// ---------------------------------------------------------------------------
template <int KB, int VB, int THREADS, int IPT, int RBITS>
struct CtaSortGeom {
    static constexpr int BINS = 1 << RBITS;
    static constexpr int PASSES = KB * 8 / RBITS;
    static constexpr int WARPS = THREADS / 32;
    static constexpr int TILE = THREADS * IPT;  // largest segment
    static constexpr int IPW = 32 * IPT;
    static constexpr size_t KEY_BYTES = size_t(TILE) * KB;
    static constexpr size_t VAL_OFF = (KEY_BYTES + 127) & ~size_t(127);
    static constexpr size_t BUF_BYTES = (VAL_OFF + size_t(TILE) * VB + 127) & ~size_t(127);
    static constexpr size_t HIST_OFF = 2 * BUF_BYTES;                              // u32 [WARPS][BINS]
    static constexpr size_t MATCH_OFF = HIST_OFF + size_t(WARPS) * BINS * 4;       // u32 [WARPS][256] (RBITS 8)
    static constexpr size_t SCAN_OFF = MATCH_OFF + (RBITS == 8 ? size_t(WARPS) * 256 * 4 : 0);  // u32 [16]
    static constexpr size_t SEG_OFF = SCAN_OFF + 64;                               // SegItem
    static constexpr size_t SMEM_BYTES = SEG_OFF + sizeof(SegItem);
    static_assert(RBITS == 8 || RBITS == 4, "8- or 4-bit digits");
    static_assert(THREADS >= BINS, "one bin owner per digit");
};

template <int RBITS, class U>
__device__ __forceinline__ uint32_t digit_bits(U x, int pass) {
    if constexpr (RBITS == 8) return digit_of(x, pass);
    else return uint32_t(x >> (pass * RBITS)) & ((1u << RBITS) - 1u);
}

// Lanes holding the same RBITS-bit digit, from one ballot per bit.
template <int RBITS>
__device__ __forceinline__ uint32_t match_ballot_bits(uint32_t d) {
    uint32_t peers = 0xffffffffu;
#pragma unroll
    for (int bit = 0; bit < RBITS; ++bit) {
        const uint32_t m = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
        peers &= ((d >> bit) & 1u) ? m : ~m;
    }
    return peers;
}

template <int KB, int VB, int THREADS, int IPT, int RBITS>
__global__ void __launch_bounds__(THREADS) cta_sort_kernel(CtaSortParams p) {
    using U = typename KeyBits<KB>::U;
    using V = typename ValBits<VB>::V;
    using G = CtaSortGeom<KB, VB, THREADS, IPT, RBITS>;
    constexpr bool PAIRS = VB > 0;
    constexpr int BINS = G::BINS;
    extern __shared__ __align__(128) uint8_t smem[];
    uint32_t* whist = reinterpret_cast<uint32_t*>(smem + G::HIST_OFF);
    uint32_t* match_scratch = reinterpret_cast<uint32_t*>(smem + G::MATCH_OFF);
    uint32_t* scan32 = reinterpret_cast<uint32_t*>(smem + G::SCAN_OFF);
    SegItem* s_seg = reinterpret_cast<SegItem*>(smem + G::SEG_OFF);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int kind = p.kind, desc = p.desc;
    if constexpr (RBITS == 8) {
        for (int i = tid; i < G::WARPS * 256; i += THREADS) match_scratch[i] = 0u;
    }
    U* gkeys = static_cast<U*>(p.keys);
    V* gvals = static_cast<V*>(p.vals);
    const uint32_t lt = lanemask_lt();
    uint32_t* wh = whist + warp * BINS;
    uint32_t* mb = match_scratch + warp * 256;

    for (;;) {
        if (tid == 0) {
            const uint32_t i = atomicAdd(p.seg_counter, 1u);
            SegItem s{};
            if (i < p.num_segs) s = p.segs[i];
            s.pad = i < p.num_segs;
            *s_seg = s;
        }
        __syncthreads();
        const SegItem sg = *s_seg;
        if (!sg.pad) break;
        const uint32_t cnt = uint32_t(sg.end - sg.begin);
        auto live = [&](int u) { return uint32_t(warp * G::IPW + u * 32) < cnt; };  // warp-uniform

        U keys[IPT];
        V vals[PAIRS ? IPT : 1];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            const uint32_t j = uint32_t(warp * G::IPW + u * 32 + lane);
            if (j < cnt) {
                keys[u] = twiddle_in<U>(gkeys[sg.begin + j], kind, desc);
                if constexpr (PAIRS) vals[u] = gvals[sg.begin + j];
            } else {
                keys[u] = U(~U(0));  // filler: after every valid key
            }
        }
        int last_buf = 0;
        for (int pass = 0; pass < G::PASSES; ++pass) {
            uint8_t* buf = smem + size_t(pass & 1) * G::BUF_BYTES;
            U* sk = reinterpret_cast<U*>(buf);
            V* sv = reinterpret_cast<V*>(buf + G::VAL_OFF);
            for (int i = lane; i < BINS; i += 32) wh[i] = 0u;
            __syncwarp();
#pragma unroll
            for (int u = 0; u < IPT; ++u)
                if (live(u)) atomicAdd(&wh[digit_bits<RBITS>(keys[u], pass)], 1u);
            __syncthreads();
            uint32_t total = 0;
            if (tid < BINS) {
#pragma unroll
                for (int w = 0; w < G::WARPS; ++w) {
                    const uint32_t c = whist[w * BINS + tid];
                    whist[w * BINS + tid] = total;
                    total += c;
                }
            }
            uint32_t excl, counted = 0;  // counted: items in live columns (fillers included)
            if constexpr (BINS == 256) {
                excl = block_exclusive_scan_256<uint32_t>(total, scan32, &counted);
            } else {  // one warp scans the bins
                uint32_t v = (tid < BINS) ? total : 0u;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
                    if (lane >= o) v += y;
                }
                excl = v - total;
                counted = __shfl_sync(0xffffffffu, v, BINS - 1);
            }
            if (tid < BINS) {
#pragma unroll
                for (int w = 0; w < G::WARPS; ++w) whist[w * BINS + tid] += excl;
            }
            // one digit holding the whole segment leaves its order unchanged
            const bool uniform = __syncthreads_or(tid < BINS && total == counted);
            uint32_t rank[IPT];
            if (uniform) {
#pragma unroll
                for (int u = 0; u < IPT; ++u) rank[u] = uint32_t(warp * G::IPW + u * 32 + lane);
            } else {
                StaticFor<0, IPT>::run([&](auto uc) {
                    constexpr int u = decltype(uc)::value;
                    if (!live(u)) return;
                    const uint32_t d = digit_bits<RBITS>(keys[u], pass);
                    uint32_t peers;
                    if constexpr (RBITS == 8) peers = warp_match_digit<rank_method(u)>(d, mb, lane, lt);
                    else peers = match_ballot_bits<RBITS>(d);
                    const uint32_t below = __popc(peers & lt);
                    uint32_t old = 0;
                    if (below == 0) old = atomicAdd(&wh[d], uint32_t(__popc(peers)));
                    rank[u] = __shfl_sync(0xffffffffu, old, __ffs(peers) - 1) + below;
                });
            }
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                if (!live(u)) continue;
                sk[rank[u]] = keys[u];
                if constexpr (PAIRS) sv[rank[u]] = vals[u];
            }
            __syncthreads();
            last_buf = pass & 1;
            if (pass + 1 < G::PASSES) {
#pragma unroll
                for (int u = 0; u < IPT; ++u) {
                    if (!live(u)) continue;
                    const int j = warp * G::IPW + u * 32 + lane;
                    keys[u] = sk[j];
                    if constexpr (PAIRS) vals[u] = sv[j];
                }
            }
        }
        // coalesced write-out of the sorted segment
        const uint8_t* buf = smem + size_t(last_buf) * G::BUF_BYTES;
        const U* sk = reinterpret_cast<const U*>(buf);
        const V* sv = reinterpret_cast<const V*>(buf + G::VAL_OFF);
        for (uint32_t i = tid; i < cnt; i += THREADS) {
            gkeys[sg.begin + i] = twiddle_out<U>(sk[i], kind, desc);
            if constexpr (PAIRS) gvals[sg.begin + i] = sv[i];
        }
        __syncthreads();
    }
}

}  // namespace gbsort
