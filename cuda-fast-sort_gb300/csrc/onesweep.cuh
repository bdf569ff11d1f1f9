// onesweep.cuh — the hot path: global-histogram upsweep and the persistent
// onesweep digit-binning pass, written for sm_103a (GB300).
//
// Reference behaviour followed (AwardOfSky/CUDA-Fast-Sort "rsort" v0.4.0):
//   upsweep      include/rsort/detail/histogram.cuh:88-211 (all digit
//                histograms from one read of the keys)
//   pass kernel  include/rsort/detail/radix_kernel.cuh:118-294 (load +
//                twiddle, rank, lookback, staged scatter), ranker.cuh:61-170
//                (warp histograms, early PARTIAL publication, per-item rank by
//                warp match + popc + leader atomic), lookback.cuh:252-303
//                (per-bin chained lookback), scatter.cuh:159-202 (stage at
//                rank in shared memory, thread-linear coalesced write-out)
// What is GB300-specific here rather than a translation:
//   - persistent CTAs (grid = SMs x resident CTAs) pull tile ids from a
//     per-pass atomic counter and double-buffer tiles: while tile t is ranked
//     and scattered, tile t+1 is already streaming into shared memory by a
//     bulk copy (cp.async.bulk + mbarrier, L2 evict-first);
//   - keys stay twiddled between passes (twiddle on the first load and last
//     store only);
//   - rank via __match_any_sync (one MATCH per 32 items) instead of 8 ballots;
//   - status words carry the pass as epoch, so one clear (fused into the
//     upsweep) serves every pass; all waits are bounded by %globaltimer.
#pragma once

#include <type_traits>

#include "device_common.cuh"
#include "shapes.h"
#include "sort_params.h"

namespace gbsort {

template <int KB>
struct HistGeom {
    static constexpr int P = KB;
    static constexpr int COPIES = P <= 4 ? 32 : (P == 8 ? 16 : 8);
    static constexpr int NBINS = P * 256;
    static constexpr size_t SMEM_BYTES = size_t(NBINS) * COPIES * 4;
};

// Grid-stride copy of `bytes` bytes (16-byte vectors when both sides allow).
__device__ __forceinline__ void grid_copy(void* dst, const void* src, uint64_t bytes) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const uint64_t t0 = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
        const uint64_t nv = bytes >> 4;
        const uint4* s = static_cast<const uint4*>(src);
        uint4* d = static_cast<uint4*>(dst);
        for (uint64_t i = t0; i < nv; i += stride) d[i] = s[i];
        for (uint64_t i = (nv << 4) + t0; i < bytes; i += stride)
            static_cast<uint8_t*>(dst)[i] = static_cast<const uint8_t*>(src)[i];
    } else {
        for (uint64_t i = t0; i < bytes; i += stride)
            static_cast<uint8_t*>(dst)[i] = static_cast<const uint8_t*>(src)[i];
    }
}

// ---------------------------------------------------------------------------
// Upsweep: every digit histogram from one read of the keys.  Counters are
// spread over COPIES lane-private copies ([bin][copy] layout) so the shared
// atomics of a warp land in distinct banks; 16-byte vector loads.
// ---------------------------------------------------------------------------
template <int KB>
__global__ void __launch_bounds__(HIST_THREADS, 1) upsweep_kernel(HistParams p) {
    using U = typename KeyBits<KB>::U;
    using G = HistGeom<KB>;
    extern __shared__ __align__(16) uint32_t cnt[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int copy = lane & (G::COPIES - 1);

    for (int i = tid; i < G::NBINS * G::COPIES / 4; i += HIST_THREADS)
        reinterpret_cast<uint4*>(cnt)[i] = make_uint4(0, 0, 0, 0);
    grid_launch_dependents();  // the first pass may be scheduled; it waits for this grid
    if (p.msd_state) {  // the digit passes' histogram after the MSD kernels
        grid_dependency_wait();
        if (ld_relaxed(p.msd_state) == MSD_OK) return;
    }
    const int dlo = p.digit_lo, dhi = p.digit_hi ? p.digit_hi : G::P;

    // Fused clears / copies that must precede the first pass.
    {
        const uint64_t nv = p.status_bytes >> 4;
        uint4* s = static_cast<uint4*>(p.status);
        const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
        for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + tid; i < nv; i += stride) s[i] = make_uint4(0, 0, 0, 0);
        if (p.mirror_keys) grid_copy(p.mirror_keys, p.keys, p.n * KB);
        if (p.mirror_vals) grid_copy(p.mirror_vals, p.vals, p.val_bytes_total);
    }
    __syncthreads();

    const int kind = p.kind, desc = p.desc;
    // every digit (the usual case, fully unrolled) or the digits in
    // [dlo, dhi): the loop is compiled once for each
    auto sweep = [&](auto all_digits) {
        constexpr bool ALL = decltype(all_digits)::value;
        auto count = [&](U k) {
            const U t = twiddle_in<U>(k, kind, desc);
#pragma unroll
            for (int d = 0; d < G::P; ++d)
                if (ALL || (d >= dlo && d < dhi)) atomicAdd(&cnt[(d * 256 + digit_of(t, d)) * G::COPIES + copy], 1u);
        };
        const U* keys = static_cast<const U*>(p.keys);
        const uint64_t n = p.n;
        const uintptr_t addr = reinterpret_cast<uintptr_t>(keys);
        uint64_t head = ((16u - (addr & 15u)) & 15u) / KB;
        if (head > n) head = n;
        const uint64_t nvec = (n - head) * KB / 16;
        constexpr int PER_VEC = 16 / KB;
        const uint64_t gthreads = uint64_t(gridDim.x) * HIST_THREADS;
        const uint64_t gtid = uint64_t(blockIdx.x) * HIST_THREADS + tid;

        if (gtid < head) count(keys[gtid]);
        const uint4* vec = reinterpret_cast<const uint4*>(keys + head);
        constexpr int UNROLL = 4;  // (8 for the top digit alone: u64 2^27 0.19 -> 0.28 ms)
        uint64_t i = gtid;
        for (; i + (UNROLL - 1) * gthreads < nvec; i += UNROLL * gthreads) {
            uint4 v[UNROLL];
#pragma unroll
            for (int r = 0; r < UNROLL; ++r) v[r] = __ldcs(vec + i + r * gthreads);
#pragma unroll
            for (int r = 0; r < UNROLL; ++r) {
                union { uint4 q; U k[PER_VEC]; } w;
                w.q = v[r];
#pragma unroll
                for (int e = 0; e < PER_VEC; ++e) count(w.k[e]);
            }
        }
        for (; i < nvec; i += gthreads) {
            union { uint4 q; U k[PER_VEC]; } w;
            w.q = __ldcs(vec + i);
#pragma unroll
            for (int e = 0; e < PER_VEC; ++e) count(w.k[e]);
        }
        for (uint64_t j = head + nvec * PER_VEC + gtid; j < n; j += gthreads) count(keys[j]);
    };
    if (dlo == 0 && dhi == G::P) sweep(std::true_type{});
    else sweep(std::false_type{});
    __syncthreads();

    // Reduce the copies: one warp per bin, conflict-free row read.
    for (int bin = dlo * 256 + warp; bin < dhi * 256; bin += HIST_THREADS / 32) {
        uint32_t s = (lane < G::COPIES) ? cnt[bin * G::COPIES + lane] : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0 && s) atomicAdd(&p.gp_counts[bin], static_cast<unsigned long long>(s));
    }
}


// ---------------------------------------------------------------------------
// Onesweep pass geometry and shared-memory layout.
// ---------------------------------------------------------------------------
// What thread 0 tells the CTA about a tile (one copy per buffer).
struct TileInfo {
    unsigned long long base;  // index of the tile's first element
    uint32_t id;              // global tile id (>= num_tiles: no tile)
    uint32_t cnt;             // elements in the tile
    uint32_t seg;             // segment (batched mode)
    uint32_t first;           // first tile of its segment / of the array
    uint32_t last;            // last tile of its segment / of the array
    uint32_t pad;
};

template <int KB, int VB, int THREADS, int IPT>
struct PassGeom {
    static constexpr int WARPS = THREADS / 32;
    static constexpr int TILE = THREADS * IPT;
    static constexpr int IPW = 32 * IPT;
    // +16: a tile starting off the 16-byte grid is copied from the aligned
    // address below it and lands that many bytes into its region.
    // LATE: only keys are double-buffered; each tile's values are copied into
    // one value buffer when the tile starts (they land during its histogram
    // and scan), so a tile costs 2K + V bytes of shared memory, not 2(K + V).
    static constexpr bool LATE = GBSORT_LATE_VALUES != 0 && VB > 0;
    static constexpr size_t KEY_BYTES = size_t(TILE) * KB + 16;
    static constexpr size_t VAL_BYTES = VB ? size_t(TILE) * VB + 16 : 0;
    static constexpr size_t VAL_OFF = (KEY_BYTES + 127) & ~size_t(127);  // values inside a buffer (not LATE)
    static constexpr size_t BUF_BYTES = LATE ? VAL_OFF : (VAL_OFF + VAL_BYTES + 127) & ~size_t(127);
    static constexpr size_t LATE_VAL_OFF = 2 * BUF_BYTES;         // the value buffer (LATE)
    static constexpr size_t HIST_OFF = LATE ? LATE_VAL_OFF + ((VAL_BYTES + 127) & ~size_t(127))
                                            : 2 * BUF_BYTES;     // u32 [WARPS][256]
    // HALF: per half-warp digit words [position:16 | lane mask:16] replace the
    // per-warp counters and the per-warp match words
    static constexpr bool HALF = GBSORT_RANK_HALF != 0;
    static constexpr int HIST_ROWS = HALF ? 2 * WARPS : WARPS;
    static constexpr int HPW = 16 * IPT;  // HALF: items per half-warp
    static constexpr size_t GEXCL_OFF = HIST_OFF + size_t(HIST_ROWS) * 256 * 4;  // u64 [256]
    static constexpr size_t BINB_OFF = GEXCL_OFF + 256 * 8;       // u64 [256]
    static constexpr size_t SCAN64_OFF = BINB_OFF + 256 * 8;      // u64 [8]
    static constexpr size_t SCAN32_OFF = SCAN64_OFF + 64;         // u32 [8]
    static constexpr size_t MBAR_OFF = SCAN32_OFF + 64;           // u64 [3]: buffers 0, 1, values
    static constexpr size_t INFO_OFF = MBAR_OFF + 32;             // TileInfo [2]
    static constexpr size_t BINB32_OFF = INFO_OFF + 2 * sizeof(TileInfo);  // u32 [256]
    static constexpr size_t MATCH_OFF = BINB32_OFF + 256 * 4;     // u32 [WARPS][256] when RANK_OR is used
    // u32 [4]: [0] uniform-pass mask (prologue), [1] this tile is uniform
    static constexpr size_t SKIP_OFF = MATCH_OFF + ((!HALF && rank_uses_or(IPT)) ? size_t(WARPS) * 256 * 4 : 0);
    static_assert(!HALF || TILE <= 65535, "HALF packs tile positions into 16 bits");
    static constexpr size_t SMEM_BYTES = SKIP_OFF + 16;
    static_assert(THREADS >= 256 && THREADS % 32 == 0, "bin owners need 256 threads");
    static_assert(TILE % 16 == 0, "plain tiles start on the 16-byte grid");
    // offset of the values of the tile in buffer b
    __host__ __device__ static constexpr size_t val_off(int b) {
        return LATE ? LATE_VAL_OFF : size_t(b) * BUF_BYTES + VAL_OFF;
    }
};

// One onesweep digit pass.  SEG = false: one array of n keys.  SEG = true:
// many independent segments; global tile g is p.tiles[g] (segment, base,
// count), each segment's first tile publishes an inclusive prefix of its own
// so lookback chains never cross segments, and digit bases come per segment
// from p.seg_gofs.
// The pass as a device function, run once by the pass kernel below.
template <int KB, int VB, class W, int THREADS, int IPT, bool SEG, int LBW>
__device__ __forceinline__ void onesweep_pass_body(const PassParams& p, uint8_t* smem) {
    using U = typename KeyBits<KB>::U;
    using V = typename ValBits<VB>::V;
    using G = PassGeom<KB, VB, THREADS, IPT>;
    using Codec = StatusCodec<W, KB>;
    constexpr bool PAIRS = VB > 0;
    uint32_t* whist = reinterpret_cast<uint32_t*>(smem + G::HIST_OFF);
    unsigned long long* gexcl = reinterpret_cast<unsigned long long*>(smem + G::GEXCL_OFF);
    unsigned long long* binb = reinterpret_cast<unsigned long long*>(smem + G::BINB_OFF);
    unsigned long long* scan64 = reinterpret_cast<unsigned long long*>(smem + G::SCAN64_OFF);
    uint32_t* scan32 = reinterpret_cast<uint32_t*>(smem + G::SCAN32_OFF);
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + G::MBAR_OFF);
    TileInfo* info_slot = reinterpret_cast<TileInfo*>(smem + G::INFO_OFF);
    uint32_t* binb32 = reinterpret_cast<uint32_t*>(smem + G::BINB32_OFF);
    uint32_t* match_scratch = reinterpret_cast<uint32_t*>(smem + G::MATCH_OFF);
    if constexpr (!G::HALF && rank_uses_or(IPT)) {
        for (int i = threadIdx.x; i < G::WARPS * 256; i += THREADS) match_scratch[i] = 0u;
    }
    // Launched as a dependent of the previous kernel of the sort (plain mode):
    // let the next one be scheduled, then wait for this one's inputs.  Every
    // CTA of a pass is resident at once (grid <= SMs x occupancy), so the
    // successor never holds slots a CTA of this pass still needs.
    grid_launch_dependents();
    grid_dependency_wait();
    if (p.msd_state && ld_relaxed(p.msd_state) == MSD_OK) return;  // the MSD kernels sorted

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // Tile position of item u of this thread: warp-striped (a warp's 32 lanes
    // read 32 consecutive keys per column), or with HALF half-warp-striped
    // (each half-warp owns a contiguous run, so its own counters rank stably).
    auto item = [&](int u) -> uint32_t {
        if constexpr (G::HALF)
            return uint32_t((warp * 2 + (lane >> 4)) * G::HPW + u * 16 + (lane & 15));
        else
            return uint32_t(warp * G::IPW + u * 32 + lane);
    };
    const uint32_t T = p.num_tiles;
    const uint64_t n = p.n;
    const int pass = p.pass, kind = p.kind, desc = p.desc;
    const uint32_t epoch = uint32_t(pass);
    W* status = static_cast<W*>(p.status);
    const void* keys_in = p.keys_in;
    void* keys_out = p.keys_out;
    const void* vals_in = p.vals_in;
    void* vals_out = p.vals_out;
    int twiddle_load = p.twiddle_load, twiddle_store = p.twiddle_store;
    {
        if (p.skip || p.copy_keys_in) {
            uint32_t uniform = 0;
            const uint32_t all = (p.passes >= 32) ? 0xffffffffu : ((1u << p.passes) - 1u);
            if (p.skip) {
                if constexpr (SEG) {
                    // the batched scan marked every pass whose digit varies in some segment
                    uniform = ~ld_relaxed(p.nonuniform_mask) & all;
                } else {
                    // a pass is uniform when one digit holds all n keys
                    uint32_t* smask = reinterpret_cast<uint32_t*>(smem + G::SKIP_OFF);
                    if (tid == 0) *smask = 0u;
                    __syncthreads();
                    if (tid < 256) {
                        uint32_t m = 0;
                        for (int q = 0; q < p.passes; ++q)
                            m |= uint32_t(p.gp_all[size_t(q) * 256 + tid] == n) << q;
                        if (m) atomicOr(smask, m);
                    }
                    __syncthreads();
                    uniform = *smask;
                }
                if ((uniform >> pass) & 1u) return;  // every CTA of this pass leaves: a no-op pass
            }
            const int before = __popc(~uniform & ((1u << pass) - 1u));  // executed passes before this one
            const int total = __popc(~uniform & all);
            if (p.copy_keys_in) {
                // the last executed pass writes the caller's output (a)
                const bool to_a = ((total - 1 - before) & 1) == 0;
                keys_out = to_a ? p.keys_a : p.keys_b;
                vals_out = to_a ? p.vals_a : p.vals_b;
                keys_in = before == 0 ? p.copy_keys_in : (to_a ? p.keys_b : p.keys_a);
                vals_in = before == 0 ? p.copy_vals_in : (to_a ? p.vals_b : p.vals_a);
            } else {
                const bool from_b = ((p.start_alt + before) & 1) != 0;
                keys_in = from_b ? p.keys_b : p.keys_a;
                keys_out = from_b ? p.keys_a : p.keys_b;
                vals_in = from_b ? p.vals_b : p.vals_a;
                vals_out = from_b ? p.vals_a : p.vals_b;
            }
            twiddle_load = before == 0;
            twiddle_store = before + 1 == total;
            if constexpr (!SEG) {
                if (p.executed && blockIdx.x == 0 && tid == 0) *p.executed = 0x80000000u | uint32_t(total);
            }
        }
    }
    const U* gkeys_in = static_cast<const U*>(keys_in);
    const V* gvals_in = static_cast<const V*>(vals_in);

    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        mbar_init(&mbar[2], 1);
        fence_mbar_init();
    }
    if constexpr (!SEG) {  // global exclusive digit offsets of this pass (once per CTA)
        const unsigned long long c = (tid < 256) ? p.gp_counts[tid] : 0ull;
        const unsigned long long ex = block_exclusive_scan_256<unsigned long long>(c, scan64, nullptr);
        if (tid < 256) gexcl[tid] = ex;
    }

    // Thread 0: describe tile t (its table entry `rec` in batched mode).
    auto make_info = [&](uint32_t t, const TileRec& rec) {
        TileInfo ti{};
        ti.id = t;
        if (t >= T) return ti;
        if constexpr (SEG) {
            ti.base = rec.base;
            ti.cnt = rec.cnt;
            ti.seg = rec.seg_flags >> 2;
            ti.first = rec.seg_flags & 1u;
            ti.last = (rec.seg_flags >> 1) & 1u;
        } else {
            ti.base = uint64_t(t) * G::TILE;
            const uint64_t rem = n - ti.base;
            ti.cnt = rem < uint64_t(G::TILE) ? uint32_t(rem) : uint32_t(G::TILE);
            ti.first = t == 0;
            ti.last = t + 1 == T;
        }
        return ti;
    };
    auto load_rec = [&](uint32_t t) {
        TileRec r{};
        if constexpr (SEG) {
            if (t < T) r = p.tiles[t];
        }
        return r;
    };
    // Bulk copies of a tile into buffer `slot`, from the 16-byte-aligned
    // address at or below the tile's start; the ragged tail (< 16 bytes) is
    // left to plain loads.
    auto issue_tile = [&](const TileInfo& ti, int slot) {
        uint8_t* buf = smem + size_t(slot) * G::BUF_BYTES;
        uint32_t kbytes = 0, vbytes = 0;
        const uint64_t pol = l2_evict_first_policy();
        const uintptr_t ka = reinterpret_cast<uintptr_t>(gkeys_in + ti.base);
        const uint32_t mk = uint32_t(ka & 15u);
        if (p.tma_keys) kbytes = (mk + ti.cnt * uint32_t(KB)) & ~15u;
        uint32_t mv = 0;
        uintptr_t va = 0;
        if constexpr (PAIRS && !G::LATE) {
            va = reinterpret_cast<uintptr_t>(gvals_in + ti.base);
            mv = uint32_t(va & 15u);
            if (p.tma_vals) vbytes = (mv + ti.cnt * uint32_t(VB)) & ~15u;
        }
        mbar_arrive_expect_tx(&mbar[slot], kbytes + vbytes);
        if (kbytes) bulk_copy_g2s(buf, reinterpret_cast<const void*>(ka - mk), kbytes, &mbar[slot], pol);
        if (PAIRS && vbytes)
            bulk_copy_g2s(smem + G::val_off(slot), reinterpret_cast<const void*>(va - mv), vbytes, &mbar[slot],
                          pol);
    };
    // LATE: the values of tile ti into the value buffer (barrier 2).
    auto issue_vals = [&](const TileInfo& ti) {
        const uintptr_t va = reinterpret_cast<uintptr_t>(gvals_in + ti.base);
        const uint32_t mv = uint32_t(va & 15u);
        const uint32_t vbytes = p.tma_vals ? ((mv + ti.cnt * uint32_t(VB)) & ~15u) : 0u;
        mbar_arrive_expect_tx(&mbar[2], vbytes);
        if (vbytes)
            bulk_copy_g2s(smem + G::LATE_VAL_OFF, reinterpret_cast<const void*>(va - mv), vbytes, &mbar[2],
                          l2_evict_first_policy());
    };

    // Tile ids come from the pass's atomic counter.  Thread 0 claims the next
    // tile when the current one starts and bulk-copies it into the other
    // buffer meanwhile (GBSORT_TILE_LOOKAHEAD 3 claims two more ahead).
#if GBSORT_TILE_LOOKAHEAD >= 3
    uint32_t id_an = 0, id_aan = 0;  // thread 0: ids of the tiles after next
    TileRec rec_an{};                // thread 0: table entry of id_an
#endif
    __syncthreads();
    if (tid == 0) {
        const uint32_t t0 = atomicAdd(p.tile_counter, 1u);
        const TileInfo i0 = make_info(t0, load_rec(t0));
        info_slot[0] = i0;
        if (t0 < T) issue_tile(i0, 0);
#if GBSORT_TILE_LOOKAHEAD >= 3
        id_an = t0 < T ? atomicAdd(p.tile_counter, 1u) : T;
        rec_an = load_rec(id_an);
        id_aan = id_an < T ? atomicAdd(p.tile_counter, 1u) : T;
#endif
    }
    __syncthreads();
    TileInfo cur = info_slot[0];
    uint32_t parity = 0;  // bit s: parity of the next wait on buffer s
    uint32_t vparity = 0;  // LATE: parity of the next wait on the value buffer
    uint32_t it = 0;

    bool next_issued = false;  // thread 0 only: a copy into the other buffer is in flight
    while (cur.id < T) {
        const int b = int(it & 1u);
        if (tid == 0) {
            if constexpr (G::LATE) {  // this tile's values first: they are needed sooner
                fence_proxy_async_smem();
                issue_vals(cur);
            }
#if GBSORT_TILE_LOOKAHEAD >= 3
            const TileInfo ni = make_info(id_an, rec_an);
#else  // claim the next tile only now: a CTA holds two claims at most
            const uint32_t nid = atomicAdd(p.tile_counter, 1u);
            const TileInfo ni = make_info(nid, load_rec(nid));
#endif
            info_slot[(it + 1) & 1u] = ni;
            next_issued = ni.id < T;
            if (next_issued) {
                fence_proxy_async_smem();
                issue_tile(ni, b ^ 1);
#if GBSORT_TILE_LOOKAHEAD >= 3
                rec_an = load_rec(id_aan);
                id_an = id_aan;
                id_aan = id_aan < T ? atomicAdd(p.tile_counter, 1u) : T;
#endif
            }
        }
        unsigned long long seg_base_d = 0;  // batched: this tile's segment's digit base (bin owners)
        if constexpr (SEG) {
            if (tid < 256) seg_base_d = p.seg_gofs[size_t(cur.seg) * 256 + tid];
        }
        const bool landed = mbar_wait_bounded(&mbar[b], (parity >> b) & 1u, p.wait_limit_ns, p.err);
        parity ^= (1u << b);

        const uint32_t cnt = cur.cnt;
        const bool full = cnt == uint32_t(G::TILE);
        uint8_t* buf = smem + size_t(b) * G::BUF_BYTES;
        U* sk = reinterpret_cast<U*>(buf);                 // staging (aligned)
        V* sv = reinterpret_cast<V*>(smem + G::val_off(b));

        // ---- load the tile into registers (warp-striped: stable rank order)
        U keys[IPT];
        V vals[PAIRS ? IPT : 1];
        const uint32_t mk = uint32_t(reinterpret_cast<uintptr_t>(gkeys_in + cur.base) & 15u);
        const uint32_t mv = PAIRS ? uint32_t(reinterpret_cast<uintptr_t>(gvals_in + cur.base) & 15u) : 0u;
        const bool fast =
            full && mk == 0 && p.tma_keys && (!PAIRS || G::LATE || (mv == 0 && p.tma_vals));
        if (fast) {
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                const uint32_t j = item(u);
                keys[u] = sk[j];
                if constexpr (PAIRS && !G::LATE) vals[u] = sv[j];
            }
        } else {
            const uint32_t kbytes = p.tma_keys ? ((mk + cnt * uint32_t(KB)) & ~15u) : 0u;
            const uint32_t vbytes = (PAIRS && p.tma_vals) ? ((mv + cnt * uint32_t(VB)) & ~15u) : 0u;
            const U* ski = reinterpret_cast<const U*>(buf + mk);
            const V* svi = reinterpret_cast<const V*>(smem + G::val_off(b) + mv);
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                const uint32_t j = item(u);
                if (j < cnt) {
                    keys[u] = (mk + (j + 1) * KB <= kbytes) ? ski[j] : gkeys_in[cur.base + j];
                    if constexpr (PAIRS && !G::LATE)
                        vals[u] = (mv + (j + 1) * VB <= vbytes) ? svi[j] : gvals_in[cur.base + j];
                } else {
                    keys[u] = U(~U(0));  // tail filler: sorts after every valid key
                }
            }
        }
        if (twiddle_load) {
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                const uint32_t j = item(u);
                if (full || j < cnt) keys[u] = twiddle_in<U>(keys[u], kind, desc);
            }
        }

        // ---- warp-private digit histograms (early counts)
        // HALF: one row per half-warp, counts in the upper 16 bits
        uint32_t* wh = whist + (G::HALF ? (warp * 2 + (lane >> 4)) : warp) * 256;
        uint32_t* uniform_tile = reinterpret_cast<uint32_t*>(smem + G::SKIP_OFF) + 1;
        if constexpr (GBSORT_TILE_SHORTCUT) {
            if (tid == 0) *uniform_tile = 0u;  // the last tile's readers passed its final barrier
        }
        {
            constexpr int ROW_WORDS = (G::HALF ? 2 : 1) * 256;
            uint32_t* mine = whist + warp * ROW_WORDS;
#pragma unroll
            for (int i = lane; i < ROW_WORDS; i += 32) mine[i] = 0u;
        }
        __syncwarp();
        constexpr uint32_t ONE = G::HALF ? (1u << 16) : 1u;
#pragma unroll
        for (int u = 0; u < IPT; ++u) atomicAdd(&wh[digit_of(keys[u], pass)], ONE);
        if (__syncthreads_or(!landed)) {
            // A bulk copy did not land within the limit (error word already
            // set).  Publish nothing computed from this buffer — garbage counts
            // could steer successors' writes — drain the copies still in
            // flight (bounded) and leave; successors' lookback waits run out
            // and the launch completes with the error reported.
            if (tid == 0) {
                mbar_wait_bounded(&mbar[b], ((parity >> b) & 1u) ^ 1u, DRAIN_LIMIT_NS, p.err);
                if (next_issued) mbar_wait_bounded(&mbar[b ^ 1], (parity >> (b ^ 1)) & 1u, DRAIN_LIMIT_NS, p.err);
                if constexpr (G::LATE) mbar_wait_bounded(&mbar[2], vparity, DRAIN_LIMIT_NS, p.err);
            }
            return;
        }
        const TileInfo next_info = info_slot[(it + 1) & 1u];

        // ---- per-bin tile totals, warp bases, early PARTIAL publication
        uint32_t total = 0, valid_total = 0;
        W lb_pre[LBW];
        if (tid < 256) {
#pragma unroll
            for (int w = 0; w < G::HIST_ROWS; ++w) {
                const uint32_t c = G::HALF ? (whist[w * 256 + tid] >> 16) : whist[w * 256 + tid];
                whist[w * 256 + tid] = G::HALF ? (total << 16) : total;
                total += c;
            }
            valid_total = total - ((tid == 255) ? (uint32_t(G::TILE) - cnt) : 0u);
            if (GBSORT_TILE_SHORTCUT && total == uint32_t(G::TILE)) *uniform_tile = 1u;  // all keys: this digit
            st_relaxed(status + size_t(cur.id) * 256 + tid,
                       Codec::pack(cur.first ? Codec::GLOBAL : Codec::PARTIAL, epoch, valid_total));
#if GBSORT_LOOKBACK_PREFETCH
            // first lookback round trip overlaps the scan and the rank
            if (!cur.first) lookback_prefetch<LBW>(status, cur.id, tid, lb_pre);
#endif
        }
        const uint32_t excl = block_exclusive_scan_256<uint32_t>(total, scan32, nullptr);
        if (tid < 256) {
#pragma unroll
            for (int w = 0; w < G::HIST_ROWS; ++w) whist[w * 256 + tid] += G::HALF ? (excl << 16) : excl;
        }
        // LATE: this tile's values, copied in since the tile started.  A copy
        // that did not land in time leaves garbage values (positions are
        // unaffected, the error word is set); the CTA stops after this tile.
        bool vfail = false;
        if constexpr (G::LATE) {
            vfail = !mbar_wait_bounded(&mbar[2], vparity, p.wait_limit_ns, p.err);
            vparity ^= 1u;
            const uint32_t vbytes = p.tma_vals ? ((mv + cnt * uint32_t(VB)) & ~15u) : 0u;
            const V* svi = reinterpret_cast<const V*>(smem + G::LATE_VAL_OFF + mv);
            if (full && mv == 0 && p.tma_vals) {
#pragma unroll
                for (int u = 0; u < IPT; ++u) vals[u] = svi[item(u)];
            } else {
#pragma unroll
                for (int u = 0; u < IPT; ++u) {
                    const uint32_t j = item(u);
                    if (j < cnt) vals[u] = (mv + (j + 1) * VB <= vbytes) ? svi[j] : gvals_in[cur.base + j];
                }
            }
        }
        __syncthreads();

        // ---- rank: warp match + popc + one shared atomic per digit group;
        // the group's base comes from the leader (lowest lane) by shuffle.
        uint32_t rank[IPT];
        if (GBSORT_TILE_SHORTCUT && *uniform_tile) {
            // Block-level short-circuit: one digit holds the whole tile, so
            // the stable order is the input order.
#pragma unroll
            for (int u = 0; u < IPT; ++u) rank[u] = item(u);
        } else if constexpr (G::HALF) {
            // Packed half-warp words: one OR registers the lane in its digit's
            // word, one read returns the peers (low 16 bits) and the group's
            // next position (high 16 bits), and the group's lowest lane stores
            // the advanced position with the mask cleared.
            const uint32_t bit = 1u << (lane & 15);
            const uint32_t lt16 = bit - 1u;
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                const uint32_t d = digit_of(keys[u], pass);
                atomicOr(&wh[d], bit);
                __syncwarp();
                const uint32_t w = wh[d];
                const uint32_t peers = w & 0xFFFFu;
                const uint32_t below = __popc(peers & lt16);
                rank[u] = (w >> 16) + below;
                __syncwarp();
                if (below == 0) wh[d] = (w & 0xFFFF0000u) + (uint32_t(__popc(peers)) << 16);
                __syncwarp();
            }
        } else {
            const uint32_t lt = lanemask_lt();
            uint32_t* mb = match_scratch + warp * 256;
            StaticFor<0, IPT>::run([&](auto uc) {
                constexpr int u = decltype(uc)::value;
                const uint32_t d = digit_of(keys[u], pass);
                const uint32_t peers = warp_match_digit<rank_method(u)>(d, mb, lane, lt);
                const uint32_t below = __popc(peers & lt);
#if GBSORT_RANK_LEADER_BRANCH
                uint32_t old = 0;
                if (below == 0) old = atomicAdd(&wh[d], uint32_t(__popc(peers)));
#else
                // every lane issues the atomic, non-leaders add 0: no divergence
                const uint32_t old = atomicAdd(&wh[d], below == 0 ? uint32_t(__popc(peers)) : 0u);
#endif
                rank[u] = __shfl_sync(0xffffffffu, old, __ffs(peers) - 1) + below;
            });
        }

        // ---- stage at rank: every thread read its input before the first
        // barrier of this tile, so the buffer is free; keys/ranks die here,
        // which leaves the registers to the lookback window.
        bool bad = false;
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
#if GBSORT_DEBUG_CHECKS
            if (rank[u] >= uint32_t(G::TILE)) {
                bad = true;
                continue;
            }
#endif
            sk[rank[u]] = keys[u];
            if constexpr (PAIRS) sv[rank[u]] = vals[u];
        }

        // ---- decoupled lookback (bin owners), GLOBAL publication, bases
        if (tid < 256) {
            unsigned long long prefix = 0;
            if (!cur.first) {
#if GBSORT_LOOKBACK_PREFETCH
                prefix = lookback_finish<Codec, LBW>(status, cur.id, tid, lb_pre, epoch, p.wait_limit_ns, p.err);
#else
                prefix = lookback_window<Codec, LBW>(status, cur.id, tid, epoch, p.wait_limit_ns, p.err);
#endif
                if (!cur.last)
                    st_relaxed(status + size_t(cur.id) * 256 + tid,
                               Codec::pack(Codec::GLOBAL, epoch, prefix + valid_total));
            }
            const unsigned long long dbase = SEG ? seg_base_d : gexcl[tid];
            const unsigned long long base = dbase + prefix - excl;
            binb[tid] = base;
            binb32[tid] = uint32_t(base);
        }
        __syncthreads();

        // ---- coalesced write-out: thread-linear over the digit-sorted tile
        U* okeys = static_cast<U*>(keys_out);
        V* ovals = static_cast<V*>(vals_out);
        // Full tiles with 32-bit positions (n < 2^32) take a lean loop: one
        // shared load of the key, of its 32-bit base, one wide-address store.
        auto scatter32 = [&](auto twiddle_tag) {
            constexpr bool TW = decltype(twiddle_tag)::value;
            const uint32_t n32 = uint32_t(n);
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                const uint32_t i = uint32_t(u * THREADS + tid);
                const U k = sk[i];
                const uint32_t pos = binb32[digit_of(k, pass)] + i;
                bool ok = true;
#if GBSORT_BOUNDS_CHECK
                ok = pos < n32;
                bad |= !ok;
#endif
                if (ok) {
                    okeys[pos] = TW ? twiddle_out<U>(k, kind, desc) : k;
                    if constexpr (PAIRS) ovals[pos] = sv[i];
                }
            }
        };
        if (full && n < 0xFFFFFFFFull) {
            if (twiddle_store) scatter32(BoolTag<true>{});
            else scatter32(BoolTag<false>{});
        } else {
            const int tw_store = twiddle_store;
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                const uint32_t i = uint32_t(u * THREADS + tid);
                const U k = sk[i];  // i < TILE: always inside the staging buffer
                const unsigned long long pos = binb[digit_of(k, pass)] + i;
                bool ok = full || i < cnt;
#if GBSORT_BOUNDS_CHECK
                bad |= ok && pos >= n;
                ok = ok && pos < n;
#endif
                if (ok) {
                    okeys[pos] = tw_store ? twiddle_out<U>(k, kind, desc) : k;
                    if constexpr (PAIRS) ovals[pos] = sv[i];
                }
            }
        }
        if (bad) atomicOr(p.err, ERRBIT_BOUNDS);
        if constexpr (G::LATE) {
            if (__syncthreads_or(vfail)) {  // a value copy ran out of time: drain and leave
                if (tid == 0) {
                    mbar_wait_bounded(&mbar[2], vparity ^ 1u, DRAIN_LIMIT_NS, p.err);
                    if (next_issued)
                        mbar_wait_bounded(&mbar[b ^ 1], (parity >> (b ^ 1)) & 1u, DRAIN_LIMIT_NS, p.err);
                }
                return;
            }
        } else {
            __syncthreads();
        }
        cur = next_info;
        ++it;
    }
}

template <int KB, int VB, class W, int THREADS, int IPT, bool SEG, int MIN_CTAS, int LBW>
__global__ void __launch_bounds__(THREADS, MIN_CTAS) onesweep_pass_kernel(PassParams p) {
    extern __shared__ __align__(128) uint8_t smem[];
    onesweep_pass_body<KB, VB, W, THREADS, IPT, SEG, LBW>(p, smem);
}

// Copies `bytes` from src to dst with all threads of the grid (16-byte
// vectors when both ends allow, else 4-byte words, else bytes).
__device__ __forceinline__ void grid_copy_bytes(void* dst, const void* src, uint64_t bytes) {
    const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src);
    uint64_t done = 0;
    if ((a & 15u) == 0) {
        const uint64_t v = bytes / 16;
        for (uint64_t i = t; i < v; i += stride) static_cast<uint4*>(dst)[i] = static_cast<const uint4*>(src)[i];
        done = v * 16;
    } else if ((a & 3u) == 0) {
        const uint64_t v = bytes / 4;
        for (uint64_t i = t; i < v; i += stride)
            static_cast<uint32_t*>(dst)[i] = static_cast<const uint32_t*>(src)[i];
        done = v * 4;
    }
    for (uint64_t i = done + t; i < bytes; i += stride)
        static_cast<uint8_t*>(dst)[i] = static_cast<const uint8_t*>(src)[i];
}

// After uniform-pass skipping: the executed passes' parity left the result
// in the other buffer than the one it belongs in (in place: an odd count
// left it in the alternate buffer); copy it across.  Otherwise nothing to do.
__device__ __forceinline__ void fixup_body(const FixupParams& f) {
    if (f.msd_state && ld_relaxed(f.msd_state) == MSD_OK) return;  // the MSD kernels sorted
    // the executed pass kernels left their count; none ran when the word is 0
    const uint32_t w = *f.executed;
    const int executed = (w >> 31) ? int(w & 0xFFu) : 0;
    if (f.copy_keys_in) {  // input-preserving: only when no pass wrote the output
        if (executed != 0) return;
        grid_copy_bytes(f.keys_a, f.copy_keys_in, f.key_bytes_total);
        if (f.val_bytes_total) grid_copy_bytes(f.vals_a, f.copy_vals_in, f.val_bytes_total);
        return;
    }
    if ((executed & 1) == f.want_odd) return;
    // the result sits in b after an odd number of executed passes, else in a
    const bool in_b = (executed & 1) != 0;
    grid_copy_bytes(in_b ? f.keys_a : f.keys_b, in_b ? f.keys_b : f.keys_a, f.key_bytes_total);
    if (f.val_bytes_total) grid_copy_bytes(in_b ? f.vals_a : f.vals_b, in_b ? f.vals_b : f.vals_a, f.val_bytes_total);
}

}  // namespace gbsort
