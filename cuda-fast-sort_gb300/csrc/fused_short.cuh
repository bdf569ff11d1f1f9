// fused_short.cuh — the whole sort of a short keys-only array in one
// cooperative launch (sm_103a).
//
// A short array (n <= 2^22, the reference's short mode,
// include/rsort/detail/radix_kernel.cuh:525-559) is latency-bound: each pass
// of the multi-launch path is a chain of dependent global round trips
// (digit offsets, uniform-pass check, tile claim, tile copy, lookback walk,
// next claim, kernel boundary) around a few microseconds of ranking.  Here
// one cooperative launch (every CTA resident at once, or the launch fails)
// runs
//   phase 0: every pass's digit counts from one read of the keys (plus the
//            status clear and, for odd pass counts, the mirror);
//   then, once per CTA, every pass's exclusive digit offsets and the mask of
//            uniform (skipped) passes, kept in shared memory;
//   one phase per executed pass: each CTA ranks its tiles (static
//            round-robin, keys loaded straight into registers) and writes
//            them out as coalesced per-digit runs; a tile's global digit
//            bases come from a two-level prefix instead of a walk over every
//            predecessor: tiles publish their counts, the last tile of each
//            group of 16 publishes the group's sum, and a tile adds the sums
//            of the groups before its own plus its own group's earlier
//            counts — a fixed few round trips however many tiles;
//   the parity fix-up copy when skipped passes leave the result elsewhere;
// with a grid barrier between the phases whose wait is bounded like the
// lookback's (GBSORT_ERR_TIMEOUT, then every CTA leaves).
// The rank is the multi-launch pass's: warp histograms, early publication,
// per-column warp match (shared-memory OR) + popc + one counter atomic per
// digit group, staging at rank in shared memory (radix_kernel.cuh:118-294,
// ranker.cuh:61-170, scatter.cuh:159-202 of the reference).
#pragma once

#include "onesweep.cuh"

namespace gbsort {

// Tiles per group of the two-level prefix.
constexpr uint32_t SHORT_GROUP = 16;

template <int KB, int THREADS, int IPT, int LIPT>
struct ShortGeom {
    static constexpr int P = KB;
    static constexpr int WARPS = THREADS / 32;
    static constexpr int TILE = THREADS * IPT;
    static constexpr int IPW = 32 * IPT;
    // the bucket sort's capacity (keys per bucket one CTA sorts locally)
    static constexpr int LOCAL_TILE = THREADS * LIPT;
    static_assert(LOCAL_TILE >= TILE, "a pass's tile is staged in the first bucket buffer");
    static constexpr size_t LBUF_BYTES = (size_t(LOCAL_TILE) * KB + 127) & ~size_t(127);
    static constexpr size_t STAGE_OFF = 0;                       // U [TILE] (in the bucket buffer)
    static constexpr size_t WHIST_OFF = LBUF_BYTES;              // u32 [WARPS][256]
    static constexpr size_t MATCH_OFF = WHIST_OFF + size_t(WARPS) * 1024;          // u32 [WARPS][256]
    static constexpr size_t COUNT_BYTES = MATCH_OFF + size_t(WARPS) * 1024;        // phase 0 counters here
    static constexpr size_t GEXCL_OFF = COUNT_BYTES;                               // u32 [P][256]
    static constexpr size_t BINB_OFF = GEXCL_OFF + size_t(P) * 1024;               // u32 [256]
    static constexpr size_t SCAN_OFF = BINB_OFF + 1024;                            // u32 [32]
    static constexpr size_t MISC_OFF = SCAN_OFF + 128;  // u32 [4]: uniform mask, largest top bucket
    static constexpr size_t SMEM_BYTES = MISC_OFF + 16;
    static_assert(THREADS >= 256 && THREADS % 32 == 0, "bin owners need 256 threads");
};

// Workspace status words of the short sort: [tiles][256] tile counts, then
// [groups][256] group sums, all tagged with the pass (one clear per sort).
inline size_t short_status_words(uint32_t tiles) {
    return (size_t(tiles) + (tiles + SHORT_GROUP - 1) / SHORT_GROUP) * 256;
}

// Phase 0: every digit count of the whole array into h.gp_counts, using
// smem_bytes of the CTA's shared memory for counters.
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
    auto count = [&](U k) {
        const U t = twiddle_in<U>(k, h.kind, h.desc);
#pragma unroll
        for (int d = 0; d < P; ++d) atomicAdd(&mine[d * 256 + digit_of(t, d)], 1u);
    };
    // 16-byte loads, four in flight per thread before any counting (the
    // unaligned head and the tail by single keys)
    const U* keys = static_cast<const U*>(h.keys);
    const uint64_t n = h.n;
    uint64_t head = ((16u - (reinterpret_cast<uintptr_t>(keys) & 15u)) & 15u) / KB;
    if (head > n) head = n;
    const uint64_t nvec = (n - head) * KB / 16;
    constexpr int PER_VEC = 16 / KB;
    const uint64_t gthreads = uint64_t(gridDim.x) * THREADS;
    const uint64_t gtid = uint64_t(blockIdx.x) * THREADS + tid;
    if (gtid < head) count(keys[gtid]);
    const uint4* vec = reinterpret_cast<const uint4*>(keys + head);
    constexpr int UNROLL = 4;
    for (uint64_t i = gtid; i < nvec; i += UNROLL * gthreads) {
        uint4 v[UNROLL];
#pragma unroll
        for (int r = 0; r < UNROLL; ++r)
            v[r] = (i + r * gthreads < nvec) ? vec[i + r * gthreads] : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int r = 0; r < UNROLL; ++r) {
            if (i + r * gthreads >= nvec) break;
            union { uint4 q; U k[PER_VEC]; } w;
            w.q = v[r];
#pragma unroll
            for (int e = 0; e < PER_VEC; ++e) count(w.k[e]);
        }
    }
    for (uint64_t j = head + nvec * PER_VEC + gtid; j < n; j += gthreads) count(keys[j]);
    __syncthreads();
    for (int b = tid; b < NB; b += THREADS) {
        uint32_t s = 0;
        for (int c = 0; c < copies; ++c) s += cnt[c * NB + b];
        if (s) atomicAdd(&h.gp_counts[b], static_cast<unsigned long long>(s));
    }
}

// Sum of `count` status words of `epoch` at words[0], words[256], ...:
// sixteen loads issued at once; words not yet published are re-read
// together until they are (bounded like every wait: on timeout, or when
// another CTA already flagged an error, a missing word counts 0).
template <class Codec>
__device__ __forceinline__ uint32_t sum_published(const uint32_t* words, uint32_t count, uint32_t epoch,
                                                  uint64_t limit_ns, uint32_t* err) {
    uint32_t sum = 0;
    for (uint32_t i = 0; i < count; i += 16) {
        uint32_t w[16];
        uint32_t pending = 0;
#pragma unroll
        for (int j = 0; j < 16; ++j) w[j] = (i + j < count) ? ld_relaxed_nb(words + size_t(i + j) * 256) : 0u;
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (i + j < count && !Codec::ready(w[j], epoch)) pending |= 1u << j;
        if (pending) {
            const uint64_t t0 = global_timer_ns();
            while (pending) {
                __nanosleep(32);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if ((pending >> j) & 1u) w[j] = ld_relaxed_nb(words + size_t(i + j) * 256);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (((pending >> j) & 1u) && Codec::ready(w[j], epoch)) pending &= ~(1u << j);
                if (pending && (ld_relaxed(err) != 0u || global_timer_ns() - t0 > limit_ns)) {
                    if (ld_relaxed(err) == 0u) atomicOr(err, ERRBIT_TIMEOUT);
#pragma unroll
                    for (int j = 0; j < 16; ++j)
                        if ((pending >> j) & 1u) w[j] = 0u;
                    break;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (i + j < count) sum += uint32_t(Codec::value(w[j]));
    }
    return sum;
}

// One bucket (cnt <= THREADS * LIPT twiddled keys at src) sorted whole in the
// CTA's shared memory over digits 0 .. passes-1, the result written to dst
// with the output twiddle: the batched sort's CTA sort (segmented.cuh), keys
// only, in one buffer (a pass writes it only after the barrier that follows
// every thread's read of the previous pass).  Every warp takes an equal run
// of columns (ceil(cnt / 32 / warps), not LIPT), so a half-full bucket
// still uses all warps and each warp's serial chain of columns is short.  A
// digit held by the whole bucket leaves the order unchanged and skips the
// match.
template <int KB, int THREADS, int LIPT>
__device__ __forceinline__ void cta_bucket_sort(const typename KeyBits<KB>::U* src, typename KeyBits<KB>::U* dst,
                                                uint32_t cnt, int passes, uint8_t* buf, uint32_t* whist,
                                                uint32_t* mscratch, uint32_t* scan, int kind, int desc) {
    using U = typename KeyBits<KB>::U;
    constexpr int WARPS = THREADS / 32;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lt = lanemask_lt();
    uint32_t* wh = whist + warp * 256;
    uint32_t* mb = mscratch + warp * 256;
    const uint32_t cols = (cnt + 32 * WARPS - 1) / (32 * WARPS);  // columns per warp (<= LIPT)
    const uint32_t IPW = 32 * cols;
    auto live = [&](int u) { return uint32_t(u) < cols && uint32_t(warp) * IPW + uint32_t(u) * 32 < cnt; };
    U keys[LIPT];
#pragma unroll
    for (int u = 0; u < LIPT; ++u) {
        const uint32_t j = uint32_t(warp) * IPW + uint32_t(u) * 32 + lane;
        keys[u] = (uint32_t(u) < cols && j < cnt) ? src[j] : U(~U(0));  // filler: after every valid key
    }
    U* sk = reinterpret_cast<U*>(buf);
    for (int pass = 0; pass < passes; ++pass) {
#pragma unroll
        for (int i = lane; i < 256; i += 32) wh[i] = 0u;
        __syncwarp();
#pragma unroll
        for (int u = 0; u < LIPT; ++u)
            if (live(u)) atomicAdd(&wh[digit_of(keys[u], pass)], 1u);
        __syncthreads();
        uint32_t total = 0;
        if (tid < 256) {
#pragma unroll
            for (int w = 0; w < WARPS; ++w) {
                const uint32_t c = whist[w * 256 + tid];
                whist[w * 256 + tid] = total;
                total += c;
            }
        }
        uint32_t counted = 0;  // items in live columns (fillers included)
        const uint32_t excl = block_exclusive_scan_256<uint32_t>(total, scan, &counted);
        if (tid < 256) {
#pragma unroll
            for (int w = 0; w < WARPS; ++w) whist[w * 256 + tid] += excl;
        }
        const bool uniform = __syncthreads_or(tid < 256 && total == counted);
        uint32_t rank[LIPT];
        if (uniform) {
#pragma unroll
            for (int u = 0; u < LIPT; ++u) rank[u] = uint32_t(warp) * IPW + uint32_t(u) * 32 + lane;
        } else {
            StaticFor<0, LIPT>::run([&](auto uc) {
                constexpr int u = decltype(uc)::value;
                if (!live(u)) return;
                const uint32_t d = digit_of(keys[u], pass);
                const uint32_t peers = match_or(d, mb, lane, lt);
                const uint32_t below = __popc(peers & lt);
                uint32_t old = 0;
                if (below == 0) old = atomicAdd(&wh[d], uint32_t(__popc(peers)));
                rank[u] = __shfl_sync(0xffffffffu, old, __ffs(peers) - 1) + below;
            });
        }
#pragma unroll
        for (int u = 0; u < LIPT; ++u)
            if (live(u)) sk[rank[u]] = keys[u];
        __syncthreads();
        if (pass + 1 < passes) {
#pragma unroll
            for (int u = 0; u < LIPT; ++u)
                if (live(u)) keys[u] = sk[uint32_t(warp) * IPW + uint32_t(u) * 32 + lane];
        }
    }
    for (uint32_t i = tid; i < cnt; i += THREADS) dst[i] = twiddle_out<U>(sk[i], kind, desc);
    __syncthreads();  // the buffers and counters are free for the next bucket
}

template <int KB, int THREADS, int IPT, int LIPT, int MIN_CTAS>
__global__ void __launch_bounds__(THREADS, MIN_CTAS) fused_short_kernel(FusedParams f) {
    using U = typename KeyBits<KB>::U;
    using G = ShortGeom<KB, THREADS, IPT, LIPT>;
    using Codec = StatusCodec<uint32_t, KB>;
    extern __shared__ __align__(128) uint8_t smem[];
    U* stage = reinterpret_cast<U*>(smem + G::STAGE_OFF);
    uint32_t* whist = reinterpret_cast<uint32_t*>(smem + G::WHIST_OFF);
    uint32_t* mscratch = reinterpret_cast<uint32_t*>(smem + G::MATCH_OFF);
    uint32_t* gex = reinterpret_cast<uint32_t*>(smem + G::GEXCL_OFF);
    uint32_t* binb = reinterpret_cast<uint32_t*>(smem + G::BINB_OFF);
    uint32_t* scan = reinterpret_cast<uint32_t*>(smem + G::SCAN_OFF);
    uint32_t* misc = reinterpret_cast<uint32_t*>(smem + G::MISC_OFF);

    const PassParams& p = f.pass;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint64_t limit = p.wait_limit_ns;
    uint32_t* err = p.err;
    const uint32_t T = p.num_tiles;
    const uint32_t n = uint32_t(p.n);
    const int kind = p.kind, desc = p.desc;
    uint32_t* partial = static_cast<uint32_t*>(p.status);  // [T][256]
    uint32_t* agg = partial + size_t(T) * 256;              // [groups][256]
    uint32_t phase = 0;

    const uint32_t lt = lanemask_lt();
    uint32_t* wh = whist + warp * 256;
    uint32_t* mb = mscratch + warp * 256;
    // A tile's work in two halves.  Front: keys straight into registers
    // (warp-striped: a warp's lanes read 32 consecutive keys per column, so
    // rank order = input order), warp histograms, per-bin totals and warp
    // bases, early publication of the tile's counts, tile-local digit starts,
    // and — for the last tile of its group of 16 — the group's sum, published
    // before the rank (the group's tiles published their counts at about the
    // same time; every later tile needs the sum after its rank).
    struct TileState {
        uint64_t base;
        uint32_t cnt, excl, valid, in_group, g, g0;
        bool full, leader;
    };
    auto tile_front = [&](int q, uint32_t t, const U* kin, bool tw_load, U (&keys)[IPT], TileState& st) {
        const uint32_t epoch = uint32_t(q);
        st.base = uint64_t(t) * G::TILE;
        st.cnt = (n - st.base) < uint64_t(G::TILE) ? uint32_t(n - st.base) : uint32_t(G::TILE);
        st.full = st.cnt == uint32_t(G::TILE);
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            const uint32_t j = uint32_t(warp * G::IPW + u * 32 + lane);
            const bool in = st.full || j < st.cnt;
            keys[u] = in ? kin[st.base + j] : U(~U(0));  // filler sorts last
            if (tw_load && in) keys[u] = twiddle_in<U>(keys[u], kind, desc);
        }
#pragma unroll
        for (int i = lane; i < 256; i += 32) wh[i] = 0u;
        __syncwarp();
#pragma unroll
        for (int u = 0; u < IPT; ++u) atomicAdd(&wh[digit_of(keys[u], q)], 1u);
        __syncthreads();
        uint32_t tot = 0;
        st.valid = 0;
        if (tid < 256) {
#pragma unroll
            for (int w = 0; w < G::WARPS; ++w) {
                const uint32_t c = whist[w * 256 + tid];
                whist[w * 256 + tid] = tot;
                tot += c;
            }
            st.valid = tot - ((tid == 255) ? (uint32_t(G::TILE) - st.cnt) : 0u);
            st_relaxed(partial + size_t(t) * 256 + tid, Codec::pack(Codec::PARTIAL, epoch, st.valid));
        }
        st.g = t / SHORT_GROUP;
        st.g0 = st.g * SHORT_GROUP;
        st.in_group = 0;
        st.leader = t % SHORT_GROUP == SHORT_GROUP - 1 || t + 1 == T;
        if (st.leader && tid < 256) {
            st.in_group = sum_published<Codec>(partial + size_t(st.g0) * 256 + tid, t - st.g0, epoch, limit, err);
            st_relaxed(agg + size_t(st.g) * 256 + tid, Codec::pack(Codec::PARTIAL, epoch, st.in_group + st.valid));
        }
        st.excl = block_exclusive_scan_256<uint32_t>(tot, scan, nullptr);
        if (tid < 256) {
#pragma unroll
            for (int w = 0; w < G::WARPS; ++w) whist[w * 256 + tid] += st.excl;
        }
        __syncthreads();
    };
    // Back: rank (warp match + popc + one counter atomic per digit group),
    // staging at rank, the two-level prefix (earlier groups' sums + this
    // group's earlier tiles) over the pass's global digit offsets `gexq`, and
    // the coalesced write-out, thread-linear over the digit-sorted tile.
    auto tile_back = [&](int q, uint32_t t, U* kout, bool tw_store, const U (&keys)[IPT], const TileState& st,
                         const uint32_t* gexq) {
        const uint32_t epoch = uint32_t(q);
        StaticFor<0, IPT>::run([&](auto uc) {
            constexpr int u = decltype(uc)::value;
            const uint32_t d = digit_of(keys[u], q);
            const uint32_t peers = match_or(d, mb, lane, lt);
            const uint32_t below = __popc(peers & lt);
            uint32_t old = 0;
            if (below == 0) old = atomicAdd(&wh[d], uint32_t(__popc(peers)));
            const uint32_t r = __shfl_sync(0xffffffffu, old, __ffs(peers) - 1) + below;
            stage[r] = keys[u];
        });
        if (tid < 256) {
            const uint32_t in_group =
                st.leader ? st.in_group
                          : sum_published<Codec>(partial + size_t(st.g0) * 256 + tid, t - st.g0, epoch, limit, err);
            const uint32_t earlier = sum_published<Codec>(agg + tid, st.g, epoch, limit, err);
            binb[tid] = gexq[tid] + earlier + in_group - st.excl;
        }
        __syncthreads();
        U ks[IPT];
        uint32_t pos[IPT];
#pragma unroll
        for (int u = 0; u < IPT; ++u) ks[u] = stage[u * THREADS + tid];
#pragma unroll
        for (int u = 0; u < IPT; ++u) pos[u] = binb[digit_of(ks[u], q)] + uint32_t(u * THREADS + tid);
        bool bad = false;
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            if (st.full || uint32_t(u * THREADS + tid) < st.cnt) {
                if (pos[u] < n) kout[pos[u]] = tw_store ? twiddle_out<U>(ks[u], kind, desc) : ks[u];
                else bad = true;
            }
        }
        if (bad) atomicOr(err, ERRBIT_BOUNDS);
    };
    // One digit pass over every tile of this CTA (static round-robin).
    auto run_pass = [&](int q, const U* kin, U* kout, bool tw_load, bool tw_store) {
        for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
            U keys[IPT];
            TileState st;
            tile_front(q, t, kin, tw_load, keys, st);
            tile_back(q, t, kout, tw_store, keys, st, gex + q * 256);
        }
    };
    // The buckets of the top digit (offsets `top`), each sorted by one CTA
    // from the partition `part` home.
    auto bucket_sorts = [&](const U* part, U* home, const uint32_t* top) {
        for (uint32_t b = blockIdx.x; b < 256; b += gridDim.x) {
            const uint32_t begin = top[b], end = (b < 255) ? top[b + 1] : n;
            if (end > begin)  // the top digit is the bucket's: digits below it only
                cta_bucket_sort<KB, THREADS, LIPT>(part + begin, home + begin, end - begin, G::P - 1, smem, whist,
                                                   mscratch, scan, kind, desc);
        }
    };

    const U* msd_src = static_cast<const U*>(p.copy_keys_in ? p.copy_keys_in : p.keys_a);
    U* msd_part = static_cast<U*>(p.keys_b);
    U* msd_home = static_cast<U*>(p.keys_a);
    if (tid == 0) {
        misc[0] = 0u;
        misc[1] = 0u;
    }

    // MSD first (keys of 2 bytes or more, at most one tile per CTA): the
    // partition pass takes the top digit's global counts from its own group
    // sums (every CTA adds all of them up), so no counting phase and no
    // barrier precede it.  The status words start cleared (the host clears
    // them with the control block).  If a bucket is too big for one CTA,
    // nothing has moved yet: once every CTA has read the status words, the
    // counting phase below clears them and every digit takes a pass.
    if (G::P >= 2 && f.msd && T <= gridDim.x) {
        for (int i = tid; i < G::WARPS * 256; i += THREADS) mscratch[i] = 0u;
        __syncthreads();
        constexpr int q = G::P - 1;
        const uint32_t t = blockIdx.x;
        const bool has_tile = t < T;  // CTA-uniform
        U keys[IPT];
        TileState st{};
        if (has_tile) tile_front(q, t, msd_src, true, keys, st);
        uint32_t* top = gex + q * 256;
        uint32_t tot = 0;
        if (tid < 256)
            tot = sum_published<Codec>(agg + tid, (T + SHORT_GROUP - 1) / SHORT_GROUP, uint32_t(q), limit, err);
        const uint32_t ex = block_exclusive_scan_256<uint32_t>(tot, scan, nullptr);
        if (tid < 256) {
            top[tid] = ex;
            atomicMax(&misc[1], tot);
        }
        __syncthreads();
        if (misc[1] <= uint32_t(G::LOCAL_TILE)) {
            if (has_tile) tile_back(q, t, msd_part, false, keys, st, top);
            if (!grid_barrier(f.barrier, f.barrier_gen, ++phase, limit, err)) return;
            if (ld_relaxed(err) != 0u) return;
            bucket_sorts(msd_part, msd_home, top);
            return;  // the result is home: no fix-up
        }
        if (!grid_barrier(f.barrier, f.barrier_gen, ++phase, limit, err)) return;
        if (tid == 0) misc[1] = 0u;
    }

    fused_counts<KB, THREADS>(f.hist, smem, G::COUNT_BYTES);
    if (!grid_barrier(f.barrier, f.barrier_gen, ++phase, limit, err)) return;

    // Every pass's exclusive digit offsets (one warp per pass) and the mask
    // of passes whose digit holds all n keys.
    for (int i = tid; i < G::WARPS * 256; i += THREADS) mscratch[i] = 0u;
    for (int q = warp; q < G::P; q += G::WARPS) {
        uint32_t c[8];
        uint32_t run = 0, uni = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const unsigned long long x = p.gp_all[size_t(q) * 256 + lane * 8 + j];
            uni |= uint32_t(x == p.n);
            c[j] = run;
            run += uint32_t(x);
        }
        uint32_t incl = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) gex[q * 256 + lane * 8 + j] = c[j] + incl - run;
        if (__any_sync(0xffffffffu, uni) && lane == 0) atomicOr(&misc[0], 1u << q);
        if (q == G::P - 1) {  // the largest bucket of the top digit
            uint32_t mx = 0;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const uint32_t next = (j < 7) ? c[j + 1] : run;
                mx = max(mx, next - c[j]);
            }
            mx = __reduce_max_sync(0xffffffffu, mx);
            if (lane == 0) misc[1] = mx;
        }
    }
    __syncthreads();
    const uint32_t all = (G::P >= 32) ? 0xffffffffu : ((1u << G::P) - 1u);
    const uint32_t uniform = p.skip ? (misc[0] & all) : 0u;
    const int total = __popc(~uniform & all);
    if (p.executed && blockIdx.x == 0 && tid == 0) *p.executed = 0x80000000u | uint32_t(total);

    // MSD partition (keys of 2 bytes or more), after the counts of every
    // digit: when every bucket of the top digit fits one CTA's local sort,
    // one pass on the top digit moves the keys into their buckets (caller's
    // buffer or input -> alternate buffer, twiddled), and each CTA then sorts
    // whole buckets in shared memory over the remaining digits and writes
    // them home: one grid-wide exchange instead of one per digit.
    if (G::P >= 2 && f.msd && misc[1] <= uint32_t(G::LOCAL_TILE)) {
        run_pass(G::P - 1, msd_src, msd_part, true, false);
        if (!grid_barrier(f.barrier, f.barrier_gen, ++phase, limit, err)) return;
        if (ld_relaxed(err) != 0u) return;
        bucket_sorts(msd_part, msd_home, gex + (G::P - 1) * 256);
        return;  // the result is home: no fix-up
    }

    int before = 0;  // executed passes so far
    for (int q = 0; q < G::P; ++q) {
        if ((uniform >> q) & 1u) continue;  // one digit holds every key: a no-op pass
        // buffers as the multi-launch passes derive them
        const U* kin;
        U* kout;
        if (p.copy_keys_in) {  // the last executed pass writes the caller's output (a)
            const bool to_a = ((total - 1 - before) & 1) == 0;
            kout = static_cast<U*>(to_a ? p.keys_a : p.keys_b);
            kin = static_cast<const U*>(before == 0 ? p.copy_keys_in : (to_a ? p.keys_b : p.keys_a));
        } else {
            const bool from_b = ((p.start_alt + before) & 1) != 0;
            kin = static_cast<const U*>(from_b ? p.keys_b : p.keys_a);
            kout = static_cast<U*>(from_b ? p.keys_a : p.keys_b);
        }
        const bool tw_load = before == 0, tw_store = before + 1 == total;
        ++before;

        run_pass(q, kin, kout, tw_load, tw_store);
        if (before == total && !f.fixup) break;  // the last pass: nothing reads its output in this launch
        if (!grid_barrier(f.barrier, f.barrier_gen, ++phase, limit, err)) return;
        if (ld_relaxed(err) != 0u) return;  // a failed wait or bounds check: every CTA leaves
    }
    if (f.fixup) fixup_body(f.fix);
}

}  // namespace gbsort
