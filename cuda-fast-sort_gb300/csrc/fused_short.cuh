// fused_short.cuh — the whole sort of a short keys-only array in one
// cooperative launch (sm_103a).
//
// A short array (n <= 2^22, the reference's short mode,
// include/rsort/detail/radix_kernel.cuh:525-559) is latency-bound: each pass
// of the multi-launch path is a chain of dependent global round trips
// (digit offsets, uniform-pass check, tile claim, tile copy, lookback walk,
// next claim, kernel boundary) around a few microseconds of ranking.  Here
// one cooperative launch (every CTA resident at once, or the launch fails)
// sorts it, with a grid barrier between phases whose wait is bounded like
// the lookback's (GBSORT_ERR_TIMEOUT, then every CTA leaves).
//
// Keys of 2 bytes or more, most significant digit first (keys only, so
// equal twiddled keys are equal bytes and no step needs a stable order):
//   partition: each tile counts its keys per top digit with shared-memory
//            atomics, claims its places in the 256 fixed-capacity regions
//            of the workspace (one per top digit) with one global atomic
//            per digit, and writes its keys there as coalesced runs — no
//            tile waits for another;
//   one grid barrier;
//   buckets: each CTA sorts whole top-digit buckets in shared memory (a
//            counting pass on the next 12-13 bits, then a comparison rank
//            inside the tiny sub-buckets; or, where a sub-bucket is too big,
//            one ranked pass per remaining digit) and writes them to their
//            places in the result.
// A region that would overflow (skewed top digits) sends every CTA, after
// the barrier, to the per-digit flow below, from the untouched input.
//
// Per-digit flow (1-byte keys, and the fallback):
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
//   the parity fix-up copy when skipped passes leave the result elsewhere.
// The per-digit rank is the multi-launch pass's: warp histograms, early
// publication, per-column warp match (shared-memory OR) + popc + one counter
// atomic per digit group, staging at rank in shared memory
// (radix_kernel.cuh:118-294, ranker.cuh:61-170, scatter.cuh:159-202 of the
// reference).
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

// Exclusive scan of one value per thread over the whole CTA (warp_tmp: one
// word per warp).  Every thread must call it.
template <int THREADS>
__device__ __forceinline__ uint32_t block_exclusive_scan_all(uint32_t x, uint32_t* warp_tmp) {
    constexpr int WARPS = THREADS / 32;
    static_assert(WARPS <= 32, "one warp scans the warp totals");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) warp_tmp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint32_t t = (lane < WARPS) ? warp_tmp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < WARPS; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < WARPS) warp_tmp[lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    return (warp > 0 ? warp_tmp[warp - 1] : 0u) + v - x;
}

__host__ __device__ constexpr int floor_log2(int x) { return x <= 1 ? 0 : 1 + floor_log2(x / 2); }

// Largest sub-bucket the split sort ranks by comparison (a key compares
// itself with every key of its sub-bucket).
#ifndef GBSORT_SPLIT_MAX
#define GBSORT_SPLIT_MAX 32
#endif
// 0: every bucket takes the per-digit bucket sort.
#ifndef GBSORT_BUCKET_SPLIT
#define GBSORT_BUCKET_SPLIT 1
#endif

// One bucket (cnt <= THREADS * LIPT twiddled keys that share their top digit,
// already in registers: key u of this thread is the bucket's key
// u * THREADS + tid) sorted by splitting it, keys only.  One counting pass
// over the next RB bits below the top digit (2^RB sub-buckets) moves every
// key into its sub-bucket with a shared-memory atomic, in no particular
// order: equal twiddled keys are equal bytes, so once the keys are in
// order, the order among equal keys cannot show.  A sub-bucket then holds
// the keys of one value of the top 8 + RB bits, cnt / 2^RB on average (about
// half a key at 2^20 keys), and a key's place in it is the number of the
// sub-bucket's other keys below it (equal keys ordered by where the
// counting pass put them), written straight to dst.  Where nothing is left
// below the RB bits (2-byte keys), the counting pass alone sorts.  So the
// bucket costs one counting pass and a comparison or two per key instead
// of a ranked pass per remaining digit.  Returns false, having written
// nothing outside shared memory, when a sub-bucket holds more than
// GBSORT_SPLIT_MAX keys (repeated keys, or keys that share those bits): the
// per-digit bucket sort takes those.
// One word per sub-bucket at ctr (2^RB <= CTR_WORDS words, zero on entry
// and left zeroed; here the warp histograms and the match words after
// them, cleared before the grid barrier that precedes the buckets): the
// count, then start << 16 | cursor (cnt < 2^16).  Sub-bucket b lives in word
// b ^ ((b >> 5) & 31), which puts the scan's runs of 2^k consecutive
// sub-buckets per thread on distinct banks.
__host__ __device__ constexpr int split_slot(int b) { return b ^ ((b >> 5) & 31); }

template <int KB, int THREADS, int LIPT, int CTR_WORDS, int BELOW = 8 * (KB - 1)>
__device__ __forceinline__ bool cta_bucket_split(const typename KeyBits<KB>::U (&keys)[LIPT],
                                                 typename KeyBits<KB>::U* dst, uint32_t cnt, uint8_t* buf,
                                                 uint32_t* ctr, uint32_t* scan, uint32_t* largest, int kind,
                                                 int desc) {
    using U = typename KeyBits<KB>::U;
    // BELOW: key bits below the bits the bucket's keys share (its top digit)
    constexpr int RB_CAP = floor_log2(CTR_WORDS);
    constexpr int RB = RB_CAP < BELOW ? RB_CAP : BELOW;
    constexpr int BINS = 1 << RB;
    static_assert(BINS >= 32 && BINS <= CTR_WORDS, "sub-bucket words");
    static_assert(THREADS * LIPT < 65536, "16-bit starts and cursors");
    constexpr int SHIFT = BELOW - RB;  // key bits left to compare inside a sub-bucket
    constexpr int PER = (BINS + THREADS - 1) / THREADS;
    static_assert((PER & (PER - 1)) == 0 && PER <= 32, "runs of 2^k sub-buckets per thread");
    const int tid = threadIdx.x;
    U* sk = reinterpret_cast<U*>(buf);
    auto slot = [](U k) { return split_slot(int(uint32_t(k >> SHIFT) & uint32_t(BINS - 1))); };
    auto valid = [&](int u) { return uint32_t(u * THREADS + tid) < cnt; };
    if (tid == 0) *largest = 0u;
#pragma unroll
    for (int u = 0; u < LIPT; ++u)
        if (valid(u)) atomicAdd(&ctr[slot(keys[u])], 1u);
    __syncthreads();
    uint32_t c[PER], sum = 0, big = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int b = tid * PER + i;
        c[i] = (b < BINS) ? ctr[split_slot(b)] : 0u;
        sum += c[i];
        big = max(big, c[i]);
    }
    uint32_t run = block_exclusive_scan_all<THREADS>(sum, scan);
    big = __reduce_max_sync(0xffffffffu, big);
    if ((tid & 31) == 0 && big > uint32_t(GBSORT_SPLIT_MAX)) atomicMax(largest, big);
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int b = tid * PER + i;
        if (b < BINS) ctr[split_slot(b)] = run << 16 | run;
        run += c[i];
    }
    __syncthreads();
    if (SHIFT > 0 && *largest > uint32_t(GBSORT_SPLIT_MAX)) {
        for (int i = tid; i < BINS; i += THREADS) ctr[i] = 0u;
        __syncthreads();
        return false;
    }
#pragma unroll
    for (int u = 0; u < LIPT; ++u)
        if (valid(u)) sk[atomicAdd(&ctr[slot(keys[u])], 1u) & 0xffffu] = keys[u];
    __syncthreads();
    if constexpr (SHIFT > 0) {
        // the key at place i goes to its sub-bucket's start plus the
        // sub-bucket's other keys below it: a place near i, so a warp's
        // stores stay nearly coalesced; CH places per thread compared at once
#ifdef GBSORT_SPLIT_CH
        constexpr int CH = GBSORT_SPLIT_CH;
#else
        constexpr int CH = 1;
#endif
        for (uint32_t i0 = tid; i0 < cnt; i0 += CH * THREADS) {
            U k[CH];
            uint32_t st[CH], others[CH], below[CH], most = 0;
#pragma unroll
            for (int u = 0; u < CH; ++u) {
                const uint32_t i = i0 + u * THREADS;
                k[u] = (i < cnt) ? sk[i] : U(0);
            }
#pragma unroll
            for (int u = 0; u < CH; ++u) {
                const uint32_t i = i0 + u * THREADS;
                const uint32_t w = (i < cnt) ? ctr[slot(k[u])] : 0u;
                st[u] = w >> 16;
                others[u] = (i < cnt) ? (w & 0xffffu) - st[u] - 1u : 0u;
                below[u] = 0;
                most = max(most, others[u]);
            }
            for (uint32_t j = 0; j < most; ++j) {
#pragma unroll
                for (int u = 0; u < CH; ++u) {
                    if (j < others[u]) {
                        const uint32_t i = i0 + u * THREADS;
                        const uint32_t q = st[u] + j + uint32_t(st[u] + j >= i);  // every place but i
                        const U o = sk[q];
                        below[u] += uint32_t(o < k[u] || (o == k[u] && q < i));
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < CH; ++u) {
                const uint32_t i = i0 + u * THREADS;
                if (i < cnt) dst[st[u] + below[u]] = twiddle_out<U>(k[u], kind, desc);
            }
        }
    } else {
        for (uint32_t i = tid; i < cnt; i += THREADS) dst[i] = twiddle_out<U>(sk[i], kind, desc);
    }
    __syncthreads();
    for (int i = tid; i < BINS; i += THREADS) ctr[i] = 0u;
    __syncthreads();
    return true;
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
    // MSD partition of one tile (keys of 2 bytes or more): its keys go to
    // the regions of their top digit (f.regions: 256 regions of
    // f.region_cap keys), where the tile claims its places with one atomic
    // per digit on the region's fill count (f.fill) — no tile waits for
    // another, and the order inside a region is arbitrary (keys only: equal
    // twiddled keys are equal bytes, and the bucket sorts need no order).
    // A region that would overflow is not written past its end and raises
    // f.overflow.
    auto partition_tile = [&](uint32_t t, const U* kin, U* regions, uint32_t cap) {
        constexpr int q = G::P - 1;
        uint32_t* gbase = gex;  // [256] the tile's first place in each region
        const uint64_t base = uint64_t(t) * G::TILE;
        const uint32_t cnt = (n - base) < uint64_t(G::TILE) ? uint32_t(n - base) : uint32_t(G::TILE);
        U keys[IPT];
        uint32_t slot[IPT];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            const uint32_t j = uint32_t(u * THREADS + tid);
            keys[u] = (j < cnt) ? twiddle_in<U>(kin[base + j], kind, desc) : U(0);
        }
        if (tid < 256) binb[tid] = 0u;
        __syncthreads();
#pragma unroll
        for (int u = 0; u < IPT; ++u)
            if (uint32_t(u * THREADS + tid) < cnt) slot[u] = atomicAdd(&binb[digit_of(keys[u], q)], 1u);
        __syncthreads();
        uint32_t c = 0, g = 0;
        if (tid < 256) {
            c = binb[tid];
            if (c) {
                g = atomicAdd(f.fill + tid, c);
                if (g + c > cap) atomicOr(f.overflow, 1u);
            }
        }
        const uint32_t ex = block_exclusive_scan_256<uint32_t>(c, scan, nullptr);
        if (tid < 256) binb[tid] = ex;
        __syncthreads();
#pragma unroll
        for (int u = 0; u < IPT; ++u)
            if (uint32_t(u * THREADS + tid) < cnt) stage[binb[digit_of(keys[u], q)] + slot[u]] = keys[u];
        if (tid < 256) gbase[tid] = g;  // the claim's answer: only the write-out needs it
        __syncthreads();
        // coalesced runs, one per digit (each key straight from registers
        // to its region measured slower: 2^20 u32 26.1 vs 23.7 us, partial
        // sector stores from every CTA at once)
        for (uint32_t j = tid; j < cnt; j += THREADS) {
            const U k = stage[j];
            const uint32_t d = digit_of(k, q);
            const uint32_t pos = gbase[d] + (j - binb[d]);
            if (pos < cap) regions[size_t(d) * cap + pos] = k;
        }
        __syncthreads();  // the stage and the digit words are free for the next tile
    };

    // MSD first (keys of 2 bytes or more, when the plan has regions): the
    // partition, one grid barrier, then each CTA sorts whole buckets from
    // their regions into their places in the result (the result is home: no
    // fix-up).  After an overflow every CTA goes on to the per-digit passes
    // below, which start from the untouched input.
    if (tid == 0) misc[0] = 0u;
    if constexpr (G::P >= 2) {
        if (f.msd) {
            // the bucket sorts' counters and match words start zeroed
            for (int i = tid; i < 2 * G::WARPS * 256; i += THREADS) whist[i] = 0u;
            U* regions = static_cast<U*>(f.regions);
            const uint32_t cap = f.region_cap;
            const U* src = static_cast<const U*>(p.copy_keys_in ? p.copy_keys_in : p.keys_a);
            for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) partition_tile(t, src, regions, cap);
            if (!grid_barrier(f.barrier, f.barrier_gen, ++phase, limit, err)) return;
            if (ld_relaxed(err) != 0u) return;
            if (ld_relaxed(f.overflow) == 0u) {
                // every bucket's size and place in the result; the keys of this
                // CTA's first bucket are loaded meanwhile (every place of its
                // region: those past its size are never used)
                uint32_t* top = gex + 256;
                U keys[LIPT];
                const U* first = regions + size_t(blockIdx.x) * cap;
#pragma unroll
                for (int u = 0; u < LIPT; ++u) {
                    const uint32_t j = uint32_t(u * THREADS + tid);
                    keys[u] = (blockIdx.x < 256 && j < cap) ? first[j] : U(0);
                }
                const uint32_t fc = (tid < 256) ? ld_relaxed(f.fill + tid) : 0u;
                const uint32_t ex = block_exclusive_scan_256<uint32_t>(fc, scan, nullptr);
                if (tid < 256) {
                    binb[tid] = fc;
                    top[tid] = ex;
                }
                __syncthreads();
                U* home = static_cast<U*>(p.keys_a);
                // the top digit is the bucket's: digits below it only; the split
                // first, the per-digit sort where a sub-bucket is too big
                auto sort_bucket = [&](uint32_t b, const U (&keys)[LIPT]) {
                    const uint32_t c = binb[b];
                    if (c == 0) return;
                    U* to = home + top[b];
                    if (GBSORT_BUCKET_SPLIT && cta_bucket_split<KB, THREADS, LIPT, 2 * G::WARPS * 256>(
                                                   keys, to, c, smem, whist, scan, misc + 2, kind, desc))
                        return;
                    cta_bucket_sort<KB, THREADS, LIPT>(regions + size_t(b) * cap, to, c, G::P - 1, smem, whist,
                                                       mscratch, scan, kind, desc);
                    for (int i = tid; i < G::WARPS * 256; i += THREADS) whist[i] = 0u;  // the split's counters
                    __syncthreads();
                };
                if (blockIdx.x < 256) sort_bucket(blockIdx.x, keys);
                for (uint32_t b = blockIdx.x + gridDim.x; b < 256; b += gridDim.x) {
                    U more[LIPT];
                    const U* from = regions + size_t(b) * cap;
#pragma unroll
                    for (int u = 0; u < LIPT; ++u) {
                        const uint32_t j = uint32_t(u * THREADS + tid);
                        more[u] = (j < binb[b]) ? from[j] : U(0);
                    }
                    sort_bucket(b, more);
                }
                return;
            }
        }
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
    }
    __syncthreads();
    const uint32_t all = (G::P >= 32) ? 0xffffffffu : ((1u << G::P) - 1u);
    const uint32_t uniform = p.skip ? (misc[0] & all) : 0u;
    const int total = __popc(~uniform & all);
    if (p.executed && blockIdx.x == 0 && tid == 0) *p.executed = 0x80000000u | uint32_t(total);

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
