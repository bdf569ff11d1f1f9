// msd.cuh — keys-only sorts of 8- and 16-byte keys, most significant digit
// first (sm_103a).
//
// A least-significant-digit sort of 16-byte keys makes 16 passes over the
// data (8 for 8-byte keys), each bound by its stable rank.  Keys only, equal
// twiddled keys are equal bytes, so the order among equal keys cannot show
// and no step needs a stable order.  This path instead:
//   top split:    every tile counts its keys per top digit with shared
//                 atomics, claims its places in the digit's range (exact: the
//                 upsweep's counts) with one global atomic per digit, stages
//                 the tile by digit and writes each digit's run — no tile
//                 waits for another (input -> alternate buffer, twiddled);
//   pair count:   tiles of each top bucket count the second digit into
//                 per-(top, second) totals;
//   scan:         one CTA turns the 65536 totals into group offsets and
//                 decides: every group fits a CTA's local sort (MSD_OK), or
//                 not (MSD_OFF);
//   second split: as the top split, within each top bucket, into the groups'
//                 exact ranges (alternate buffer -> caller's buffer);
//   local sorts:  each CTA sorts whole groups in place in shared memory (the
//                 bucket split of fused_short.cuh: a counting pass on the next
//                 11-12 bits, then a comparison rank inside the sub-buckets)
//                 and writes them untwiddled; a group with a sub-bucket too
//                 big for the comparison rank goes back untwiddled unsorted
//                 and turns the state to MSD_OFF.
// With MSD_OFF the least-significant-digit passes, launched after these
// kernels, sort from the caller's buffer, which then holds the input's keys
// in some order (untouched, or as the local sorts left them); with MSD_OK
// they exit at once.
// Every key is read and written three times (plus the upsweep's and the pair
// count's reads): 16-byte keys 2^26 measured 0.38 ms per split against 0.54
// ms per digit pass.
#pragma once

#include "fused_short.cuh"

namespace gbsort {

struct MsdParams {
    const void* keys_in;   // the top split's input: the caller's keys or the input-preserving source
    void* keys_a;          // the caller's buffer (second split's output, sorted in place)
    void* keys_b;          // the alternate buffer (top split's output)
    uint64_t n;
    int kind, desc;
    const unsigned long long* gp_top;  // the upsweep's counts of the top digit [256]
    uint32_t* state;       // MSD_OK / MSD_OFF, zeroed before the sort
    uint32_t* cursor1;     // [256] claimed places per top digit, zeroed
    uint32_t* joint;       // [256 * 256] keys per (top, second) digit, zeroed
    uint32_t* cursor2;     // [256 * 256] claimed places per group, zeroed
    uint32_t* offs2;       // [256 * 256] first place of every group
    uint32_t group_cap;    // largest group a local sort takes
    uint32_t* err;         // workspace error word
};

// The MSD path's first kernel: the top digit's counts of the input into
// h.gp_counts (the row of digit P-1), and the clear of the status words and
// the MSD block (h.status, h.status_bytes).  One digit needs 256 counters
// (32 copies, one per lane: no same-word atomics), so several CTAs fit an
// SM and keep more loads in flight than the all-digit histogram kernel
// (one CTA of 1024 threads an SM for its 128 KB of counters).
constexpr int MSD_HIST_THREADS = 512;
template <int KB>
__global__ void __launch_bounds__(MSD_HIST_THREADS, 2) msd_hist_kernel(HistParams h) {
    using U = typename KeyBits<KB>::U;
    __shared__ uint32_t cnt[256 * 32];
    const int tid = threadIdx.x, lane = tid & 31;
    for (int i = tid; i < 256 * 32; i += MSD_HIST_THREADS) cnt[i] = 0u;
    grid_launch_dependents();
    {
        const uint64_t nv = h.status_bytes >> 4;
        uint4* st = static_cast<uint4*>(h.status);
        const uint64_t stride = uint64_t(gridDim.x) * MSD_HIST_THREADS;
        for (uint64_t i = uint64_t(blockIdx.x) * MSD_HIST_THREADS + tid; i < nv; i += stride)
            st[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();
    const U* keys = static_cast<const U*>(h.keys);
    const uint64_t n = h.n;
    auto count = [&](U k) { atomicAdd(&cnt[digit_of(twiddle_in<U>(k, h.kind, h.desc), KB - 1) * 32 + lane], 1u); };
    uint64_t head = ((16u - (reinterpret_cast<uintptr_t>(keys) & 15u)) & 15u) / KB;
    if (head > n) head = n;
    const uint64_t nvec = (n - head) * KB / 16;
    constexpr int PER_VEC = 16 / KB, UNROLL = 4;
    const uint64_t gthreads = uint64_t(gridDim.x) * MSD_HIST_THREADS;
    const uint64_t gtid = uint64_t(blockIdx.x) * MSD_HIST_THREADS + tid;
    if (gtid < head) count(keys[gtid]);
    const uint4* vec = reinterpret_cast<const uint4*>(keys + head);
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
    __syncthreads();
    // one warp per bin: the 32 copies summed by a shuffle reduction
    for (int bin = tid >> 5; bin < 256; bin += MSD_HIST_THREADS / 32) {
        uint32_t c = cnt[bin * 32 + lane];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0 && c) atomicAdd(&h.gp_counts[size_t(KB - 1) * 256 + bin], static_cast<unsigned long long>(c));
    }
}

// One tile split by one digit: `cnt` keys at src (twiddled on load when
// TWIDDLE) go to dst at base[d] + (their place among the keys of digit d
// that every tile claims from claim[d]), d = the key's digit `q`.  No order
// among a digit's keys.  Shared: stage (the tile), bins / delta / scan.
template <int KB, int THREADS, int IPT, bool TWIDDLE>
__device__ __forceinline__ void msd_load_tile(const typename KeyBits<KB>::U* src, uint32_t cnt, int kind, int desc,
                                              typename KeyBits<KB>::U (&keys)[IPT]) {
    using U = typename KeyBits<KB>::U;
#pragma unroll
    for (int u = 0; u < IPT; ++u) {
        const uint32_t j = uint32_t(u * THREADS + threadIdx.x);
        keys[u] = U(0);
        if (j < cnt) keys[u] = TWIDDLE ? twiddle_in<U>(src[j], kind, desc) : src[j];
    }
}

// The split of a tile whose keys are in registers (msd_load_tile's layout).
template <int KB, int THREADS, int IPT, class Base>
__device__ __forceinline__ void msd_split_loaded(const typename KeyBits<KB>::U (&keys)[IPT], uint32_t cnt, int q,
                                                 uint32_t* claim, Base base, typename KeyBits<KB>::U* dst, uint64_t n,
                                                 uint32_t* err, typename KeyBits<KB>::U* stage, uint32_t* bins,
                                                 uint32_t* delta, uint32_t* scan) {
    using U = typename KeyBits<KB>::U;
    const int tid = threadIdx.x;
    uint32_t slot[IPT];
    if (tid < 256) bins[tid] = 0u;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < IPT; ++u)
        if (uint32_t(u * THREADS + tid) < cnt) slot[u] = atomicAdd(&bins[digit_of(keys[u], q)], 1u);
    __syncthreads();
    uint32_t c = 0, g = 0;
    if (tid < 256) {
        c = bins[tid];
        if (c) g = atomicAdd(claim + tid, c);
    }
    const uint32_t ex = block_exclusive_scan_256<uint32_t>(c, scan, nullptr);
    if (tid < 256) bins[tid] = ex;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < IPT; ++u)
        if (uint32_t(u * THREADS + tid) < cnt) stage[bins[digit_of(keys[u], q)] + slot[u]] = keys[u];
    if (tid < 256) delta[tid] = base(tid) + g - ex;  // the claim's answer: only the write-out needs it
    __syncthreads();
    bool bad = false;
    for (uint32_t j = tid; j < cnt; j += THREADS) {  // coalesced runs, one per digit
        const U k = stage[j];
        const uint32_t pos = delta[digit_of(k, q)] + j;
        if (pos < n) dst[pos] = k;
        else bad = true;
    }
    if (bad) atomicOr(err, ERRBIT_BOUNDS);
    __syncthreads();  // the stage and the digit words are free for the next tile
}

template <int KB, int THREADS, int IPT, bool TWIDDLE, class Base>
__device__ __forceinline__ void msd_split_tile(const typename KeyBits<KB>::U* src, uint32_t cnt, int q, int kind,
                                               int desc, uint32_t* claim, Base base, typename KeyBits<KB>::U* dst,
                                               uint64_t n, uint32_t* err, typename KeyBits<KB>::U* stage,
                                               uint32_t* bins, uint32_t* delta, uint32_t* scan) {
    typename KeyBits<KB>::U keys[IPT];
    msd_load_tile<KB, THREADS, IPT, TWIDDLE>(src, cnt, kind, desc, keys);
    msd_split_loaded<KB, THREADS, IPT>(keys, cnt, q, claim, base, dst, n, err, stage, bins, delta, scan);
}

// Every top bucket's first key, size and first tile of the second level
// (tiles of `tile` keys that never cross a bucket), from the upsweep's
// counts; tfirst[256] = the number of tiles.
__device__ __forceinline__ void msd_top_table(const unsigned long long* gp_top, uint32_t tile, uint32_t* tstart,
                                              uint32_t* tcnt, uint32_t* tfirst, uint32_t* scan) {
    const int tid = threadIdx.x;
    const uint32_t c = (tid < 256) ? uint32_t(gp_top[tid]) : 0u;
    const uint32_t ex = block_exclusive_scan_256<uint32_t>(c, scan, nullptr);
    __syncthreads();  // the scan words are read by every thread before the next scan writes them
    uint32_t tiles = 0;
    const uint32_t tex = block_exclusive_scan_256<uint32_t>((c + tile - 1) / tile, scan, &tiles);
    if (tid < 256) {
        tstart[tid] = ex;
        tcnt[tid] = c;
        tfirst[tid] = tex;
    }
    if (tid == 0) tfirst[256] = tiles;
    __syncthreads();
}

// The top bucket of second-level tile t: the last b with tfirst[b] <= t.
__device__ __forceinline__ uint32_t msd_bucket_of(const uint32_t* tfirst, uint32_t t) {
    uint32_t lo = 0, hi = 256;  // tfirst[lo] <= t < tfirst[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (tfirst[mid] <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

template <int KB, int THREADS, int IPT>
struct MsdSplitGeom {
    static constexpr int TILE = THREADS * IPT;
    static constexpr size_t STAGE_BYTES = size_t(TILE) * KB;
    static constexpr size_t WORDS_OFF = STAGE_BYTES;  // u32 bins[256], delta[256], tstart, tcnt, tfirst[257], scan[32]
    static constexpr size_t SMEM_BYTES = WORDS_OFF + (256 * 5 + 1 + 32 + 4) * 4;
};

// Top split.  A top bucket holding more than 256 groups' worth of keys must
// leave some group too big for a local sort: then MSD_OFF at once.
template <int KB, int THREADS, int IPT, int MIN_CTAS>
__global__ void __launch_bounds__(THREADS, MIN_CTAS) msd_top_kernel(MsdParams p) {
    using U = typename KeyBits<KB>::U;
    using G = MsdSplitGeom<KB, THREADS, IPT>;
    extern __shared__ __align__(128) uint8_t smem[];
    U* stage = reinterpret_cast<U*>(smem);
    uint32_t* bins = reinterpret_cast<uint32_t*>(smem + G::WORDS_OFF);
    uint32_t* delta = bins + 256;
    uint32_t* tstart = delta + 256;
    uint32_t* scan = tstart + 256 * 3 + 1;
    uint32_t* flag = scan + 32;
    grid_launch_dependents();
    grid_dependency_wait();
    const int tid = threadIdx.x;
    if (tid == 0) *flag = 0u;
    const uint32_t c = (tid < 256) ? uint32_t(p.gp_top[tid]) : 0u;
    const uint32_t ex = block_exclusive_scan_256<uint32_t>(c, scan, nullptr);
    if (tid < 256) {
        tstart[tid] = ex;
        if (c > 256u * p.group_cap) atomicOr(flag, 1u);
    }
    __syncthreads();
    if (*flag) {
        if (blockIdx.x == 0 && tid == 0) *p.state = MSD_OFF;
        return;
    }
    const U* in = static_cast<const U*>(p.keys_in);
    U* out = static_cast<U*>(p.keys_b);
    const uint64_t n = p.n;
    const uint32_t T = uint32_t((n + G::TILE - 1) / G::TILE);
    auto tile_cnt = [&](uint32_t t) {
        const uint64_t base = uint64_t(t) * G::TILE;
        return (t >= T) ? 0u : (n - base) < uint64_t(G::TILE) ? uint32_t(n - base) : uint32_t(G::TILE);
    };
    auto base = [&](int d) { return tstart[d]; };
    if constexpr (KB == 8) {
        // 8-byte keys: the CTA's next tile loads into a second register set
        // while it splits this one (2^27 keys: 0.95 -> 0.68 ms; ncu had the
        // split waiting on global loads, 10 long-scoreboard stalls per issue
        // against 3 in the second split).  16-byte keys measured slower so
        // (2^26: 0.36 -> 0.56 ms).
        U keys[IPT];
        uint32_t t = blockIdx.x;
        msd_load_tile<KB, THREADS, IPT, true>(in + uint64_t(t) * G::TILE, tile_cnt(t), p.kind, p.desc, keys);
        for (; t < T; t += gridDim.x) {
            U next[IPT];
            const uint32_t tn = t + gridDim.x;
            msd_load_tile<KB, THREADS, IPT, true>(in + uint64_t(tn < T ? tn : t) * G::TILE, tile_cnt(tn), p.kind,
                                                  p.desc, next);
            msd_split_loaded<KB, THREADS, IPT>(keys, tile_cnt(t), KB - 1, p.cursor1, base, out, n, p.err, stage,
                                               bins, delta, scan);
#pragma unroll
            for (int u = 0; u < IPT; ++u) keys[u] = next[u];
        }
    } else {
        for (uint32_t t = blockIdx.x; t < T; t += gridDim.x)
            msd_split_tile<KB, THREADS, IPT, true>(in + uint64_t(t) * G::TILE, tile_cnt(t), KB - 1, p.kind, p.desc,
                                                   p.cursor1, base, out, n, p.err, stage, bins, delta, scan);
    }
}

// Pair count: keys per (top, second) digit.  Its shared memory is the
// words of the split's layout only (no stage).
template <int KB, int THREADS, int IPT>
struct MsdCountGeom {
    static constexpr int TILE = THREADS * IPT;
    static constexpr size_t WORDS_OFF = 0;
    static constexpr size_t SMEM_BYTES = MsdSplitGeom<KB, THREADS, IPT>::SMEM_BYTES -
                                         MsdSplitGeom<KB, THREADS, IPT>::WORDS_OFF;
};
template <int KB, int THREADS, int IPT, int MIN_CTAS>
__global__ void __launch_bounds__(THREADS, MIN_CTAS) msd_count_kernel(MsdParams p) {
    using U = typename KeyBits<KB>::U;
    using G = MsdCountGeom<KB, THREADS, IPT>;
    extern __shared__ __align__(128) uint8_t smem[];
    uint32_t* bins = reinterpret_cast<uint32_t*>(smem + G::WORDS_OFF);
    uint32_t* tstart = bins + 512;
    uint32_t* tcnt = tstart + 256;
    uint32_t* tfirst = tcnt + 256;
    uint32_t* scan = tfirst + 257;
    grid_launch_dependents();
    grid_dependency_wait();
    if (ld_relaxed(p.state) == MSD_OFF) return;
    const int tid = threadIdx.x;
    msd_top_table(p.gp_top, G::TILE, tstart, tcnt, tfirst, scan);
    const U* keys = static_cast<const U*>(p.keys_b);
    const uint32_t T = tfirst[256];
    for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
        const uint32_t b = msd_bucket_of(tfirst, t);
        const uint32_t off = tstart[b] + (t - tfirst[b]) * G::TILE;
        const uint32_t end = tstart[b] + tcnt[b];
        const uint32_t cnt = (end - off) < uint32_t(G::TILE) ? end - off : uint32_t(G::TILE);
        U k[IPT];
#pragma unroll
        for (int u = 0; u < IPT; ++u) {
            const uint32_t j = uint32_t(u * THREADS + tid);
            k[u] = (j < cnt) ? keys[off + j] : U(0);
        }
        if (tid < 256) bins[tid] = 0u;
        __syncthreads();
#pragma unroll
        for (int u = 0; u < IPT; ++u)
            if (uint32_t(u * THREADS + tid) < cnt) atomicAdd(&bins[digit_of(k[u], KB - 2)], 1u);
        __syncthreads();
        if (tid < 256 && bins[tid]) atomicAdd(p.joint + b * 256 + tid, bins[tid]);
        __syncthreads();
    }
}

// Scan of the 65536 group sizes (one CTA of 1024 threads, 64 groups each)
// and the decision.
constexpr int MSD_SCAN_THREADS = 1024;
template <int KB>  // (one instance per key width's translation unit)
__global__ void __launch_bounds__(MSD_SCAN_THREADS, 1) msd_scan_kernel(MsdParams p) {
    __shared__ uint32_t scan[32];
    __shared__ uint32_t biggest;
    grid_launch_dependents();
    grid_dependency_wait();
    if (ld_relaxed(p.state) == MSD_OFF) return;
    const int tid = threadIdx.x;
    if (tid == 0) biggest = 0u;
    constexpr int PER = 65536 / MSD_SCAN_THREADS;
    const uint4* src = reinterpret_cast<const uint4*>(p.joint) + tid * (PER / 4);
    uint32_t c[PER];
#pragma unroll
    for (int i = 0; i < PER / 4; ++i) {
        const uint4 v = src[i];
        c[4 * i] = v.x;
        c[4 * i + 1] = v.y;
        c[4 * i + 2] = v.z;
        c[4 * i + 3] = v.w;
    }
    uint32_t sum = 0, big = 0;
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        sum += c[i];
        big = max(big, c[i]);
    }
    uint32_t run = block_exclusive_scan_all<MSD_SCAN_THREADS>(sum, scan);
    big = __reduce_max_sync(0xffffffffu, big);
    if ((tid & 31) == 0) atomicMax(&biggest, big);
    uint4* dst = reinterpret_cast<uint4*>(p.offs2) + tid * (PER / 4);
#pragma unroll
    for (int i = 0; i < PER / 4; ++i) {
        uint4 v;
        v.x = run;
        run += c[4 * i];
        v.y = run;
        run += c[4 * i + 1];
        v.z = run;
        run += c[4 * i + 2];
        v.w = run;
        run += c[4 * i + 3];
        dst[i] = v;
    }
    __syncthreads();
    if (tid == 0) *p.state = (biggest <= p.group_cap) ? MSD_OK : MSD_OFF;
}

// Second split: within every top bucket, into the groups' ranges.
template <int KB, int THREADS, int IPT, int MIN_CTAS>
__global__ void __launch_bounds__(THREADS, MIN_CTAS) msd_second_kernel(MsdParams p) {
    using U = typename KeyBits<KB>::U;
    using G = MsdSplitGeom<KB, THREADS, IPT>;
    extern __shared__ __align__(128) uint8_t smem[];
    U* stage = reinterpret_cast<U*>(smem);
    uint32_t* bins = reinterpret_cast<uint32_t*>(smem + G::WORDS_OFF);
    uint32_t* delta = bins + 256;
    uint32_t* tstart = delta + 256;
    uint32_t* tcnt = tstart + 256;
    uint32_t* tfirst = tcnt + 256;
    uint32_t* scan = tfirst + 257;
    grid_launch_dependents();
    grid_dependency_wait();
    if (ld_relaxed(p.state) != MSD_OK) return;
    msd_top_table(p.gp_top, G::TILE, tstart, tcnt, tfirst, scan);
    const U* in = static_cast<const U*>(p.keys_b);
    U* out = static_cast<U*>(p.keys_a);
    const uint32_t T = tfirst[256];
    for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
        const uint32_t b = msd_bucket_of(tfirst, t);
        const uint32_t off = tstart[b] + (t - tfirst[b]) * G::TILE;
        const uint32_t end = tstart[b] + tcnt[b];
        const uint32_t cnt = (end - off) < uint32_t(G::TILE) ? end - off : uint32_t(G::TILE);
        const uint32_t* group_base = p.offs2 + b * 256;
        msd_split_tile<KB, THREADS, IPT, false>(in + off, cnt, KB - 2, p.kind, p.desc, p.cursor2 + b * 256,
                                                [&](int d) { return group_base[d]; }, out, p.n, p.err, stage, bins,
                                                delta, scan);
    }
}

template <int KB, int THREADS, int LIPT>
struct MsdLocalGeom {
    static constexpr int WARPS = THREADS / 32;
    static constexpr int CTR_WORDS = 2 * WARPS * 256;  // the split's sub-buckets
    static constexpr size_t BUF_BYTES = (size_t(THREADS) * LIPT * KB + 127) & ~size_t(127);
    static constexpr size_t CTR_OFF = BUF_BYTES;
    static constexpr size_t SCAN_OFF = CTR_OFF + size_t(CTR_WORDS) * 4;  // u32 [32]
    static constexpr size_t MISC_OFF = SCAN_OFF + 128;                    // u32 [4]
    static constexpr size_t SMEM_BYTES = MISC_OFF + 16;
};

// 1: each CTA pulls its next group into L2 while it sorts the current one
// (2^26 u128 local sorts 0.795 -> 0.779 ms, 2^27 u64 1.048 -> 1.040).
#ifndef GBSORT_MSD_LOCAL_L2
#define GBSORT_MSD_LOCAL_L2 1
#endif

// Local sorts: each group (keys sharing their top two digits) sorted in
// place; the split counts over SPLIT_WORDS sub-buckets (about twice the mean
// group: fewer scan words per key, a comparison or two per key).
template <int KB, int THREADS, int LIPT, int MIN_CTAS, int SPLIT_WORDS>
__global__ void __launch_bounds__(THREADS, MIN_CTAS) msd_local_kernel(MsdParams p) {
    using U = typename KeyBits<KB>::U;
    using G = MsdLocalGeom<KB, THREADS, LIPT>;
    extern __shared__ __align__(128) uint8_t smem[];
    uint32_t* ctr = reinterpret_cast<uint32_t*>(smem + G::CTR_OFF);
    uint32_t* scan = reinterpret_cast<uint32_t*>(smem + G::SCAN_OFF);
    uint32_t* misc = reinterpret_cast<uint32_t*>(smem + G::MISC_OFF);
    grid_launch_dependents();
    grid_dependency_wait();
    if (ld_relaxed(p.state) != MSD_OK) return;
    const int tid = threadIdx.x;
    for (int i = tid; i < G::CTR_WORDS; i += THREADS) ctr[i] = 0u;
    __syncthreads();
    // Groups blockIdx.x, + gridDim.x, ...: the next group's size and place
    // load one group ahead.  (Its keys too, into a second register set or
    // into this one once the current keys sit in shared memory, measured
    // slower: 16-byte keys 2^26 2.32 vs 2.15 ms, the extra live registers
    // spill.)
    U* keys = static_cast<U*>(p.keys_a);
    U k[LIPT];
    auto load = [&](uint32_t cnt, uint32_t off) {
#pragma unroll
        for (int u = 0; u < LIPT; ++u) {
            const uint32_t j = uint32_t(u * THREADS + tid);
            k[u] = (j < cnt) ? keys[off + j] : U(0);
        }
    };
    uint32_t g = blockIdx.x;
    uint32_t c = (g < 65536u) ? p.joint[g] : 0u, o = (g < 65536u) ? p.offs2[g] : 0u;
    load(c, o);
    while (g < 65536u) {
        const uint32_t gn = g + gridDim.x;
        const uint32_t cn = (gn < 65536u) ? p.joint[gn] : 0u, on = (gn < 65536u) ? p.offs2[gn] : 0u;
#if GBSORT_MSD_LOCAL_L2
        {  // the next group into L2 while this one sorts
            const uintptr_t a = reinterpret_cast<uintptr_t>(keys + on) & ~uintptr_t(127);
            const uintptr_t e = reinterpret_cast<uintptr_t>(keys + on + cn);
            for (uintptr_t q = a + uintptr_t(tid) * 128; q < e; q += uintptr_t(THREADS) * 128)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(q));
        }
#endif
        if (c != 0u) {
            U* at = keys + o;
            static_assert(SPLIT_WORDS <= G::CTR_WORDS, "the split's counters");
            const bool split =
                cta_bucket_split<KB, THREADS, LIPT, SPLIT_WORDS, 8 * (KB - 2)>(k, at, c, smem, ctr, scan, misc, p.kind,
                                                                              p.desc);
            if (!split) {
                // a sub-bucket too big for the comparison rank (repeated
                // keys): the group goes back untwiddled, like every group
                // sorted here, so the buffer holds the input's keys in some
                // order, and the digit passes sort it (keys only: any order
                // of the input sorts to the same bytes)
#pragma unroll
                for (int u = 0; u < LIPT; ++u) {
                    const uint32_t j = uint32_t(u * THREADS + tid);
                    if (j < c) at[j] = twiddle_out<U>(k[u], p.kind, p.desc);
                }
                if (tid == 0) *p.state = MSD_OFF;
            }
        }
        load(cn, on);
        g = gn;
        c = cn;
        o = on;
    }
}

}  // namespace gbsort
