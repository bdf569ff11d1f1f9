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

template <int KB, int THREADS, int IPT>
struct ShortGeom {
    static constexpr int P = KB;
    static constexpr int WARPS = THREADS / 32;
    static constexpr int TILE = THREADS * IPT;
    static constexpr int IPW = 32 * IPT;
    static constexpr size_t STAGE_OFF = 0;  // U [TILE]
    static constexpr size_t WHIST_OFF = (size_t(TILE) * KB + 127) & ~size_t(127);  // u32 [WARPS][256]
    static constexpr size_t MATCH_OFF = WHIST_OFF + size_t(WARPS) * 1024;          // u32 [WARPS][256]
    static constexpr size_t COUNT_BYTES = MATCH_OFF + size_t(WARPS) * 1024;        // phase 0 counters here
    static constexpr size_t GEXCL_OFF = COUNT_BYTES;                               // u32 [P][256]
    static constexpr size_t BINB_OFF = GEXCL_OFF + size_t(P) * 1024;               // u32 [256]
    static constexpr size_t SCAN_OFF = BINB_OFF + 1024;                            // u32 [32]
    static constexpr size_t MISC_OFF = SCAN_OFF + 128;                             // u32 [4]: uniform mask
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

template <int KB, int THREADS, int IPT, int MIN_CTAS>
__global__ void __launch_bounds__(THREADS, MIN_CTAS) fused_short_kernel(FusedParams f) {
    using U = typename KeyBits<KB>::U;
    using G = ShortGeom<KB, THREADS, IPT>;
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

    if (tid == 0) misc[0] = 0u;
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

    const uint32_t lt = lanemask_lt();
    uint32_t* wh = whist + warp * 256;
    uint32_t* mb = mscratch + warp * 256;
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
        const uint32_t epoch = uint32_t(q);
        ++before;

        for (uint32_t t = blockIdx.x; t < T; t += gridDim.x) {
            const uint64_t base = uint64_t(t) * G::TILE;
            const uint32_t cnt = (n - base) < uint64_t(G::TILE) ? uint32_t(n - base) : uint32_t(G::TILE);
            const bool full = cnt == uint32_t(G::TILE);

            // ---- keys straight into registers (warp-striped: a warp's lanes
            // read 32 consecutive keys per column; rank order = input order)
            U keys[IPT];
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                const uint32_t j = uint32_t(warp * G::IPW + u * 32 + lane);
                keys[u] = (full || j < cnt) ? kin[base + j] : U(~U(0));  // filler sorts last
                if (tw_load && (full || j < cnt)) keys[u] = twiddle_in<U>(keys[u], kind, desc);
            }

            // ---- warp histograms
#pragma unroll
            for (int i = lane; i < 256; i += 32) wh[i] = 0u;
            __syncwarp();
#pragma unroll
            for (int u = 0; u < IPT; ++u) atomicAdd(&wh[digit_of(keys[u], q)], 1u);
            __syncthreads();

            // ---- per-bin totals, warp bases, early publication, tile starts
            uint32_t tot = 0, valid = 0;
            if (tid < 256) {
#pragma unroll
                for (int w = 0; w < G::WARPS; ++w) {
                    const uint32_t c = whist[w * 256 + tid];
                    whist[w * 256 + tid] = tot;
                    tot += c;
                }
                valid = tot - ((tid == 255) ? (uint32_t(G::TILE) - cnt) : 0u);
                st_relaxed(partial + size_t(t) * 256 + tid, Codec::pack(Codec::PARTIAL, epoch, valid));
            }
            // The group's last tile publishes the group sum now, before its
            // rank: the group's tiles published their counts at about the
            // same time, and every later tile needs the sum after its rank.
            const uint32_t g = t / SHORT_GROUP, g0 = g * SHORT_GROUP;
            uint32_t in_group = 0;
            const bool leader = t % SHORT_GROUP == SHORT_GROUP - 1 || t + 1 == T;
            if (leader && tid < 256) {
                in_group = sum_published<Codec>(partial + size_t(g0) * 256 + tid, t - g0, epoch, limit, err);
                st_relaxed(agg + size_t(g) * 256 + tid, Codec::pack(Codec::PARTIAL, epoch, in_group + valid));
            }
            const uint32_t excl = block_exclusive_scan_256<uint32_t>(tot, scan, nullptr);
            if (tid < 256) {
#pragma unroll
                for (int w = 0; w < G::WARPS; ++w) whist[w * 256 + tid] += excl;
            }
            __syncthreads();

            // ---- rank (warp match + popc + one counter atomic per digit
            // group) and staging at rank
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

            // ---- two-level prefix: earlier groups' sums + this group's
            // earlier tiles
            if (tid < 256) {
                if (!leader) in_group = sum_published<Codec>(partial + size_t(g0) * 256 + tid, t - g0, epoch, limit, err);
                const uint32_t earlier = sum_published<Codec>(agg + tid, g, epoch, limit, err);
                binb[tid] = gex[q * 256 + tid] + earlier + in_group - excl;
            }
            __syncthreads();

            // ---- coalesced write-out: thread-linear over the digit-sorted tile
            U ks[IPT];
            uint32_t pos[IPT];
#pragma unroll
            for (int u = 0; u < IPT; ++u) ks[u] = stage[u * THREADS + tid];
#pragma unroll
            for (int u = 0; u < IPT; ++u) pos[u] = binb[digit_of(ks[u], q)] + uint32_t(u * THREADS + tid);
            bool bad = false;
#pragma unroll
            for (int u = 0; u < IPT; ++u) {
                if (full || uint32_t(u * THREADS + tid) < cnt) {
                    if (pos[u] < n) kout[pos[u]] = tw_store ? twiddle_out<U>(ks[u], kind, desc) : ks[u];
                    else bad = true;
                }
            }
            if (bad) atomicOr(err, ERRBIT_BOUNDS);
        }
        if (before == total && !f.fixup) break;  // the last pass: nothing reads its output in this launch
        if (!grid_barrier(f.barrier, f.barrier_gen, ++phase, limit, err)) return;
        if (ld_relaxed(err) != 0u) return;  // a failed wait or bounds check: every CTA leaves
    }
    if (f.fixup) fixup_body(f.fix);
}

}  // namespace gbsort
