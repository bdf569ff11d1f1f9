// device_common.cuh — key bit types, twiddling, status-word codec, TMA /
// mbarrier / memory-order helpers and bounded waits for the sm_103a sort.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gbsort {

using u128 = unsigned __int128;

// Key kinds of the twiddle (reference: include/rsort/detail/tuning.cuh:352-384).
enum KeyKind : int { KIND_UNSIGNED = 0, KIND_SIGNED = 1, KIND_FLOAT = 2 };

// Error bits of the workspace error word.
enum : uint32_t { ERRBIT_TIMEOUT = 1u, ERRBIT_BOUNDS = 2u };

// Device-side bounds check on every scatter position (one compare per key): a
// failed check records ERRBIT_BOUNDS and skips the store instead of faulting.
#ifndef GBSORT_BOUNDS_CHECK
#define GBSORT_BOUNDS_CHECK 1
#endif
// Debug-only extra check of the shared-memory staging rank (always < tile by
// construction).
#ifndef GBSORT_DEBUG_CHECKS
#define GBSORT_DEBUG_CHECKS 0
#endif
// Rank atomics: 1 = only the leader lane of a digit group issues it (a
// divergent branch), 0 = every lane issues it and non-leaders add 0.
#ifndef GBSORT_RANK_LEADER_BRANCH
#define GBSORT_RANK_LEADER_BRANCH 1
#endif

// Lookback: issue the window's reads before the rank (1) or after it (0).
// Measured equal on GB300 (2^28 u32: 66.9 vs 67.2 Gkeys/s); 0 keeps the
// registers free during the rank.
// Tiles a pass CTA claims beyond the one it is ranking.  1 (default): the
// next tile is claimed when the current one starts, so tiles are ranked in
// about the order they were claimed.  3: the two ids after next are claimed
// early too, hiding the atomic's and the table load's latency, but a CTA
// then sits on claims its successors wait for; when CTAs start staggered
// (another kernel releasing the SMs one by one) the lookback degenerates into
// a serial chain, ~35x slower on GB300, and even alone it is not faster.
#ifndef GBSORT_TILE_LOOKAHEAD
#define GBSORT_TILE_LOOKAHEAD 1
#endif

// Key-value passes: double-buffer only the keys and copy each tile's values
// when the tile starts (1), or double-buffer keys and values (0).
#ifndef GBSORT_LATE_VALUES
#define GBSORT_LATE_VALUES 1
#endif

// Block-level short-circuit: a tile whose keys all share the pass's digit
// skips the warp match (its stable order is the input order).  Off: measured
// on GB300 it gains nothing (after the first pass LSD has permuted the keys,
// so a digit is uniform within tiles only where it is uniform across the
// whole array, and those passes are skipped outright) and costs ~1 % on
// random keys (2^28 u32: 66.4 vs 67.0 Gkeys/s; sorted input 3.76 vs 3.71 ms).
#ifndef GBSORT_TILE_SHORTCUT
#define GBSORT_TILE_SHORTCUT 0
#endif

// Rank with per-half-warp packed digit words (1) instead of per-warp
// counters plus per-warp match words (0).  One read returns peers and
// position, one leader store clears and advances, no counter atomic and no
// shuffle; but half-warp-striped loads conflict for even items per thread.
// Measured on GB300: +0.8 % at best on u32 keys-only (384 x 27), -8 % on
// f32+u32, so off.
#ifndef GBSORT_RANK_HALF
#define GBSORT_RANK_HALF 0
#endif

#ifndef GBSORT_LOOKBACK_PREFETCH
#define GBSORT_LOOKBACK_PREFETCH 0
#endif

template <bool B> struct BoolTag { static constexpr bool value = B; };
template <int I> struct IntTag { static constexpr int value = I; };

// Compile-time loop: f(IntTag<U>{}) for U in [U0, N).
template <int U0, int N>
struct StaticFor {
    template <class F>
    __device__ __forceinline__ static void run(F&& f) {
        if constexpr (U0 < N) {
            f(IntTag<U0>{});
            StaticFor<U0 + 1, N>::run(f);
        }
    }
};

// After a wait ran out, copies still in flight are drained for at most this
// long before a CTA leaves (a bulk copy from valid memory lands in microseconds).
constexpr uint64_t DRAIN_LIMIT_NS = 1000000000ull;

template <int KB> struct KeyBits;
template <> struct KeyBits<1> { using U = uint8_t; };
template <> struct KeyBits<2> { using U = uint16_t; };
template <> struct KeyBits<4> { using U = uint32_t; };
template <> struct KeyBits<8> { using U = uint64_t; };
template <> struct KeyBits<16> { using U = u128; };

// Value payloads are moved as raw bytes of these types.
struct alignas(16) Val16 { uint64_t lo, hi; };
template <int VB> struct ValBits { using V = uint8_t; };  // VB == 0: unused
template <> struct ValBits<1> { using V = uint8_t; };
template <> struct ValBits<2> { using V = uint16_t; };
template <> struct ValBits<4> { using V = uint32_t; };
template <> struct ValBits<8> { using V = uint64_t; };
template <> struct ValBits<16> { using V = Val16; };

// Programmatic dependent launch.  A kernel launched with the
// programmatic-stream-serialization attribute may be scheduled while its
// predecessor in the stream is still running: grid_dependency_wait() returns
// once that predecessor has completed and its memory writes are visible, so
// it comes before the kernel's first global access.  grid_launch_dependents()
// lets the successor be scheduled once every CTA of this grid has called it
// or exited.  Both do nothing for an ordinary launch.
__device__ __forceinline__ void grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Order-preserving map of a key's bits to an unsigned value (and back).
// kind/desc are launch-uniform, so the selects compile to predicated ops.
template <class U>
__device__ __forceinline__ U twiddle_in(U b, int kind, int desc) {
    const U sign = U(U(1) << (8 * sizeof(U) - 1));
    const U base = (kind == KIND_UNSIGNED) ? U(0) : sign;
    const bool neg_float = (kind == KIND_FLOAT) && ((b & sign) != U(0));
    U x = U(b ^ (neg_float ? U(~U(0)) : base));
    return desc ? U(~x) : x;
}

template <class U>
__device__ __forceinline__ U twiddle_out(U t, int kind, int desc) {
    const U sign = U(U(1) << (8 * sizeof(U) - 1));
    const U base = (kind == KIND_UNSIGNED) ? U(0) : sign;
    U y = desc ? U(~t) : t;
    const bool was_neg_float = (kind == KIND_FLOAT) && ((y & sign) == U(0));
    return U(y ^ (was_neg_float ? U(~U(0)) : base));
}

// 8-bit digit `pass` (0 = least significant byte) of a twiddled key.
__device__ __forceinline__ uint32_t digit_of(uint8_t x, int) { return x; }
__device__ __forceinline__ uint32_t digit_of(uint16_t x, int pass) {
    return __byte_perm(uint32_t(x), 0u, 0x4440u | uint32_t(pass));
}
__device__ __forceinline__ uint32_t digit_of(uint32_t x, int pass) {
    return __byte_perm(x, 0u, 0x4440u | uint32_t(pass));
}
__device__ __forceinline__ uint32_t digit_of(uint64_t x, int pass) {
    const uint32_t w = (pass & 4) ? uint32_t(x >> 32) : uint32_t(x);
    return __byte_perm(w, 0u, 0x4440u | uint32_t(pass & 3));
}
__device__ __forceinline__ uint32_t digit_of(u128 x, int pass) {
    const uint64_t h = (pass & 8) ? uint64_t(x >> 64) : uint64_t(x);
    const uint32_t w = (pass & 4) ? uint32_t(h >> 32) : uint32_t(h);
    return __byte_perm(w, 0u, 0x4440u | uint32_t(pass & 3));
}

// ---------------------------------------------------------------------------
// Status words of the decoupled lookback: [state:2 | epoch:E | value:VB_].
// state 0 = not published, 1 = PARTIAL (tile-local count), 2 = GLOBAL
// (inclusive prefix).  The epoch is the digit pass, so one clear per sort
// serves every pass.  E = log2(key bytes) bits (one per pass value).
// ---------------------------------------------------------------------------
template <class W, int KB>
struct StatusCodec {
    static constexpr int BITS = 8 * sizeof(W);
    static constexpr int EPOCH_BITS = KB == 1 ? 0 : KB == 2 ? 1 : KB == 4 ? 2 : KB == 8 ? 3 : 4;
    static constexpr int VALUE_BITS = BITS - 2 - EPOCH_BITS;
    static constexpr W VALUE_MASK = (W(1) << VALUE_BITS) - 1;
    static constexpr W PARTIAL = W(1) << (BITS - 2);
    static constexpr W GLOBAL = W(2) << (BITS - 2);

    __device__ __forceinline__ static W pack(W state, uint32_t epoch, uint64_t value) {
        return state | (W(epoch) << VALUE_BITS) | (W(value) & VALUE_MASK);
    }
    __device__ __forceinline__ static bool ready(W w, uint32_t epoch) {
        return (w >> (BITS - 2)) != 0 && uint32_t((w >> VALUE_BITS) & ((W(1) << EPOCH_BITS) - 1)) == epoch;
    }
    __device__ __forceinline__ static bool is_global(W w) { return (w & GLOBAL) != 0; }
    __device__ __forceinline__ static uint64_t value(W w) { return uint64_t(w & VALUE_MASK); }
};

// ---------------------------------------------------------------------------
// Memory-order helpers (relaxed, device scope: the value travels in the word).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
// Same loads without a compiler memory barrier, so a window of them issues
// back to back (used for the lookback window).
__device__ __forceinline__ uint32_t ld_relaxed_nb(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ uint64_t ld_relaxed_nb(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Mask of the lanes of this warp holding the same 8-bit digit.  Three ways to
// build it, identical results, each loading a different SM pipe:
//   RANK_BALLOT: 8 ballots, one per digit bit (integer ALU pipe)
//   RANK_MATCH:  the MATCH instruction (its own, low-throughput pipe)
//   RANK_OR:     lanes OR their bit into a per-warp shared word of the digit
//                and read it back (load/store pipe)
// GBSORT_RANK_PATTERN lists the method per column of items (4 bits each,
// column u uses nibble u % GBSORT_RANK_PATTERN_LEN), spreading the work.
//   RANK_OR5:    OR into one of 32 words by the digit's high 5 bits (one
//                word per bank: different words never conflict), then 3
//                ballots on the low 3 bits
enum RankMethod : int { RANK_BALLOT = 0, RANK_MATCH = 1, RANK_OR = 2, RANK_OR5 = 3 };
#ifndef GBSORT_RANK_PATTERN
#define GBSORT_RANK_PATTERN 0x2  // every column: shared-memory OR (fastest on GB300)
#define GBSORT_RANK_PATTERN_LEN 1
#endif
__host__ __device__ constexpr int rank_method(int column) {
    return int((uint64_t(GBSORT_RANK_PATTERN) >> (4 * (column % GBSORT_RANK_PATTERN_LEN))) & 0xF);
}
__host__ __device__ constexpr bool rank_uses_or(int ipt) {
    for (int u = 0; u < ipt; ++u)
        if (rank_method(u) == RANK_OR || rank_method(u) == RANK_OR5) return true;
    return false;
}

__device__ __forceinline__ uint32_t match_ballot(uint32_t d) {
    uint32_t peers = 0xffffffffu;
#pragma unroll
    for (int bit = 0; bit < 8; ++bit) {
        const uint32_t m = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
        peers &= ((d >> bit) & 1u) ? m : ~m;
    }
    return peers;
}

// `mb`: this warp's 256 zeroed shared words; left zeroed on return.
__device__ __forceinline__ uint32_t match_or(uint32_t d, uint32_t* mb, int lane, uint32_t lt) {
    atomicOr(&mb[d], 1u << lane);
    __syncwarp();
    const uint32_t peers = mb[d];
    __syncwarp();
    if ((peers & lt) == 0) mb[d] = 0u;  // the group's lowest lane clears
    __syncwarp();
    return peers;
}

// `mb`: this warp's zeroed shared words (32 used, 32-word aligned); left
// zeroed on return.
__device__ __forceinline__ uint32_t match_or5(uint32_t d, uint32_t* mb, int lane, uint32_t lt) {
    const uint32_t hi = d >> 3;
    atomicOr(&mb[hi], 1u << lane);
    uint32_t lo = 0xffffffffu;
#pragma unroll
    for (int bit = 0; bit < 3; ++bit) {
        const uint32_t m = __ballot_sync(0xffffffffu, (d >> bit) & 1u);
        lo &= ((d >> bit) & 1u) ? m : ~m;
    }
    __syncwarp();
    const uint32_t hi_peers = mb[hi];
    __syncwarp();
    if ((hi_peers & lt) == 0) mb[hi] = 0u;  // the high group's lowest lane clears
    __syncwarp();
    return hi_peers & lo;
}

template <int METHOD>
__device__ __forceinline__ uint32_t warp_match_digit(uint32_t d, uint32_t* mb, int lane, uint32_t lt) {
    if constexpr (METHOD == RANK_MATCH) return __match_any_sync(0xffffffffu, d);
    else if constexpr (METHOD == RANK_OR) return match_or(d, mb, lane, lt);
    else if constexpr (METHOD == RANK_OR5) return match_or5(d, mb, lane, lt);
    else return match_ballot(d);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---------------------------------------------------------------------------
// mbarrier + bulk-copy (TMA, non-tensor) helpers.  Plain global->shared bulk
// copies; no multicast.  Addresses and sizes are 16-byte aligned by callers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                              uint64_t policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_test_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase.  Returns false (after flagging the
// workspace error word) if the limit ran out.  The first probe does not
// block; after it the limit is checked before every (potentially blocking)
// try_wait, so a limit shorter than the copy always runs out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns,
                                                  uint32_t* err) {
    if (mbar_test_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    for (;;) {
        if (global_timer_ns() - t0 > limit_ns) {
            atomicOr(err, ERRBIT_TIMEOUT);
            return false;
        }
        if (mbar_try_wait(bar, parity)) return true;
    }
}

// Grid-wide barrier of a cooperative launch (every CTA resident at once).
// counter and gen start at 0.  The k-th barrier of the launch (k = 1, 2,
// ...): thread 0 of each CTA fences and adds 1 to counter, then polls
// counter with acquire loads until it reaches k * gridDim.x (by default), or
// — with GBSORT_BARRIER_POLL_COUNTER 0 — the CTA that brings counter there
// publishes gen = k (another 128-byte line, away from the arrivals'
// atomics) and the others poll gen.  Either wait is bounded by limit_ns: a
// wait that runs out records ERRBIT_TIMEOUT and the barrier returns false
// on every thread of that CTA, so the caller can leave instead of hanging.
// Polling the counter saves the generation word's extra round trip: 2^20
// u32 keys in one launch 24.3 vs 25.2 us, 2^19 u128 22.4 vs 24.1.
// Nonzero: the ns each poll of the counter sleeps before the next.
#ifndef GBSORT_BARRIER_POLL_COUNTER
#define GBSORT_BARRIER_POLL_COUNTER 32
#endif
__device__ __forceinline__ bool grid_barrier(uint32_t* counter, uint32_t* gen, uint32_t k, uint64_t limit_ns,
                                             uint32_t* err) {
    __syncthreads();
    int ok = 1;
    if (GBSORT_BARRIER_POLL_COUNTER && threadIdx.x == 0) {
        // every CTA polls the counter itself: no generation word to publish
        __threadfence();
        asm volatile("red.relaxed.gpu.global.add.u32 [%0], 1;" ::"l"(counter) : "memory");
        const uint32_t target = k * gridDim.x;
        const uint64_t t0 = global_timer_ns();
        while (ld_acquire(counter) < target) {
            if (global_timer_ns() - t0 > limit_ns) {
                atomicOr(err, ERRBIT_TIMEOUT);
                ok = 0;
                break;
            }
            __nanosleep(GBSORT_BARRIER_POLL_COUNTER);
        }
        __threadfence();
    } else if (threadIdx.x == 0) {
        __threadfence();
        const uint32_t arrived = atomicAdd(counter, 1u) + 1u;
        if (arrived == k * gridDim.x) {
            __threadfence();
            asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(gen), "r"(k) : "memory");
        } else if (ld_acquire(gen) < k) {
            const uint64_t t0 = global_timer_ns();
            while (ld_acquire(gen) < k) {
                if (global_timer_ns() - t0 > limit_ns) {
                    atomicOr(err, ERRBIT_TIMEOUT);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    return __syncthreads_and(ok) != 0;
}

// Bounded wait for a status word of the current epoch.  On timeout, or when
// another CTA already flagged an error, returns a GLOBAL word with value 0 so
// the lookback walk ends and the launch drains instead of hanging.
template <class Codec, class W>
__device__ __forceinline__ W wait_status(const W* addr, uint32_t epoch, uint64_t limit_ns, uint32_t* err) {
    W w = ld_relaxed(addr);
    if (Codec::ready(w, epoch)) return w;
    const uint64_t t0 = global_timer_ns();
    uint32_t sleep_ns = 32;
    for (;;) {
        __nanosleep(sleep_ns);
        if (sleep_ns < 512) sleep_ns <<= 1;
        w = ld_relaxed(addr);
        if (Codec::ready(w, epoch)) return w;
        if (ld_relaxed(err) != 0u) return Codec::GLOBAL;
        if (global_timer_ns() - t0 > limit_ns) {
            atomicOr(err, ERRBIT_TIMEOUT);
            return Codec::GLOBAL;
        }
    }
}

// Decoupled lookback for one digit bin of tile `cur` over a [tile][256] status
// array: reads WIN predecessors' words at once (one L2 round trip per window
// instead of per tile), then sums them nearest-first up to the first
// inclusive (GLOBAL) word, re-polling (bounded) any word not yet published.
// Tile 0 always publishes GLOBAL, so the walk ends there at the latest.
template <class Codec, int WIN, class W>
__device__ __forceinline__ unsigned long long lookback_window(const W* status, uint32_t cur, int bin,
                                                             uint32_t epoch, uint64_t limit_ns, uint32_t* err) {
    unsigned long long prefix = 0;
    int64_t j = int64_t(cur) - 1;
    while (j >= 0) {
        W w[WIN];
#pragma unroll
        for (int i = 0; i < WIN; ++i)
            w[i] = (j - i >= 0) ? ld_relaxed_nb(status + size_t(j - i) * 256 + bin) : W(0);
#pragma unroll
        for (int i = 0; i < WIN; ++i) {
            if (j - i < 0) return prefix;
            W x = w[i];
            if (!Codec::ready(x, epoch)) x = wait_status<Codec>(status + size_t(j - i) * 256 + bin, epoch, limit_ns, err);
            prefix += Codec::value(x);
            if (Codec::is_global(x)) return prefix;
        }
        j -= WIN;
    }
    return prefix;
}

// The lookback split in two so its first L2 round trip overlaps other work:
// lookback_prefetch issues the reads of the WIN nearest predecessors' words;
// lookback_finish consumes them (re-polling any not yet published, a stale
// PARTIAL is still a correct count) and walks on below the window if no
// inclusive word was among them.
template <int WIN, class W>
__device__ __forceinline__ void lookback_prefetch(const W* status, uint32_t cur, int bin, W (&pre)[WIN]) {
#pragma unroll
    for (int i = 0; i < WIN; ++i) {
        const int64_t j = int64_t(cur) - 1 - i;
        pre[i] = (j >= 0) ? ld_relaxed_nb(status + size_t(j) * 256 + bin) : W(0);
    }
}

template <class Codec, int WIN, class W>
__device__ __forceinline__ unsigned long long lookback_finish(const W* status, uint32_t cur, int bin,
                                                             const W (&pre)[WIN], uint32_t epoch,
                                                             uint64_t limit_ns, uint32_t* err) {
    unsigned long long prefix = 0;
#pragma unroll
    for (int i = 0; i < WIN; ++i) {
        const int64_t j = int64_t(cur) - 1 - i;
        if (j < 0) return prefix;
        W x = pre[i];
        if (!Codec::ready(x, epoch)) x = wait_status<Codec>(status + size_t(j) * 256 + bin, epoch, limit_ns, err);
        prefix += Codec::value(x);
        if (Codec::is_global(x)) return prefix;
    }
    if (int64_t(cur) - WIN > 0)
        prefix += lookback_window<Codec, WIN>(status, cur - WIN, bin, epoch, limit_ns, err);
    return prefix;
}

// Exclusive scan of one value per thread over threads [0, 256) of the block.
// All threads of the block must call it (it contains __syncthreads).
template <class T>
__device__ __forceinline__ T block_exclusive_scan_256(T x, T* warp_tmp /* >= 8 */, T* total_out) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    T v = (tid < 256) ? x : T(0);
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31 && warp < 8) warp_tmp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        T t = (lane < 8) ? warp_tmp[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < 8) warp_tmp[lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    T excl = T(0);
    if (tid < 256) excl = (warp > 0 ? warp_tmp[warp - 1] : T(0)) + v - x;
    if (total_out) *total_out = warp_tmp[7];
    return excl;
}

}  // namespace gbsort
