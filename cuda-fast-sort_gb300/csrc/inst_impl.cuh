// inst_impl.cuh — explicit kernel instantiations for one key width.  Each
// inst_k*.cu includes this with one width, so the five widths compile as
// parallel translation units.
#pragma once

#include "fused_short.cuh"
#include "msd.cuh"
#include "onesweep.cuh"
#include "segmented.cuh"
#include "shapes.h"

namespace gbsort {

template <int KB, int VB, class W, bool SEG, class S = PassShape<KB, VB>>
KernelEntry make_pass_entry() {
    using G = PassGeom<KB, VB, S::THREADS, S::IPT>;
    return KernelEntry{
        reinterpret_cast<const void*>(
            &onesweep_pass_kernel<KB, VB, W, S::THREADS, S::IPT, SEG, S::MIN_CTAS, S::LOOKBACK_WINDOW>),
        S::THREADS, S::IPT, G::TILE, static_cast<unsigned long>(G::SMEM_BYTES)};
}

// [value size][0: 32-bit status, 1: 64-bit status, 2: small-n shape (32-bit)]
template <int KB, int VB>
struct PassRow {
    KernelEntry e[3];
    PassRow()
        : e{make_pass_entry<KB, VB, uint32_t, false>(), make_pass_entry<KB, VB, uint64_t, false>(),
            make_pass_entry<KB, VB, uint32_t, false, PassShapeSmall<KB, VB>>()} {}
};

template <int KB>
const KernelEntry* pass_entries_for() {
    static const PassRow<KB, 0> r0;
    static const PassRow<KB, 1> r1;
    static const PassRow<KB, 2> r2;
    static const PassRow<KB, 4> r4;
    static const PassRow<KB, 8> r8;
    static const PassRow<KB, 16> r16;
    static const KernelEntry e[6][3] = {
        {r0.e[0], r0.e[1], r0.e[2]},    {r1.e[0], r1.e[1], r1.e[2]},    {r2.e[0], r2.e[1], r2.e[2]},
        {r4.e[0], r4.e[1], r4.e[2]},    {r8.e[0], r8.e[1], r8.e[2]},    {r16.e[0], r16.e[1], r16.e[2]},
    };
    return &e[0][0];
}

// The one-launch sort of short keys-only arrays, in the short-array pass shape.
template <int KB>
const KernelEntry* fused_entry_for() {
    using S = FusedShape<KB>;
    using G = ShortGeom<KB, S::THREADS, S::IPT, S::LIPT>;
    static_assert(G::TILE == PassShapeSmall<KB, 0>::THREADS * PassShapeSmall<KB, 0>::IPT, "same tiles as the short shape");
    static const KernelEntry e = {
        reinterpret_cast<const void*>(&fused_short_kernel<KB, S::THREADS, S::IPT, S::LIPT, S::MIN_CTAS>), S::THREADS,
        S::IPT, G::TILE, static_cast<unsigned long>(G::SMEM_BYTES)};
    return &e;
}

// Keys-only sorts of 8- and 16-byte keys, most significant digit first:
// top split, pair count, scan, second split, local sorts (shape 0), local
// sorts (shape 1), the top digit's histogram.
template <int KB, int L>
KernelEntry make_msd_local_entry() {
    using S = MsdShape<KB>;
    using GL = MsdLocalGeom<KB, S::C_THREADS, S::C_LIPT[L]>;
    return KernelEntry{reinterpret_cast<const void*>(&msd_local_kernel<KB, S::C_THREADS, S::C_LIPT[L],
                                                                        S::C_MIN_CTAS[L], S::C_SPLIT_WORDS[L]>),
                       S::C_THREADS, S::C_LIPT[L], S::C_THREADS * S::C_LIPT[L],
                       static_cast<unsigned long>(GL::SMEM_BYTES)};
}

template <int KB>
const KernelEntry* msd_entries_for() {
    using S = MsdShape<KB>;
    using GS = MsdSplitGeom<KB, S::THREADS, S::IPT>;
    static const KernelEntry e[7] = {
        {reinterpret_cast<const void*>(&msd_top_kernel<KB, S::THREADS, S::IPT, S::MIN_CTAS>), S::THREADS, S::IPT,
         GS::TILE, static_cast<unsigned long>(GS::SMEM_BYTES)},
        {reinterpret_cast<const void*>(&msd_count_kernel<KB, S::THREADS, S::IPT, S::MIN_CTAS>), S::THREADS, S::IPT,
         GS::TILE, static_cast<unsigned long>(MsdCountGeom<KB, S::THREADS, S::IPT>::SMEM_BYTES)},
        {reinterpret_cast<const void*>(&msd_scan_kernel<KB>), MSD_SCAN_THREADS, 0, 0, 0ul},
        {reinterpret_cast<const void*>(&msd_second_kernel<KB, S::THREADS, S::IPT, S::MIN_CTAS>), S::THREADS, S::IPT,
         GS::TILE, static_cast<unsigned long>(GS::SMEM_BYTES)},
        make_msd_local_entry<KB, 0>(),
        make_msd_local_entry<KB, 1>(),
        {reinterpret_cast<const void*>(&msd_hist_kernel<KB>), MSD_HIST_THREADS, 0, 0, 0ul},
    };
    return e;
}

template <int KB>
const KernelEntry* upsweep_entry_for() {
    static const KernelEntry e = {reinterpret_cast<const void*>(&upsweep_kernel<KB>), HIST_THREADS, 0, 0,
                                  static_cast<unsigned long>(HistGeom<KB>::SMEM_BYTES)};
    return &e;
}

// ---- batched mode ---------------------------------------------------------
// Small-segment CTA sorts: "S" = 256 threads x 8 items (8- or 4-bit digits),
// "L" = 512 threads x as many items as keep the two shared buffers within
// 128 KB (8-bit digits).
template <int KB, int VB>
struct CtaShapes {
    static constexpr int S_THREADS = 256, S_IPT = 8;
    static constexpr int L_THREADS = 512;
    static constexpr int L_ITEMS_RAW = 65536 / (KB + VB);
    static constexpr int L_IPT = L_ITEMS_RAW / L_THREADS > 32 ? 32 : (L_ITEMS_RAW / L_THREADS < 4 ? 4 : L_ITEMS_RAW / L_THREADS);
};

template <int KB, int VB, int THREADS, int IPT, int RBITS>
KernelEntry make_cta_entry() {
    using GC = CtaSortGeom<KB, VB, THREADS, IPT, RBITS>;
    return KernelEntry{reinterpret_cast<const void*>(&cta_sort_kernel<KB, VB, THREADS, IPT, RBITS>), THREADS, IPT,
                       GC::TILE, static_cast<unsigned long>(GC::SMEM_BYTES)};
}

template <int KB, int VB>
void make_seg_entries(KernelEntry* out /* [4]: pass, cta S, cta L, cta S 4-bit */) {
    using C = CtaShapes<KB, VB>;
    out[0] = make_pass_entry<KB, VB, uint32_t, true>();
    out[1] = make_cta_entry<KB, VB, C::S_THREADS, C::S_IPT, 8>();
    out[2] = make_cta_entry<KB, VB, C::L_THREADS, C::L_IPT, 8>();
    out[3] = make_cta_entry<KB, VB, C::S_THREADS, C::S_IPT, 4>();
}

template <int KB>
const KernelEntry* seg_entries_for() {
    static KernelEntry e[6][4];
    static const bool init = [] {
        make_seg_entries<KB, 0>(e[0]);
        make_seg_entries<KB, 1>(e[1]);
        make_seg_entries<KB, 2>(e[2]);
        make_seg_entries<KB, 4>(e[3]);
        make_seg_entries<KB, 8>(e[4]);
        make_seg_entries<KB, 16>(e[5]);
        return true;
    }();
    (void)init;
    return &e[0][0];
}

template <int KB>
const KernelEntry* seg_upsweep_entry_for() {
    static const KernelEntry e = {reinterpret_cast<const void*>(&seg_upsweep_kernel<KB>), SEG_UP_THREADS, 0, 0,
                                  static_cast<unsigned long>(SegHistGeom<KB>::SMEM_BYTES)};
    return &e;
}

}  // namespace gbsort
