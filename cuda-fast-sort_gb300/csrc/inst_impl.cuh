// inst_impl.cuh — explicit kernel instantiations for one key width.  Each
// inst_k*.cu includes this with GBSORT_KB set, so the five widths compile as
// five parallel translation units.
#pragma once

#include "onesweep.cuh"
#include "shapes.h"

namespace gbsort {

template <int KB, int VB, class W>
KernelEntry make_pass_entry() {
    using S = PassShape<KB, VB>;
    using G = PassGeom<KB, VB, S::THREADS, S::IPT>;
    return KernelEntry{reinterpret_cast<const void*>(&onesweep_pass_kernel<KB, VB, W, S::THREADS, S::IPT>),
                       S::THREADS, S::IPT, G::TILE, static_cast<unsigned long>(G::SMEM_BYTES)};
}

template <int KB>
const KernelEntry* pass_entries_for() {
    static const KernelEntry e[6][2] = {
        {make_pass_entry<KB, 0, uint32_t>(), make_pass_entry<KB, 0, uint64_t>()},
        {make_pass_entry<KB, 1, uint32_t>(), make_pass_entry<KB, 1, uint64_t>()},
        {make_pass_entry<KB, 2, uint32_t>(), make_pass_entry<KB, 2, uint64_t>()},
        {make_pass_entry<KB, 4, uint32_t>(), make_pass_entry<KB, 4, uint64_t>()},
        {make_pass_entry<KB, 8, uint32_t>(), make_pass_entry<KB, 8, uint64_t>()},
        {make_pass_entry<KB, 16, uint32_t>(), make_pass_entry<KB, 16, uint64_t>()},
    };
    return &e[0][0];
}

template <int KB>
const KernelEntry* upsweep_entry_for() {
    static const KernelEntry e = {reinterpret_cast<const void*>(&upsweep_kernel<KB>), HIST_THREADS, 0, 0,
                                  static_cast<unsigned long>(HistGeom<KB>::SMEM_BYTES)};
    return &e;
}

}  // namespace gbsort
