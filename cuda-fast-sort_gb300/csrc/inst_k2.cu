// inst_k2.cu — kernels for 2-byte keys (see inst_impl.cuh).
#include "inst_impl.cuh"

namespace gbsort {
const KernelEntry* pass_entries_k2() { return pass_entries_for<2>(); }
const KernelEntry* upsweep_entry_k2() { return upsweep_entry_for<2>(); }
const KernelEntry* fused_entry_k2() { return fused_entry_for<2>(); }
const KernelEntry* seg_entries_k2() { return seg_entries_for<2>(); }
const KernelEntry* seg_upsweep_entry_k2() { return seg_upsweep_entry_for<2>(); }
}  // namespace gbsort
