// inst_k1.cu — kernels for 1-byte keys (see inst_impl.cuh).
#include "inst_impl.cuh"

namespace gbsort {
const KernelEntry* pass_entries_k1() { return pass_entries_for<1>(); }
const KernelEntry* upsweep_entry_k1() { return upsweep_entry_for<1>(); }
const KernelEntry* fused_entry_k1() { return fused_entry_for<1>(); }
const KernelEntry* seg_entries_k1() { return seg_entries_for<1>(); }
const KernelEntry* seg_upsweep_entry_k1() { return seg_upsweep_entry_for<1>(); }
}  // namespace gbsort
