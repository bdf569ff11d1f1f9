// inst_k4.cu — kernels for 4-byte keys (see inst_impl.cuh).
#include "inst_impl.cuh"

namespace gbsort {
const KernelEntry* pass_entries_k4() { return pass_entries_for<4>(); }
const KernelEntry* upsweep_entry_k4() { return upsweep_entry_for<4>(); }
const KernelEntry* fused_entry_k4() { return fused_entry_for<4>(); }
const KernelEntry* seg_entries_k4() { return seg_entries_for<4>(); }
const KernelEntry* seg_upsweep_entry_k4() { return seg_upsweep_entry_for<4>(); }
}  // namespace gbsort
