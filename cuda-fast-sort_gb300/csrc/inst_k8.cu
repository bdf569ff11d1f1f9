// inst_k8.cu — kernels for 8-byte keys (see inst_impl.cuh).
#include "inst_impl.cuh"

namespace gbsort {
const KernelEntry* pass_entries_k8() { return pass_entries_for<8>(); }
const KernelEntry* upsweep_entry_k8() { return upsweep_entry_for<8>(); }
const KernelEntry* fused_entry_k8() { return fused_entry_for<8>(); }
const KernelEntry* msd_entries_k8() { return msd_entries_for<8>(); }
const KernelEntry* seg_entries_k8() { return seg_entries_for<8>(); }
const KernelEntry* seg_upsweep_entry_k8() { return seg_upsweep_entry_for<8>(); }
}  // namespace gbsort
