// inst_k16.cu — kernels for 16-byte keys (see inst_impl.cuh).
#include "inst_impl.cuh"

namespace gbsort {
const KernelEntry* pass_entries_k16() { return pass_entries_for<16>(); }
const KernelEntry* upsweep_entry_k16() { return upsweep_entry_for<16>(); }
const KernelEntry* fused_entry_k16() { return fused_entry_for<16>(); }
const KernelEntry* msd_entries_k16() { return msd_entries_for<16>(); }
const KernelEntry* seg_entries_k16() { return seg_entries_for<16>(); }
const KernelEntry* seg_upsweep_entry_k16() { return seg_upsweep_entry_for<16>(); }
}  // namespace gbsort
