// segmented_internal.h — parts of a batched-sort plan that the server and
// the host-memory batched sort use beyond the public C ABI (defined in
// segmented_api.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include "gbsort.h"

namespace gbsort {

// Device address of the plan's error word (valid once bound).
const void* segmented_error_word(const gbsort_segmented_plan* p);
// Bytes and host image of the plan's tables (segment begins, tile list,
// upsweep items, CTA segment lists), as they sit in the workspace.
size_t segmented_table_bytes(const gbsort_segmented_plan* p);
void segmented_table_image(const gbsort_segmented_plan* p, uint8_t* dst);
// gbsort_segmented_bind with the tables taken from `image`: host memory
// (pinned; nullptr: the plan's own pageable image) uploaded on `stream`, or,
// with image_on_device, a device copy moved into the workspace by a kernel.
int segmented_bind_image(gbsort_segmented_plan* p, void* d_keys, void* d_values, void* d_workspace,
                         size_t workspace_bytes, void* stream, const uint8_t* image, bool image_on_device = false);

}  // namespace gbsort
