// noalloc.cu — gbsort_sort_keys_noalloc: the keys-only sort with its
// workspace in a fixed, file-scope device array instead of caller memory.
//
// Who needs it: callers that may not allocate device memory at the point
// where they sort.  cudaMalloc/cudaFree can block, cudaFree synchronizes the
// whole device, an allocation can fail late under fragmentation, and some
// hosts (a framework whose allocator owns every device byte, a plugin with a
// pre-reserved budget, an FFI binding with no allocator of its own) forbid a
// library from allocating at all.  Such callers still own the keys buffer;
// only the scratch moves into this library.
//
// Contract:
//   - capacity: NOALLOC_SCRATCH_BYTES (16 MiB) of workspace.  A sort fits when
//     the size query (gbsort_sort_keys with a NULL workspace) reports at most
//     16 MiB for its key type and n: about 4.0 M keys of 4 bytes, 2.0 M of 8
//     bytes, 1.0 M of 16 bytes, 15 M of 1 byte, 7.9 M of 2 bytes.  A larger n
//     is rejected with GBSORT_ERR_WORKSPACE_TOO_SMALL before any device work.
//   - the array is a module global: every GPU that loads this library holds
//     the 16 MiB until the process exits.
//   - the first call on a device looks up the array's device address on that
//     device (cudaGetSymbolAddress, with that device current); make that first
//     call before any stream capture on the device.
//   - every call shares the one array and it keeps the last call's contents;
//     the sort clears what must start at zero (control block, lookback status
//     words) itself.  Calls that overlap on the GPU (different streams, or
//     different host threads without ordering) race on the array: order them.
//   - no cudaMalloc, cudaFree or other allocating call is made.
//   - a device-side failure (a bounded wait that ran out, a failed bounds
//     check) is recorded in the scratch's control block; read it with
//     gbsort_noalloc_status(key_type, n, stream) after the sort and before
//     the next noalloc call, which clears it.

#include <cstdio>
#include <mutex>
#include <string>

#include "gbsort.h"
#include "plan.h"

namespace gbsort {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(16) << 20;

// The scratch itself.  Host code must not use this name as an address (it is
// a host-side stand-in); it uses the pointer cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;

// Per-device address of the scratch.  Only a successful lookup is kept: a
// failed one (e.g. made inside a stream capture) is retried by the next call.
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch on the current device (looked up once per
// device, with that device current).
void* noalloc_scratch_for_current_device() {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_last_error("gbsort_sort_keys_noalloc: cudaGetDevice", e);
        return nullptr;
    }
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        char msg[120];
        std::snprintf(msg, sizeof msg, "gbsort_sort_keys_noalloc: device %d is beyond the %d devices supported", dev,
                      NOALLOC_MAX_DEVICES);
        set_last_error_text(msg);
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();  // do not leave the error for the caller's next CUDA call
            set_last_error("gbsort_sort_keys_noalloc: cudaGetSymbolAddress", e);
            return nullptr;
        }
        g_noalloc_ptr[dev] = p;
    }
    return g_noalloc_ptr[dev];
}

// The plan of a keys-only sort that fits the scratch, or a status.
int noalloc_plan(int key_type, size_t n, Plan* plan) {
    const int st = make_plan(key_type, 0, n, plan);
    if (st != GBSORT_OK) return st;
    if (plan->total_bytes > NOALLOC_SCRATCH_BYTES) {
        char msg[200];
        std::snprintf(msg, sizeof msg,
                      "gbsort_sort_keys_noalloc: n=%zu needs %zu scratch bytes, the static scratch holds %zu", n,
                      plan->total_bytes, NOALLOC_SCRATCH_BYTES);
        set_last_error_text(msg);
        return GBSORT_ERR_WORKSPACE_TOO_SMALL;
    }
    return GBSORT_OK;
}

}  // namespace
}  // namespace gbsort

extern "C" int gbsort_sort_keys_noalloc(int key_type, int descending, void* d_keys, size_t n, void* stream) {
    using namespace gbsort;
    Plan plan;
    const int st = noalloc_plan(key_type, n, &plan);
    if (st != GBSORT_OK) return st;
    if (n == 0) return GBSORT_OK;
    if (d_keys == nullptr) return GBSORT_ERR_INVALID_ARGUMENT;
    if (!device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    void* scratch = noalloc_scratch_for_current_device();
    if (scratch == nullptr) return GBSORT_ERR_CUDA;
    return enqueue_sort(plan, descending ? 1 : 0, d_keys, nullptr, scratch, static_cast<cudaStream_t>(stream),
                        nullptr, 0, nullptr);
}

extern "C" int gbsort_noalloc_status(int key_type, size_t n, void* stream) {
    using namespace gbsort;
    Plan plan;
    const int st = noalloc_plan(key_type, n, &plan);
    if (st != GBSORT_OK) return st;
    if (n == 0) return GBSORT_OK;
    void* scratch = noalloc_scratch_for_current_device();
    if (scratch == nullptr) return GBSORT_ERR_CUDA;
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        set_last_error("gbsort_noalloc_status: stream sync", e);
        return GBSORT_ERR_CUDA;
    }
    uint32_t err = 0;
    e = cudaMemcpy(&err, static_cast<const unsigned char*>(scratch) + plan.ctl_off + plan.ctl.err_off, sizeof err,
                   cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_last_error("gbsort_noalloc_status: error word read", e);
        return GBSORT_ERR_CUDA;
    }
    return status_from_error_word(err);
}
