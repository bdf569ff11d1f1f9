// check.cu — device-side property checks of a sort's result, the GB300 form
// of the reference's post-sort checks (benchmark/benchmark_sort.cuh:26-175:
// order, digit counts, key-value pairs).  Used by the benchmark CLI's
// validation sweep and by tests at sizes no CPU checker can follow.
//   order:    adjacent keys compared as twiddled bits (so -0.0 < +0.0, NaNs at
//             the ends), counting pairs out of order
//   checksum: sum of a 64-bit mix of every key, equal for any permutation
//   pairs:    values holding the original index must point at an input key
//             equal to the output key beside them

#include <cstdint>

#include "gbsort.h"
#include "plan.h"
#include "device_common.cuh"

namespace gbsort {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z ^= z >> 30;
    z *= 0xbf58476d1ce4e5b9ull;
    z ^= z >> 27;
    z *= 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

template <class U>
__device__ __forceinline__ uint64_t key_hash(U k) {
    if constexpr (sizeof(U) == 16) {
        const u128 v = k;
        return mix64(uint64_t(v) ^ 0x9e3779b97f4a7c15ull) + mix64(uint64_t(v >> 64) ^ 0x632be59bd9b4e019ull);
    } else {
        return mix64(uint64_t(k) ^ 0x9e3779b97f4a7c15ull);
    }
}

template <int KB>
__global__ void __launch_bounds__(256) order_kernel(const void* keys, uint64_t n, int kind, int desc,
                                                    unsigned long long* violations) {
    using U = typename KeyBits<KB>::U;
    const U* k = static_cast<const U*>(keys);
    unsigned long long bad = 0;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i + 1 < n; i += stride)
        bad += twiddle_in<U>(k[i], kind, desc) > twiddle_in<U>(k[i + 1], kind, desc);
    for (int o = 16; o; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(violations, bad);
}

template <int KB>
__global__ void __launch_bounds__(256) checksum_kernel(const void* keys, uint64_t n, unsigned long long* sum) {
    using U = typename KeyBits<KB>::U;
    const U* k = static_cast<const U*>(keys);
    unsigned long long s = 0;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) s += key_hash<U>(k[i]);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sum, s);
}

template <int KB, class I>
__global__ void __launch_bounds__(256) pairs_kernel(const void* keys_in, const void* keys_out, const void* idx,
                                                    uint64_t n, unsigned long long* violations) {
    using U = typename KeyBits<KB>::U;
    const U* a = static_cast<const U*>(keys_in);
    const U* b = static_cast<const U*>(keys_out);
    const I* v = static_cast<const I*>(idx);
    unsigned long long bad = 0;
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint64_t j = uint64_t(v[i]);
        bad += (j >= n) || !(a[j] == b[i]);
    }
    for (int o = 16; o; o >>= 1) bad += __shfl_xor_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(violations, bad);
}

int kind_of(int kt) {
    if (kt >= GBSORT_KEY_F32) return KIND_FLOAT;
    if (kt >= GBSORT_KEY_I8) return KIND_SIGNED;
    return KIND_UNSIGNED;
}

// Runs `launch` with a zeroed device counter on `stream` and returns it.
template <class F>
int with_counter(cudaStream_t s, uint64_t* out, F launch) {
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        launch(d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (d) cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_last_error("check", e);
        return GBSORT_ERR_CUDA;
    }
    *out = h;
    return GBSORT_OK;
}

uint32_t grid_of(uint64_t n) {
    const uint64_t blocks = (n + 255) / 256;
    const uint64_t cap = uint64_t(device_sm_count() > 0 ? device_sm_count() : 1) * 8;
    return uint32_t(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

}  // namespace
}  // namespace gbsort

using namespace gbsort;

extern "C" {

int gbsort_check_order(int key_type, int descending, const void* d_keys, size_t n, void* stream,
                       uint64_t* violations) {
    const size_t kb = gbsort_key_bytes(key_type);
    if (kb == 0 || violations == nullptr || (n && d_keys == nullptr)) return GBSORT_ERR_INVALID_ARGUMENT;
    *violations = 0;
    if (n < 2) return GBSORT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int kind = kind_of(key_type), desc = descending ? 1 : 0;
    return with_counter(s, violations, [&](unsigned long long* d) {
        const uint32_t g = grid_of(n);
        switch (kb) {
            case 1: order_kernel<1><<<g, 256, 0, s>>>(d_keys, n, kind, desc, d); break;
            case 2: order_kernel<2><<<g, 256, 0, s>>>(d_keys, n, kind, desc, d); break;
            case 4: order_kernel<4><<<g, 256, 0, s>>>(d_keys, n, kind, desc, d); break;
            case 8: order_kernel<8><<<g, 256, 0, s>>>(d_keys, n, kind, desc, d); break;
            default: order_kernel<16><<<g, 256, 0, s>>>(d_keys, n, kind, desc, d); break;
        }
    });
}

int gbsort_checksum(int key_type, const void* d_keys, size_t n, void* stream, uint64_t* sum) {
    const size_t kb = gbsort_key_bytes(key_type);
    if (kb == 0 || sum == nullptr || (n && d_keys == nullptr)) return GBSORT_ERR_INVALID_ARGUMENT;
    *sum = 0;
    if (n == 0) return GBSORT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return with_counter(s, sum, [&](unsigned long long* d) {
        const uint32_t g = grid_of(n);
        switch (kb) {
            case 1: checksum_kernel<1><<<g, 256, 0, s>>>(d_keys, n, d); break;
            case 2: checksum_kernel<2><<<g, 256, 0, s>>>(d_keys, n, d); break;
            case 4: checksum_kernel<4><<<g, 256, 0, s>>>(d_keys, n, d); break;
            case 8: checksum_kernel<8><<<g, 256, 0, s>>>(d_keys, n, d); break;
            default: checksum_kernel<16><<<g, 256, 0, s>>>(d_keys, n, d); break;
        }
    });
}

int gbsort_check_pairs(int key_type, const void* d_keys_in, const void* d_keys_out, const void* d_index_values,
                       size_t value_bytes, size_t n, void* stream, uint64_t* violations) {
    const size_t kb = gbsort_key_bytes(key_type);
    if (kb == 0 || violations == nullptr || (value_bytes != 4 && value_bytes != 8) ||
        (n && (d_keys_in == nullptr || d_keys_out == nullptr || d_index_values == nullptr)))
        return GBSORT_ERR_INVALID_ARGUMENT;
    *violations = 0;
    if (n == 0) return GBSORT_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    return with_counter(s, violations, [&](unsigned long long* d) {
        const uint32_t g = grid_of(n);
#define GBSORT_PAIRS_LAUNCH(KBV)                                                                          \
    if (value_bytes == 4)                                                                                \
        pairs_kernel<KBV, uint32_t><<<g, 256, 0, s>>>(d_keys_in, d_keys_out, d_index_values, n, d);      \
    else                                                                                                 \
        pairs_kernel<KBV, uint64_t><<<g, 256, 0, s>>>(d_keys_in, d_keys_out, d_index_values, n, d);
        switch (kb) {
            case 1: GBSORT_PAIRS_LAUNCH(1) break;
            case 2: GBSORT_PAIRS_LAUNCH(2) break;
            case 4: GBSORT_PAIRS_LAUNCH(4) break;
            case 8: GBSORT_PAIRS_LAUNCH(8) break;
            default: GBSORT_PAIRS_LAUNCH(16) break;
        }
#undef GBSORT_PAIRS_LAUNCH
    });
}

}  // extern "C"
