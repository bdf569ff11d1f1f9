// generate.cu — seeded synthetic inputs on the device (gbsort_generate) and
// the bounded-wait probes (gbsort_probe_wait_timeout,
// gbsort_probe_barrier_timeout).
//
// The integer streams match cuda-fast-sort_gb300/gbsort/gen.py bit for bit.
// Distributions 4/5 restate the reference's init_keys kernel
// (include/rsort/detail/utils.cuh:245-317: mix32 avalanche of i ^ seed,
// byte_skip masking) so its own inputs can be reproduced.

#include <cstdint>

#include "gbsort.h"
#include "device_common.cuh"
#include "plan.h"

namespace gbsort {
namespace {

constexpr uint64_t GOLDEN = 0x9E3779B97F4A7C15ull;
constexpr uint64_t DIST_SALT = 0xD1B54A32D192ED03ull;
constexpr uint64_t TABLE_SALT = 0x5BD1E9955BD1E995ull;

// splitmix64 (Steele, Lea, Flood 2014), element i of the stream.
__device__ __forceinline__ uint64_t splitmix64_at(uint64_t seed, uint64_t i) {
    uint64_t z = seed + (i + 1) * GOLDEN;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ void store_bits(void* out, int kb, uint64_t i, uint64_t lo, uint64_t hi) {
    uint8_t* o = static_cast<uint8_t*>(out);
    switch (kb) {
        case 1: o[i] = uint8_t(lo); break;
        case 2: reinterpret_cast<uint16_t*>(o)[i] = uint16_t(lo); break;
        case 4: reinterpret_cast<uint32_t*>(o)[i] = uint32_t(lo); break;
        case 8: reinterpret_cast<uint64_t*>(o)[i] = lo; break;
        default:
            reinterpret_cast<uint64_t*>(o)[2 * i] = lo;
            reinterpret_cast<uint64_t*>(o)[2 * i + 1] = hi;
            break;
    }
}

__global__ void generate_kernel(int dist, int kb, void* out, uint64_t n, uint64_t seed) {
    const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        uint64_t lo = 0, hi = 0;
        switch (dist) {
            case 0:
                if (kb == 16) {
                    lo = splitmix64_at(seed, 2 * i);
                    hi = splitmix64_at(seed, 2 * i + 1);
                } else {
                    lo = splitmix64_at(seed, i);
                }
                break;
            case 1: {
                const uint64_t u = splitmix64_at(seed, i);
                const double r1 = (double(u >> 40) + 1.0) / double(1 << 24);
                const double r2 = double(u & 0xFFFFFFull) / double(1 << 24);
                const float z = float(sqrt(-2.0 * log(r1)) * cos(6.283185307179586 * r2));
                uint32_t bits = __float_as_uint(z);
                const uint64_t sel = splitmix64_at(seed ^ DIST_SALT, i) % 10000ull;
                if (sel < 100) bits = 0x80000000u;
                else if (sel < 110) bits = (sel % 2 == 0) ? 0x7F800000u : 0xFF800000u;
                else if (sel < 111) bits = 0x7FC00000u;
                lo = bits;
                break;
            }
            case 2: {
                const uint64_t u = splitmix64_at(seed, i);
                const uint64_t upper = splitmix64_at(seed ^ TABLE_SALT, u >> 56) & 0xFFFFFFFFull;
                lo = (upper << 32) | (u & 0xFFFFFFFFull);
                break;
            }
            case 3:
                lo = i;
                break;
            case 4:
            case 5: {
                const uint32_t s = uint32_t(seed);
                if (kb <= 4) {
                    lo = mix32(uint32_t(i ^ seed));
                } else if (kb == 8) {
                    lo = (uint64_t(mix32(uint32_t(i)) ^ s) << 32) | uint64_t(mix32(uint32_t(i + 0x9E3779B9ull)) ^ s);
                } else {
                    hi = (uint64_t(mix32(uint32_t(i)) ^ s) << 32) | uint64_t(mix32(uint32_t(i + 0x9E3779B9ull)) ^ s);
                    lo = (uint64_t(mix32(uint32_t(i + 0x3C6EF372ull)) ^ s) << 32) |
                         uint64_t(mix32(uint32_t(i + 0xDAA66D2Bull)) ^ s);
                }
                if (dist == 5) {
                    lo = (lo & 0xFF00FF00FF00FF00ull) | 0x0055005500550055ull;
                    if (kb == 16) hi = (hi & 0xFF00FF00FF00FF00ull) | 0x0055005500550055ull;
                }
                break;
            }
            default:
                break;
        }
        store_bits(out, kb, i, lo, hi);
    }
}

// One bounded lookback wait on a status word nothing publishes.
__global__ void probe_wait_kernel(uint32_t* scratch, uint64_t limit_ns) {
    using Codec = StatusCodec<uint32_t, 4>;
    uint32_t* word = scratch;       // never published
    uint32_t* err = scratch + 1;
    (void)wait_status<Codec>(word, 1u, limit_ns, err);
}

// One grid barrier that can never complete: a single CTA waits for a second
// arrival (phase 2 of a one-CTA grid) that nothing makes.
__global__ void probe_barrier_kernel(uint32_t* scratch, uint64_t limit_ns) {
    uint32_t* counter = scratch;
    uint32_t* err = scratch + 1;
    uint32_t* gen = scratch + 8;
    (void)grid_barrier(counter, gen, 2u, limit_ns, err);
}

}  // namespace
}  // namespace gbsort

extern "C" {

int gbsort_generate(int dist, size_t key_bytes, void* d_out, size_t n, uint64_t seed, void* stream) {
    using namespace gbsort;
    if (n == 0) return GBSORT_OK;
    if (d_out == nullptr || dist < 0 || dist > 5) return GBSORT_ERR_INVALID_ARGUMENT;
    if (!(key_bytes == 1 || key_bytes == 2 || key_bytes == 4 || key_bytes == 8 || key_bytes == 16))
        return GBSORT_ERR_INVALID_ARGUMENT;
    if ((dist == 1 && key_bytes != 4) || (dist == 2 && key_bytes != 8)) return GBSORT_ERR_INVALID_ARGUMENT;
    if (!device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    const int sms = device_sm_count();
    const uint64_t want = (n + 255) / 256;
    const uint32_t grid = uint32_t(want < uint64_t(sms) * 8 ? want : uint64_t(sms) * 8);
    generate_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(dist, int(key_bytes), d_out, n, seed);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error("generate launch", e);
        return GBSORT_ERR_CUDA;
    }
    return GBSORT_OK;
}

int gbsort_probe_wait_timeout(void* d_scratch, uint64_t limit_ns, void* stream) {
    using namespace gbsort;
    if (d_scratch == nullptr) return GBSORT_ERR_INVALID_ARGUMENT;
    if (!device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(d_scratch, 0, 64, s);
    if (e == cudaSuccess) {
        probe_wait_kernel<<<1, 1, 0, s>>>(static_cast<uint32_t*>(d_scratch), limit_ns);
        e = cudaGetLastError();
    }
    uint32_t err = 0;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpy(&err, static_cast<uint32_t*>(d_scratch) + 1, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_last_error("wait probe", e);
        return GBSORT_ERR_CUDA;
    }
    return err ? GBSORT_ERR_TIMEOUT : GBSORT_OK;
}

int gbsort_probe_barrier_timeout(void* d_scratch, uint64_t limit_ns, void* stream) {
    using namespace gbsort;
    if (d_scratch == nullptr) return GBSORT_ERR_INVALID_ARGUMENT;
    if (!device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemsetAsync(d_scratch, 0, 64, s);
    if (e == cudaSuccess) {
        probe_barrier_kernel<<<1, 64, 0, s>>>(static_cast<uint32_t*>(d_scratch), limit_ns);
        e = cudaGetLastError();
    }
    uint32_t err = 0;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpy(&err, static_cast<uint32_t*>(d_scratch) + 1, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_last_error("barrier probe", e);
        return GBSORT_ERR_CUDA;
    }
    return err ? GBSORT_ERR_TIMEOUT : GBSORT_OK;
}

}  // extern "C"
