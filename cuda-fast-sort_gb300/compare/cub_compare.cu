// cub_compare.cu — benchmark comparator only (not part of libgbsort): times
// the CUDA toolkit's cub::DeviceRadixSort (DoubleBuffer form, no copy) on the
// same device buffers the benchmark sorts, so bench.py can report CUB on the
// same GB300 next to gbsort.  Built as lib/libcubcompare.so.

#include <cstdint>
#include <cub/device/device_radix_sort.cuh>

namespace {

template <class K, class V>
int run(bool pairs, int desc, void* k0, void* k1, void* v0, void* v1, size_t n, void* temp, size_t* temp_bytes,
        cudaStream_t s, int* result_in_alt) {
    cub::DoubleBuffer<K> kb(static_cast<K*>(k0), static_cast<K*>(k1));
    cub::DoubleBuffer<V> vb(static_cast<V*>(v0), static_cast<V*>(v1));
    cudaError_t e;
    const int nn = int(n);
    if (pairs) {
        e = desc ? cub::DeviceRadixSort::SortPairsDescending(temp, *temp_bytes, kb, vb, nn, 0, int(8 * sizeof(K)), s)
                 : cub::DeviceRadixSort::SortPairs(temp, *temp_bytes, kb, vb, nn, 0, int(8 * sizeof(K)), s);
    } else {
        e = desc ? cub::DeviceRadixSort::SortKeysDescending(temp, *temp_bytes, kb, nn, 0, int(8 * sizeof(K)), s)
                 : cub::DeviceRadixSort::SortKeys(temp, *temp_bytes, kb, nn, 0, int(8 * sizeof(K)), s);
    }
    if (result_in_alt) *result_in_alt = kb.selector;
    return e == cudaSuccess ? 0 : int(e);
}

}  // namespace

extern "C" {

// kind: 0 = u32 keys, 1 = f32 keys + u32 values, 2 = u64 keys + u64 values,
// 3 = u64 keys, 4 = u32 keys + u32 values.  temp == NULL: size query.
int cubcmp_sort(int kind, int desc, void* k0, void* k1, void* v0, void* v1, size_t n, void* temp,
                size_t* temp_bytes, void* stream, int* result_in_alt) {
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    switch (kind) {
        case 0: return run<uint32_t, uint32_t>(false, desc, k0, k1, v0, v1, n, temp, temp_bytes, s, result_in_alt);
        case 1: return run<float, uint32_t>(true, desc, k0, k1, v0, v1, n, temp, temp_bytes, s, result_in_alt);
        case 2: return run<uint64_t, uint64_t>(true, desc, k0, k1, v0, v1, n, temp, temp_bytes, s, result_in_alt);
        case 3: return run<uint64_t, uint64_t>(false, desc, k0, k1, v0, v1, n, temp, temp_bytes, s, result_in_alt);
        case 4: return run<uint32_t, uint32_t>(true, desc, k0, k1, v0, v1, n, temp, temp_bytes, s, result_in_alt);
        default: return -1;
    }
}

}  // extern "C"
