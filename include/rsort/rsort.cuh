// rsort/rsort.cuh — drop-in replacement for rsort's public header, backed by
// libgbsort.so (the GB300 onesweep sort, C ABI in gbsort.h).
//
// Same names, template parameters and protocol as the reference
// (AwardOfSky/CUDA-Fast-Sort include/rsort/rsort.cuh:13-92):
//
//     size_t temp_bytes = 0;
//     uint8_t* d_workspace = nullptr;
//     rsort::sort(d_keys, &temp_bytes, d_workspace, n);   // size query
//     cudaMalloc(&d_workspace, temp_bytes);
//     rsort::sort(d_keys, &temp_bytes, d_workspace, n);   // sort in place
//
// Entry points return void like rsort's; the status of the last call on this
// thread is available from rsort::last_status() (0 = ok, see gbsort.h).  That
// status is what the host saw when the call returned (arguments, launches);
// the sort itself runs later on the stream.  A failure on the device (a
// bounded wait that ran out, a failed bounds check) is recorded in the
// workspace: rsort::synchronize_status() waits for the last sort of this
// thread, reads that record, folds it into last_status() and returns it.
// Differences from rsort: the stream argument is honoured (rsort replaces it,
// radix_kernel.cuh:583-601), n == 0 is a no-op, and any key type the
// reference accepts maps onto one of gbsort's 13 key types by size and
// signedness; `long double` of 16 bytes sorts as raw 128-bit patterns with
// the float twiddle at bit 127, as rsort does (radix_kernel.cuh:351-356).
//
// Plain C++ (no device code): compiles with nvcc or a host compiler that can
// see cuda_runtime_api.h; link with -lgbsort.
#pragma once

#include <cstddef>
#include <cstdint>
#include <type_traits>

#include <cuda_runtime_api.h>

#include "../gbsort.h"

namespace rsort {
namespace detail {

template <typename T>
constexpr int key_type_id() {
    static_assert(std::is_arithmetic<T>::value
#if defined(__SIZEOF_INT128__)
                      || std::is_same<T, unsigned __int128>::value || std::is_same<T, __int128>::value
#endif
                  , "Radix type must be a numeric.");
    static_assert(sizeof(T) <= 16, "Radix type too large.");
    if (std::is_same<T, float>::value) return GBSORT_KEY_F32;
    if (std::is_same<T, double>::value) return GBSORT_KEY_F64;
    if (std::is_same<T, long double>::value) return sizeof(long double) == 16 ? GBSORT_KEY_F128 : GBSORT_KEY_F64;
#if defined(__SIZEOF_INT128__)
    if (std::is_same<T, unsigned __int128>::value) return GBSORT_KEY_U128;
    if (std::is_same<T, __int128>::value) return GBSORT_KEY_I128;
#endif
    const bool is_signed = std::is_signed<T>::value;
    switch (sizeof(T)) {
        case 1: return is_signed ? GBSORT_KEY_I8 : GBSORT_KEY_U8;
        case 2: return is_signed ? GBSORT_KEY_I16 : GBSORT_KEY_U16;
        case 4: return is_signed ? GBSORT_KEY_I32 : GBSORT_KEY_U32;
        case 8: return is_signed ? GBSORT_KEY_I64 : GBSORT_KEY_U64;
        default: return is_signed ? GBSORT_KEY_I128 : GBSORT_KEY_U128;
    }
}

template <typename V>
constexpr size_t value_bytes() {
    static_assert(sizeof(V) == 1 || sizeof(V) == 2 || sizeof(V) == 4 || sizeof(V) == 8 || sizeof(V) == 16,
                  "value types of 1, 2, 4, 8 or 16 bytes are supported");
    static_assert(std::is_trivially_copyable<V>::value, "values are moved as raw bytes");
    return sizeof(V);
}

inline int& last_status_ref() {
    static thread_local int s = 0;
    return s;
}

// The last sort this thread enqueued (not a size query), for
// synchronize_status().
struct LastSort {
    bool valid = false;
    int key_type = 0;
    size_t value_bytes = 0;
    size_t n = 0;
    void* workspace = nullptr;
    cudaStream_t stream = nullptr;
};
inline LastSort& last_sort_ref() {
    static thread_local LastSort s;
    return s;
}

inline void record(int status, int key_type, size_t value_bytes, uint8_t* d_workspace, size_t n,
                   cudaStream_t stream) {
    last_status_ref() = status;
    LastSort& l = last_sort_ref();
    l.valid = status == GBSORT_OK && d_workspace != nullptr && n != 0;
    l.key_type = key_type;
    l.value_bytes = value_bytes;
    l.n = n;
    l.workspace = d_workspace;
    l.stream = stream;
}

}  // namespace detail

// Status of the last rsort call on this thread (GBSORT_OK == 0), as the host
// saw it when the call returned.
inline int last_status() { return detail::last_status_ref(); }

// Waits for the last sort this thread enqueued (its stream), then reports
// what happened on the device: GBSORT_OK, or GBSORT_ERR_TIMEOUT /
// GBSORT_ERR_INTERNAL recorded by the kernels.  The result also becomes
// last_status().  Read it before the workspace is reused: the next sort on
// the same workspace clears the record.
inline int synchronize_status() {
    detail::LastSort& l = detail::last_sort_ref();
    if (!l.valid) return detail::last_status_ref();
    const int st = gbsort_workspace_status(l.key_type, l.value_bytes, l.n, l.workspace, l.stream);
    detail::last_status_ref() = st;
    return st;
}

template <typename Key_T, typename Len_T>
inline void sort(Key_T* d_inout, size_t* temp_bytes, uint8_t* d_workspace, Len_T n,
                 cudaStream_t capture_stream = nullptr) {
    static_assert(std::is_integral<Len_T>::value, "Type of N (Len_T) must be an integral type");
    const int kt = detail::key_type_id<Key_T>();
    detail::record(gbsort_sort_keys(kt, 0, d_inout, temp_bytes, d_workspace, static_cast<size_t>(n), capture_stream),
                   kt, 0, d_workspace, static_cast<size_t>(n), capture_stream);
}

template <typename Key_T, typename Len_T>
inline void sort_descending(Key_T* d_inout, size_t* temp_bytes, uint8_t* d_workspace, Len_T n,
                            cudaStream_t capture_stream = nullptr) {
    static_assert(std::is_integral<Len_T>::value, "Type of N (Len_T) must be an integral type");
    const int kt = detail::key_type_id<Key_T>();
    detail::record(gbsort_sort_keys(kt, 1, d_inout, temp_bytes, d_workspace, static_cast<size_t>(n), capture_stream),
                   kt, 0, d_workspace, static_cast<size_t>(n), capture_stream);
}

template <typename Key_T, typename Len_T, typename Value_T>
inline void sort_pairs(Key_T* d_inout, Value_T* d_inout_values, size_t* temp_bytes, uint8_t* d_workspace, Len_T n,
                       cudaStream_t capture_stream = nullptr) {
    static_assert(std::is_integral<Len_T>::value, "Type of N (Len_T) must be an integral type");
    const int kt = detail::key_type_id<Key_T>();
    constexpr size_t vb = detail::value_bytes<Value_T>();
    detail::record(gbsort_sort_pairs(kt, 0, d_inout, d_inout_values, vb, temp_bytes, d_workspace,
                                     static_cast<size_t>(n), capture_stream),
                   kt, vb, d_workspace, static_cast<size_t>(n), capture_stream);
}

template <typename Key_T, typename Len_T, typename Value_T>
inline void sort_pairs_descending(Key_T* d_inout, Value_T* d_inout_values, size_t* temp_bytes, uint8_t* d_workspace,
                                  Len_T n, cudaStream_t capture_stream = nullptr) {
    static_assert(std::is_integral<Len_T>::value, "Type of N (Len_T) must be an integral type");
    const int kt = detail::key_type_id<Key_T>();
    constexpr size_t vb = detail::value_bytes<Value_T>();
    detail::record(gbsort_sort_pairs(kt, 1, d_inout, d_inout_values, vb, temp_bytes, d_workspace,
                                     static_cast<size_t>(n), capture_stream),
                   kt, vb, d_workspace, static_cast<size_t>(n), capture_stream);
}

}  // namespace rsort
