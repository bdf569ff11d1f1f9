// rsort_shim_test.cpp — uses the drop-in header exactly as rsort's own
// examples do (examples/example_basic.cu:27-43 of the reference: size query,
// cudaMalloc of the workspace, in-place sort) for several key/value types and
// both orders, then checks each result on the host the way the reference's
// validation does (benchmark/benchmark_sort.cuh:396-461 / utils.cuh:341-432:
// order, key-value pairing, stability) and against std::stable_sort of the
// twiddled keys.  Exit code 0 = all passed.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include <cuda_runtime.h>

#include "rsort/rsort.cuh"

namespace {

using u128 = unsigned __int128;

template <class T> struct Bits { using U = T; };
template <> struct Bits<float> { using U = uint32_t; };
template <> struct Bits<double> { using U = uint64_t; };
template <> struct Bits<long double> { using U = u128; };
template <> struct Bits<int8_t> { using U = uint8_t; };
template <> struct Bits<int32_t> { using U = uint32_t; };
template <> struct Bits<int64_t> { using U = uint64_t; };
template <> struct Bits<__int128> { using U = u128; };

// Order-preserving bits (restated from the reference's tuning.cuh:352-367).
template <class T>
typename Bits<T>::U ordered(const T& x, bool desc) {
    using U = typename Bits<T>::U;
    U b;
    std::memcpy(&b, &x, sizeof(U));
    const U sign = U(U(1) << (8 * sizeof(U) - 1));
    if (std::is_floating_point<T>::value) b = (b & sign) ? U(~b) : U(b ^ sign);
    else if (std::is_signed<T>::value || std::is_same<T, __int128>::value) b = U(b ^ sign);
    return desc ? U(~b) : b;
}

std::mt19937_64 rng(2024);

template <class T> T random_key() {
    typename Bits<T>::U b = 0;
    for (size_t i = 0; i < sizeof(b); i += 8) {
        uint64_t r = rng();
        std::memcpy(reinterpret_cast<char*>(&b) + i, &r, std::min<size_t>(8, sizeof(b) - i));
    }
    if (rng() % 8 == 0) b = 0;  // duplicates
    T x;
    std::memset(&x, 0, sizeof(T));
    std::memcpy(&x, &b, sizeof(b));
    return x;
}

template <class K, class V>
bool run_case(const char* name, size_t n, bool desc) {
    std::vector<K> keys(n);
    for (auto& k : keys) k = random_key<K>();
    std::vector<V> vals(n);
    for (size_t i = 0; i < n; ++i) vals[i] = V(i);

    K* d_keys = nullptr;
    V* d_vals = nullptr;
    cudaMalloc(&d_keys, n * sizeof(K));
    cudaMalloc(&d_vals, n * sizeof(V));
    cudaMemcpy(d_keys, keys.data(), n * sizeof(K), cudaMemcpyHostToDevice);
    cudaMemcpy(d_vals, vals.data(), n * sizeof(V), cudaMemcpyHostToDevice);

    size_t temp_bytes = 0;
    uint8_t* d_workspace = nullptr;
    if (desc) rsort::sort_pairs_descending<K, size_t, V>(d_keys, d_vals, &temp_bytes, d_workspace, n);
    else rsort::sort_pairs<K, size_t, V>(d_keys, d_vals, &temp_bytes, d_workspace, n);
    if (rsort::last_status() != 0 || temp_bytes == 0) {
        std::printf("%s: size query failed (%d)\n", name, rsort::last_status());
        return false;
    }
    cudaMalloc(&d_workspace, temp_bytes);
    if (desc) rsort::sort_pairs_descending<K, size_t, V>(d_keys, d_vals, &temp_bytes, d_workspace, n);
    else rsort::sort_pairs<K, size_t, V>(d_keys, d_vals, &temp_bytes, d_workspace, n);
    const int st = rsort::last_status();
    cudaDeviceSynchronize();

    std::vector<K> out_k(n);
    std::vector<V> out_v(n);
    cudaMemcpy(out_k.data(), d_keys, n * sizeof(K), cudaMemcpyDeviceToHost);
    cudaMemcpy(out_v.data(), d_vals, n * sizeof(V), cudaMemcpyDeviceToHost);
    cudaFree(d_keys);
    cudaFree(d_vals);
    cudaFree(d_workspace);

    // std::stable_sort of the twiddled keys: the expected permutation
    std::vector<size_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(),
                     [&](size_t a, size_t b) { return ordered(keys[a], desc) < ordered(keys[b], desc); });
    bool ok = st == 0;
    for (size_t i = 0; ok && i < n; ++i) {
        ok = std::memcmp(&out_k[i], &keys[idx[i]], sizeof(typename Bits<K>::U)) == 0 && out_v[i] == V(idx[i]);
        if (ok && i + 1 < n) {
            // the reference's own three checks: order, pairing, stability
            const auto a = ordered(out_k[i], desc), b = ordered(out_k[i + 1], desc);
            ok = a <= b && !(a == b && out_v[i] > out_v[i + 1]);
        }
    }
    std::printf("%-26s n=%-8zu %s  %s\n", name, n, desc ? "DESC" : "ASC ", ok ? "passed" : "FAILED");
    return ok;
}

template <class K>
bool run_keys_case(const char* name, size_t n) {
    std::vector<K> keys(n);
    for (auto& k : keys) k = random_key<K>();
    K* d = nullptr;
    cudaMalloc(&d, n * sizeof(K));
    cudaMemcpy(d, keys.data(), n * sizeof(K), cudaMemcpyHostToDevice);
    size_t temp_bytes = 0;
    uint8_t* ws = nullptr;
    rsort::sort(d, &temp_bytes, ws, n);
    cudaMalloc(&ws, temp_bytes);
    rsort::sort(d, &temp_bytes, ws, n);
    const int st = rsort::last_status();
    std::vector<K> out(n);
    cudaMemcpy(out.data(), d, n * sizeof(K), cudaMemcpyDeviceToHost);
    cudaFree(d);
    cudaFree(ws);
    std::vector<typename Bits<K>::U> ref(n);
    for (size_t i = 0; i < n; ++i) ref[i] = ordered(keys[i], false);
    std::sort(ref.begin(), ref.end());
    bool ok = st == 0;
    for (size_t i = 0; ok && i < n; ++i) ok = ordered(out[i], false) == ref[i];
    std::printf("%-26s n=%-8zu ASC   %s\n", name, n, ok ? "passed" : "FAILED");
    return ok;
}

// A sort whose bounded device waits run out (a 1 ns limit) returns normally
// from the host call; rsort::synchronize_status() reports the timeout the
// kernels recorded in the workspace.  The same workspace then sorts
// correctly again and reports OK.
bool run_timeout_case() {
    const size_t n = size_t(1) << 21;
    std::vector<uint32_t> keys(n);
    for (auto& k : keys) k = uint32_t(rng());
    uint32_t* d = nullptr;
    cudaMalloc(&d, n * sizeof(uint32_t));
    size_t temp_bytes = 0;
    uint8_t* ws = nullptr;
    rsort::sort(d, &temp_bytes, ws, n);
    cudaMalloc(&ws, temp_bytes);
    const uint64_t old_limit = gbsort_get_wait_limit_ns();
    gbsort_set_wait_limit_ns(1);
    int host_st = -1, dev_st = GBSORT_OK;
    for (int attempt = 0; attempt < 3 && dev_st == GBSORT_OK; ++attempt) {
        cudaMemcpy(d, keys.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice);
        rsort::sort(d, &temp_bytes, ws, n);
        host_st = rsort::last_status();
        dev_st = rsort::synchronize_status();
    }
    const bool folded = rsort::last_status() == dev_st;
    gbsort_set_wait_limit_ns(old_limit);
    cudaMemcpy(d, keys.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice);
    rsort::sort(d, &temp_bytes, ws, n);
    const int ok_st = rsort::synchronize_status();
    std::vector<uint32_t> out(n);
    cudaMemcpy(out.data(), d, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    cudaFree(d);
    cudaFree(ws);
    std::sort(keys.begin(), keys.end());
    const bool ok = host_st == GBSORT_OK && dev_st == GBSORT_ERR_TIMEOUT && folded && ok_st == GBSORT_OK &&
                    out == keys;
    std::printf("%-26s n=%-8zu host %d, device %d, after %d  %s\n", "timeout via shim", n, host_st, dev_st, ok_st,
                ok ? "passed" : "FAILED");
    return ok;
}

}  // namespace

int main() {
    bool ok = true;
    ok &= run_keys_case<uint32_t>("sort<uint32_t>", 1 << 20);
    ok &= run_keys_case<int8_t>("sort<int8_t>", 100000);
    ok &= run_keys_case<long double>("sort<long double>", 50000);
    ok &= run_case<float, uint32_t>("sort_pairs<float,u32>", 300001, false);
    ok &= run_case<int64_t, uint64_t>("sort_pairs<int64,u64>", 200003, true);
    ok &= run_case<double, uint16_t>("sort_pairs<double,u16>", 40000, false);
    ok &= run_case<__int128, uint32_t>("sort_pairs<int128,u32>", 60000, true);
    ok &= run_case<int32_t, uint8_t>("sort_pairs<int32,u8>", 255, false);
    // n == 0 is a no-op
    size_t tb = 0;
    uint32_t* none = nullptr;
    rsort::sort(none, &tb, reinterpret_cast<uint8_t*>(1), size_t(0));
    ok &= rsort::last_status() == 0;
    ok &= run_timeout_case();
    std::printf("%s\n", ok ? "ALL PASSED" : "SOME FAILED");
    return ok ? 0 : 1;
}
