// shard.cpp — bytes-balanced partition of independent sort work (the
// segments of a batched sort, or server requests) across GPUs.  No
// counterpart in the reference, which drives one GPU.
//
// Greedy longest-processing-time assignment: items in decreasing weight
// (ties: lower index first), each to the rank with the least weight so far
// (ties: lower rank).  Every rank computes the same assignment from the same
// host sizes, so ranks agree without any collective, and no data moves
// between GPUs: each rank sorts only what it owns.  Any list schedule ends
// within total/world + max_item of the ideal; LPT within 4/3 of optimal.

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#include "gbsort.h"

extern "C" {

int gbsort_partition_weights(const uint64_t* weights, size_t num_items, int world, int32_t* owner_out,
                             uint64_t* rank_load_out) {
    if (world < 1 || (num_items && (weights == nullptr || owner_out == nullptr))) return GBSORT_ERR_INVALID_ARGUMENT;
    std::vector<size_t> order(num_items);
    std::iota(order.begin(), order.end(), size_t(0));
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return weights[a] > weights[b]; });
    std::vector<uint64_t> load(size_t(world), 0);
    for (size_t i : order) {
        int best = 0;
        for (int r = 1; r < world; ++r)
            if (load[size_t(r)] < load[size_t(best)]) best = r;
        owner_out[i] = best;
        load[size_t(best)] += weights[i];
    }
    if (rank_load_out)
        for (int r = 0; r < world; ++r) rank_load_out[r] = load[size_t(r)];
    return GBSORT_OK;
}

int gbsort_partition_segments(const uint64_t* h_offsets, size_t num_segments, int world, size_t key_bytes,
                              size_t value_bytes, int32_t* owner_out, uint64_t* rank_bytes_out) {
    if (num_segments && h_offsets == nullptr) return GBSORT_ERR_INVALID_ARGUMENT;
    std::vector<uint64_t> w(num_segments);
    for (size_t i = 0; i < num_segments; ++i) {
        if (h_offsets[i + 1] < h_offsets[i]) return GBSORT_ERR_INVALID_ARGUMENT;
        w[i] = (h_offsets[i + 1] - h_offsets[i]) * uint64_t(key_bytes + value_bytes);
    }
    return gbsort_partition_weights(w.data(), num_segments, world, owner_out, rank_bytes_out);
}

}  // extern "C"
