// autotune.cu — the batched sort's autotuner and tuning-table text form.
//
// For each size bucket [2^b, 2^(b+1)) it builds a synthetic batch of segments
// of that size in caller-provided device scratch (nothing is allocated),
// times every path able to hold them — CTA sort with 4-bit digits
// (256 threads x 8 keys), CTA sort with 8-bit digits (same tile), the bigger
// CTA sort (512 threads, 8-bit), onesweep passes over the global tile list —
// with CUDA events (median of several runs on fresh random keys), and installs
// the fastest in the tuning table.  Each path is a different tile shape,
// items-per-thread and radix width, so this picks all three per bucket.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbsort.h"
#include "plan.h"

namespace {

struct Candidate {
    int path;
    const char* name;
};

int time_plan(gbsort_segmented_plan* p, int key_bytes, size_t value_bytes, void* keys, void* vals, size_t n,
              void* ws, size_t ws_bytes, cudaStream_t s, int reps, float* median_ms) {
    int st = gbsort_segmented_bind(p, keys, vals, ws, ws_bytes, s);
    if (st != GBSORT_OK) return st;
    std::vector<float> t;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    for (int r = 0; r < reps + 1; ++r) {
        st = gbsort_generate(0, size_t(key_bytes), keys, n, 977u + r, s);
        if (st == GBSORT_OK && value_bytes) st = gbsort_generate(3, value_bytes, vals, n, 0, s);
        if (st != GBSORT_OK) break;
        cudaEventRecord(a, s);
        st = gbsort_segmented_run(p, 1, s);
        cudaEventRecord(b, s);
        if (st != GBSORT_OK) break;
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (r > 0) t.push_back(ms);  // first run captures the graph
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (st != GBSORT_OK) return st;
    std::sort(t.begin(), t.end());
    *median_ms = t[t.size() / 2];
    return gbsort_segmented_status(p, s);
}

}  // namespace

extern "C" {

int gbsort_autotune_segmented(int key_type, size_t value_bytes, int descending, int min_log2, int max_log2,
                              void* d_scratch, size_t scratch_bytes, void* stream, char* report, size_t report_cap) {
    const size_t kb = gbsort_key_bytes(key_type);
    if (kb == 0 || d_scratch == nullptr || min_log2 < 1 || max_log2 > 30 || min_log2 > max_log2)
        return GBSORT_ERR_INVALID_ARGUMENT;
    if (!gbsort::device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::string rep;
    const Candidate cands[] = {{GBSORT_PATH_CTA_S4, "cta256x8/4bit"},
                               {GBSORT_PATH_CTA_S, "cta256x8/8bit"},
                               {GBSORT_PATH_CTA_L, "cta512/8bit"},
                               {GBSORT_PATH_ONESWEEP, "onesweep/8bit"}};
    uint8_t* base = static_cast<uint8_t*>(d_scratch);
    for (int b = min_log2; b <= max_log2; ++b) {
        // ~4M keys per bucket (at least 8 segments), sizes spread over the bucket
        const uint64_t lo = uint64_t(1) << b;
        const uint64_t target = uint64_t(1) << 22;
        const uint64_t m = std::max<uint64_t>(8, std::min<uint64_t>(20000, target / lo));
        std::vector<uint64_t> off(m + 1, 0);
        for (uint64_t i = 0; i < m; ++i) off[i + 1] = off[i] + lo + (lo - 1) * i / std::max<uint64_t>(1, m - 1);
        const size_t n = off[m];
        const size_t kbytes = gbsort::align_up(n * kb, 256), vbytes = gbsort::align_up(n * value_bytes, 256);
        char line[512];
        int off_line = std::snprintf(line, sizeof line, "bucket %2d (%llu segs of %llu..%llu keys):", b,
                                     (unsigned long long)m, (unsigned long long)lo,
                                     (unsigned long long)(2 * lo - 1));
        int best = -1;
        float best_ms = 0.f;
        for (const Candidate& c : cands) {
            gbsort_set_segmented_path(key_type, value_bytes, b, c.path);
            if (gbsort_get_segmented_path(key_type, value_bytes, b) != c.path) continue;  // cannot hold it
            // the plan below must put every segment of the bucket on this path
            // (the bucket's largest may not fit a CTA: then it is skipped)
            gbsort_segmented_plan* p = nullptr;
            int st = gbsort_segmented_plan_create(key_type, value_bytes, descending, off.data(), m, &p);
            if (st != GBSORT_OK) continue;
            gbsort_segmented_info info{};
            gbsort_segmented_plan_info(p, &info);
            const bool pure = (c.path == GBSORT_PATH_ONESWEEP && info.onesweep_segments == m) ||
                              (c.path == GBSORT_PATH_CTA_S && info.cta_small_segments == m) ||
                              (c.path == GBSORT_PATH_CTA_S4 && info.cta_small4_segments == m) ||
                              (c.path == GBSORT_PATH_CTA_L && info.cta_large_segments == m);
            const size_t need = kbytes + vbytes + info.workspace_bytes;
            float ms = 0.f;
            if (pure && need <= scratch_bytes) {
                st = time_plan(p, int(kb), value_bytes, base, value_bytes ? base + kbytes : nullptr, n,
                               base + kbytes + vbytes, scratch_bytes - kbytes - vbytes, s, 5, &ms);
                if (st == GBSORT_OK) {
                    off_line += std::snprintf(line + off_line, sizeof line - off_line, " %s %.1f us", c.name,
                                              1000.0 * ms);
                    if (best < 0 || ms < best_ms) {
                        best = c.path;
                        best_ms = ms;
                    }
                }
            }
            gbsort_segmented_plan_destroy(p);
        }
        gbsort_set_segmented_path(key_type, value_bytes, b, best);  // -1: built-in thresholds
        std::snprintf(line + off_line, sizeof line - off_line, " -> %s\n",
                      best < 0 ? "(default)" : best == GBSORT_PATH_CTA_S4 ? "cta256x8/4bit"
                                             : best == GBSORT_PATH_CTA_S ? "cta256x8/8bit"
                                             : best == GBSORT_PATH_CTA_L ? "cta512/8bit" : "onesweep/8bit");
        rep += line;
    }
    if (report && report_cap) {
        std::strncpy(report, rep.c_str(), report_cap - 1);
        report[report_cap - 1] = 0;
    }
    return GBSORT_OK;
}

// Tuning table as text: one line "key_type value_bytes size_log2 path" per
// bucket that has an explicit path.
int gbsort_segmented_tuning_text(char* buf, size_t cap) {
    std::string out;
    const size_t vbs[] = {0, 1, 2, 4, 8, 16};
    for (int kt = 0; kt < GBSORT_KEY_COUNT; ++kt) {
        if (kt != GBSORT_KEY_U8 && kt != GBSORT_KEY_U16 && kt != GBSORT_KEY_U32 && kt != GBSORT_KEY_U64 &&
            kt != GBSORT_KEY_U128)
            continue;  // paths are per key width; the unsigned type names each width
        for (size_t vb : vbs)
            for (int b = 0; b <= 40; ++b) {
                const int path = gbsort_segmented_path_override(kt, vb, b);
                if (path >= 0) {
                    char line[64];
                    std::snprintf(line, sizeof line, "%d %zu %d %d\n", kt, vb, b, path);
                    out += line;
                }
            }
    }
    if (buf && cap) {
        std::strncpy(buf, out.c_str(), cap - 1);
        buf[cap - 1] = 0;
    }
    return int(out.size());
}

int gbsort_segmented_tuning_load(const char* text) {
    if (!text) return GBSORT_ERR_INVALID_ARGUMENT;
    const char* p = text;
    while (*p) {
        int kt, b, path;
        size_t vb;
        int used = 0;
        if (std::sscanf(p, "%d %zu %d %d%n", &kt, &vb, &b, &path, &used) != 4) break;
        const int st = gbsort_set_segmented_path(kt, vb, b, path);
        if (st != GBSORT_OK) return st;
        p += used;
        while (*p == '\n' || *p == ' ' || *p == '\r') ++p;
    }
    return GBSORT_OK;
}

}  // extern "C"
