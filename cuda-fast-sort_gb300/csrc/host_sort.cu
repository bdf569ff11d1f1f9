// host_sort.cu — sorting arrays that live in host memory (gbsort_sort_host):
// copy in, sort, copy back, through one caller-provided device buffer.  No
// reference counterpart: rsort sorts device arrays only
// (include/rsort/rsort.cuh:13-92); its benchmark copies around the call.
//
// The host link, not the sort, bounds this call (2^28 u32 keys: ~5 ms each
// way against a 4 ms sort), so large arrays are sorted most significant digit
// first and the copy back overlaps the sorting (2^28 u32: 14.7 -> 12.1 ms):
//   1. keys arrive in chunks on a copy stream; each chunk's digits are
//      counted (upsweep) as soon as it lands; the counts are read back
//   2. one onesweep pass on the top digit partitions half A of the buffer
//      stably into the 256 buckets of half B
//   3. consecutive buckets form groups of ~2^24 keys (2 to 16 groups;
//      GBSORT_HOST_SPLIT_GROUPS overrides); each group is sorted alone (upsweep + LSD passes over its
//      slice, alternating between B and A) on the caller's stream, and its
//      slice goes back to the host on the copy stream as soon as its last
//      pass is done, while the next groups sort.
// The result is the plain LSD sort's: the partition is stable, every group's
// sort is stable, and a group holding several buckets is also sorted by the
// top digit (its last pass).  Digits uniform over the whole array are
// skipped (unless pass skipping is off); when the top digit puts more than
// half of the keys into one bucket the partition is left out (one group,
// every varying digit).  Arrays below GBSORT_HOST_SPLIT_MIN keys (2^25) and
// 1-byte keys take the plain path: copy in, sort, copy back.

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>
#include <vector>

#include "gbsort.h"
#include "plan.h"
#include "device_common.cuh"
#include "sort_params.h"
#include "segmented_internal.h"

namespace gbsort {

namespace {

uint64_t env_u64(const char* name, uint64_t dflt) {
    const char* v = std::getenv(name);
    if (v == nullptr || *v == 0) return dflt;
    char* end = nullptr;
    const unsigned long long x = std::strtoull(v, &end, 10);
    return (end != nullptr && *end == 0) ? uint64_t(x) : dflt;
}

// The split pays once each group is a sort of ~2^24 keys or more: smaller
// sorts are latency-bound (2^20 keys: ~60 us), so 16 groups of 2^20 made a
// 2^24-key call slower (1.64 ms against 0.99 ms plain), while 16 groups of
// 2^24 keys take a 2^28-key call from 14.7 to 12.1 ms.
uint64_t split_min_keys() { return env_u64("GBSORT_HOST_SPLIT_MIN", uint64_t(1) << 25); }

// Groups for n keys: GBSORT_HOST_SPLIT_GROUPS, else one per 2^24 keys (2..16).
int split_groups(uint64_t n) {
    const uint64_t dflt = std::min<uint64_t>(16, std::max<uint64_t>(2, n >> 24));
    const uint64_t g = env_u64("GBSORT_HOST_SPLIT_GROUPS", dflt);
    return int(g < 1 ? 1 : (g > 256 ? 256 : g));
}

constexpr int IN_CHUNKS = 8;  // host-to-device copies counted as they land

// Control block + lookback status of a plan, laid out back to back.
size_t ctl_status_bytes(const Plan& p) { return p.ctl.bytes + align_up(p.status_bytes, 256); }

// Split-path layout of d_buffer: [A keys][A values][B keys][B values]
// [control block + status, sized for any group of <= n keys][error word].
struct SplitLayout {
    size_t a_keys = 0, a_vals = 0, b_keys = 0, b_vals = 0;
    size_t scratch = 0, scratch_bytes = 0, err = 0, total = 0;
};

int split_layout(int key_type, size_t vb, uint64_t n, SplitLayout* L) {
    Plan full, small;
    int st = make_plan(key_type, vb, n, &full);
    if (st != GBSORT_OK) return st;
    // tiles of the short-array shape are smaller: a group of <= 2^22 keys
    // can need more status words than a longer array
    st = make_plan(key_type, vb, std::min<uint64_t>(n, SMALL_N_MAX), &small);
    if (st != GBSORT_OK) return st;
    const size_t kbytes = align_up(size_t(n) * size_t(full.kb), 256), vbytes = align_up(size_t(n) * vb, 256);
    L->a_keys = 0;
    L->a_vals = kbytes;
    L->b_keys = kbytes + vbytes;
    L->b_vals = 2 * kbytes + vbytes;
    L->scratch = 2 * (kbytes + vbytes);
    L->scratch_bytes = std::max(ctl_status_bytes(full), ctl_status_bytes(small));
    L->err = L->scratch + L->scratch_bytes;
    L->total = L->err + 256;
    return GBSORT_OK;
}

// Plain-path layout: [keys][values][the sort's workspace].
size_t plain_bytes(const Plan& p, size_t vb) {
    size_t off = align_up(size_t(p.n) * size_t(p.kb), 256);
    off = align_up(off + size_t(p.n) * vb, 256);
    return off + p.total_bytes;
}

// Two non-blocking copy streams per device (0: the host sort's copies and
// the batched copies in, 1: the batched copies out), created on first use.
cudaStream_t copy_stream(int which = 0) {
    static std::mutex mu;
    static cudaStream_t streams[64][2] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    cudaStream_t& st = streams[dev][which & 1];
    if (st == nullptr && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        st = nullptr;
    }
    return st;
}

uint32_t pass_ctas(const Plan& p) {
    const uint64_t cap = uint64_t(std::max(1, device_sm_count())) * uint64_t(std::max(1, resident_ctas(p.pass)));
    return uint32_t(std::min<uint64_t>(p.num_tiles, cap));
}

cudaError_t launch_upsweep(const Plan& p, int desc, const void* keys, uint64_t n, unsigned long long* gp,
                           void* status, uint64_t status_bytes, cudaStream_t s) {
    HistParams hp{};
    hp.keys = keys;
    hp.n = n;
    hp.kind = p.kind;
    hp.desc = desc;
    hp.gp_counts = gp;
    hp.status = status;
    hp.status_bytes = status_bytes;
    void* args[] = {&hp};
    return cudaLaunchKernel(p.upsweep.fn, dim3(upsweep_ctas(n, p.kb)), dim3(p.upsweep.threads), args, p.upsweep.smem,
                            s);
}

// One onesweep pass of plan p on digit q, keys_in -> keys_out, with the
// plan's control block and status array at ctl.
cudaError_t launch_pass(const Plan& p, int q, int desc, const void* kin, const void* vin, void* kout, void* vout,
                        bool tw_load, bool tw_store, uint8_t* ctl, uint32_t* err, cudaStream_t s) {
    PassParams pp{};
    pp.keys_in = kin;
    pp.keys_out = kout;
    pp.vals_in = p.vb ? vin : nullptr;
    pp.vals_out = p.vb ? vout : nullptr;
    pp.n = p.n;
    pp.num_tiles = p.num_tiles;
    pp.pass = q;
    pp.kind = p.kind;
    pp.desc = desc;
    pp.twiddle_load = tw_load ? 1 : 0;
    pp.twiddle_store = tw_store ? 1 : 0;
    pp.tma_keys = 1;
    pp.tma_vals = p.vb ? 1 : 0;
    pp.gp_counts = reinterpret_cast<const unsigned long long*>(ctl + p.ctl.gp_off) + size_t(q) * 256;
    pp.status = ctl + p.ctl.bytes;
    pp.tile_counter = reinterpret_cast<uint32_t*>(ctl + p.ctl.counters_off) + q;
    pp.err = err;
    pp.wait_limit_ns = wait_limit_ns();
    pp.skip = 0;  // the host chose the digits
    pp.passes = p.passes;
    void* args[] = {&pp};
    return cudaLaunchKernel(p.pass.fn, dim3(pass_ctas(p)), dim3(p.pass.threads), args, p.pass.smem, s);
}

struct Group {
    uint64_t begin = 0, end = 0;
    bool one_bucket = false;
};

int sort_host_split(const Plan& P, int key_type, int desc, uint8_t* h_keys, uint8_t* h_vals, size_t vb,
                    uint8_t* base, const SplitLayout& L, cudaStream_t s) {
    const uint64_t n = P.n;
    const size_t kb = size_t(P.kb);
    uint8_t* A_k = base + L.a_keys;
    uint8_t* A_v = vb ? base + L.a_vals : nullptr;
    uint8_t* B_k = base + L.b_keys;
    uint8_t* B_v = vb ? base + L.b_vals : nullptr;
    uint8_t* ctl = base + L.scratch;
    uint32_t* err = reinterpret_cast<uint32_t*>(base + L.err);
    cudaStream_t cs = copy_stream();
    if (cs == nullptr) {
        set_last_error_text("host sort: no copy stream");
        return GBSORT_ERR_CUDA;
    }
    int st = prepare_kernel(P.pass);
    if (st == GBSORT_OK) st = prepare_kernel(P.upsweep);
    if (st != GBSORT_OK) return st;

    std::vector<cudaEvent_t> evs;
    auto event = [&](cudaEvent_t* ev) {
        const cudaError_t e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e == cudaSuccess) evs.push_back(*ev);
        return e;
    };
    // GBSORT_HOST_TRACE=1: device times of the phases, printed on stderr
    const bool trace = env_u64("GBSORT_HOST_TRACE", 0) == 1;
    std::vector<std::pair<std::string, cudaEvent_t>> marks;
    auto mark = [&](const std::string& label, cudaStream_t st) {
        if (!trace) return;
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        evs.push_back(ev);
        cudaEventRecord(ev, st);
        marks.emplace_back(label, ev);
    };
    const auto t_host0 = std::chrono::steady_clock::now();
    auto host_ms = [&] {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_host0).count();
    };
    std::string host_log;
    auto finish = [&](int status) {
        if (trace && !marks.empty()) {
            std::fprintf(stderr, "gbsort-host n=%llu%s\n", (unsigned long long)P.n, host_log.c_str());
            for (const auto& m : marks) {
                float t = 0.f;
                if (cudaEventElapsedTime(&t, marks[0].second, m.second) != cudaSuccess) cudaGetLastError();
                std::fprintf(stderr, "  %-28s %9.3f ms\n", m.first.c_str(), double(t));
            }
        }
        for (cudaEvent_t ev : evs) cudaEventDestroy(ev);
        return status;
    };
    auto fail = [&](const char* what, cudaError_t e) {
        set_last_error(what, e);
        // nothing of this call may still run when it returns
        cudaStreamSynchronize(cs);
        cudaStreamSynchronize(s);
        cudaGetLastError();
        return finish(GBSORT_ERR_CUDA);
    };
    cudaError_t e;

    // ---- 1. keys in by chunks, each counted as it lands
    unsigned long long* gp = reinterpret_cast<unsigned long long*>(ctl + P.ctl.gp_off);
    cudaEvent_t ev_start;
    if ((e = event(&ev_start)) != cudaSuccess) return fail("host sort event", e);
    if ((e = cudaMemsetAsync(ctl, 0, P.ctl.bytes, s)) != cudaSuccess) return fail("host sort memset", e);
    if ((e = cudaMemsetAsync(err, 0, 4, s)) != cudaSuccess) return fail("host sort memset", e);
    if ((e = cudaEventRecord(ev_start, s)) != cudaSuccess) return fail("host sort event", e);
    mark("start", s);
    if ((e = cudaStreamWaitEvent(cs, ev_start, 0)) != cudaSuccess) return fail("host sort event", e);
    const uint64_t chunk = align_up((n + IN_CHUNKS - 1) / IN_CHUNKS, 1024);
    for (uint64_t c0 = 0; c0 < n; c0 += chunk) {
        const uint64_t m = std::min(chunk, n - c0);
        cudaEvent_t ev;
        if ((e = event(&ev)) != cudaSuccess) return fail("host sort event", e);
        e = cudaMemcpyAsync(A_k + c0 * kb, h_keys + c0 * kb, m * kb, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess) e = cudaEventRecord(ev, cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev, 0);
        // the first chunk's upsweep also clears the partition pass's status words
        if (e == cudaSuccess)
            e = launch_upsweep(P, desc, A_k + c0 * kb, m, gp, ctl + P.ctl.bytes, c0 == 0 ? P.status_bytes : 0, s);
        if (e != cudaSuccess) return fail("host sort copy in", e);
    }
    if (vb) {
        cudaEvent_t ev;
        if ((e = event(&ev)) != cudaSuccess) return fail("host sort event", e);
        e = cudaMemcpyAsync(A_v, h_vals, n * vb, cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess) e = cudaEventRecord(ev, cs);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev, 0);
        if (e != cudaSuccess) return fail("host sort copy in", e);
    }
    mark("keys and values in", cs);
    mark("counted", s);
    std::vector<unsigned long long> cnt(size_t(P.passes) * 256);
    e = cudaMemcpyAsync(cnt.data(), gp, cnt.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail("host sort counts", e);
    if (trace) host_log += " counts_read_ms=" + std::to_string(host_ms());

    // ---- 2. which digits vary; partition by the top digit
    const int top = P.passes - 1;
    uint32_t vary = 0;
    for (int q = 0; q < P.passes; ++q) {
        bool uniform = false;
        for (int d = 0; d < 256; ++d) uniform |= cnt[size_t(q) * 256 + d] == n;
        if (!uniform) vary |= 1u << q;
    }
    if (!gbsort_get_pass_skip()) vary = (P.passes >= 32) ? 0xffffffffu : ((1u << P.passes) - 1u);
    const unsigned long long* top_cnt = &cnt[size_t(top) * 256];
    const unsigned long long biggest = *std::max_element(top_cnt, top_cnt + 256);
    const bool partition = ((vary >> top) & 1u) != 0 && biggest <= n / 2;
    std::vector<Group> groups;
    uint8_t *src_k = A_k, *src_v = A_v;
    if (partition) {
        e = launch_pass(P, top, desc, A_k, A_v, B_k, B_v, true, true, ctl, err, s);
        if (e != cudaSuccess) return fail("host sort partition", e);
        mark("partitioned", s);
        src_k = B_k;
        src_v = B_v;
        const int G = split_groups(n);
        const uint64_t target = (n + uint64_t(G) - 1) / uint64_t(G);
        uint64_t at = 0, begin = 0;
        int first_bucket = -1;
        for (int d = 0; d < 256; ++d) {
            if (top_cnt[d] == 0) continue;
            if (first_bucket < 0) first_bucket = d;
            at += top_cnt[d];
            if (at - begin >= target || at == n) {
                groups.push_back(Group{begin, at, first_bucket == d});
                begin = at;
                first_bucket = -1;
            }
        }
    } else {
        groups.push_back(Group{0, n, false});
    }

    // ---- 3. sort every group; its slice goes home once its last pass ran
    struct Out {
        uint8_t* k;
        uint8_t* v;
        uint64_t begin, count;
        cudaEvent_t done;
    };
    std::vector<Out> outs;
    for (const Group& g : groups) {
        const uint64_t m = g.end - g.begin;
        uint8_t* cur_k = src_k + g.begin * kb;
        uint8_t* cur_v = src_v ? src_v + g.begin * vb : nullptr;
        uint8_t* oth_k = (src_k == A_k ? B_k : A_k) + g.begin * kb;
        uint8_t* oth_v = vb ? (src_k == A_k ? B_v : A_v) + g.begin * vb : nullptr;
        uint32_t digits = vary;
        if (partition) {
            digits &= (1u << top) - 1u;
            if (!g.one_bucket) digits |= 1u << top;  // buckets of the group ordered last
        }
        if (digits) {
            Plan G;
            st = make_plan(key_type, vb, m, &G);
            if (st == GBSORT_OK && ctl_status_bytes(G) > L.scratch_bytes) {
                set_last_error_text("host sort: group workspace exceeds its reservation");
                st = GBSORT_ERR_INTERNAL;
            }
            if (st == GBSORT_OK) st = prepare_kernel(G.pass);
            if (st != GBSORT_OK) {  // nothing of this call may still run when it returns
                cudaStreamSynchronize(cs);
                cudaStreamSynchronize(s);
                cudaGetLastError();
                return finish(st);
            }
            e = cudaMemsetAsync(ctl, 0, G.ctl.bytes, s);
            if (e == cudaSuccess)
                e = launch_upsweep(G, desc, cur_k, m, reinterpret_cast<unsigned long long*>(ctl + G.ctl.gp_off),
                                   ctl + G.ctl.bytes, G.status_bytes, s);
            int left = __builtin_popcount(digits);
            bool first = true;
            for (int q = 0; q < G.passes && e == cudaSuccess; ++q) {
                if (!((digits >> q) & 1u)) continue;
                e = launch_pass(G, q, desc, cur_k, cur_v, oth_k, oth_v, first, left == 1, ctl, err, s);
                std::swap(cur_k, oth_k);
                std::swap(cur_v, oth_v);
                first = false;
                --left;
            }
            if (e != cudaSuccess) return fail("host sort group", e);
        }
        cudaEvent_t done;
        if ((e = event(&done)) != cudaSuccess) return fail("host sort event", e);
        if ((e = cudaEventRecord(done, s)) != cudaSuccess) return fail("host sort event", e);
        outs.push_back(Out{cur_k, cur_v, g.begin, m, done});
        mark("group " + std::to_string(outs.size() - 1) + " sorted (" + std::to_string(m) + ")", s);
    }
    if (trace) host_log += " groups=" + std::to_string(outs.size()) + " sorts_queued_ms=" + std::to_string(host_ms());
    // every group's work is queued before the first copy back: a copy into
    // pageable memory blocks the host, and the GPU must not wait for it
    for (const Out& o : outs) {
        e = cudaStreamWaitEvent(cs, o.done, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(h_keys + o.begin * kb, o.k, o.count * kb, cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess && vb)
            e = cudaMemcpyAsync(h_vals + o.begin * vb, o.v, o.count * vb, cudaMemcpyDeviceToHost, cs);
        if (e != cudaSuccess) return fail("host sort copy out", e);
        mark("group " + std::to_string(&o - outs.data()) + " home", cs);
    }
    if (trace) host_log += " copies_queued_ms=" + std::to_string(host_ms());
    uint32_t w = 0;
    e = cudaStreamSynchronize(cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&w, err, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail("host sort finish", e);
    return finish(status_from_error_word(w));
}

// ---- batched sort from host memory ----------------------------------------
// Consecutive segments form groups of ~2^24 keys (2 to 16;
// GBSORT_HOST_SPLIT_GROUPS overrides; a segment is never split).  Group g+1's keys come in on one copy
// stream while group g sorts (one batched run per group, on the caller's
// stream) and group g-1 goes back on the other copy stream, so both
// directions of the host link work at once.

struct SegGroup {
    size_t first = 0, end = 0;  // segments [first, end)
    gbsort_segmented_plan* plan = nullptr;
    size_t ws_bytes = 0, image_bytes = 0, image_off = 0;
};

struct SegHostJob {
    std::vector<SegGroup> groups;
    size_t ws_max = 0, image_total = 0;
    // d_buffer: [keys][values][error words][every group's tables][workspace]
    size_t stage_keys = 0, stage_vals = 0, errs = 0, tables = 0, ws = 0, total = 0;
    ~SegHostJob() {
        for (SegGroup& g : groups)
            if (g.plan) gbsort_segmented_plan_destroy(g.plan);
    }
};

int seg_host_job(int key_type, size_t vb, int desc, const uint64_t* off, size_t num, SegHostJob* job) {
    const size_t kb = gbsort_key_bytes(key_type);
    if (kb == 0 || (num > 0 && off == nullptr)) return GBSORT_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < num; ++i)
        if (off[i + 1] < off[i]) return GBSORT_ERR_INVALID_ARGUMENT;
    const uint64_t n = num ? off[num] - off[0] : 0;
    const int G = split_groups(n);
    const uint64_t target = std::max<uint64_t>(1, (n + uint64_t(G) - 1) / uint64_t(G));
    size_t first = 0;
    for (size_t i = 0; i < num; ++i) {
        if (off[i + 1] - off[first] >= target || i + 1 == num) {
            SegGroup g;
            g.first = first;
            g.end = i + 1;
            job->groups.push_back(g);
            first = i + 1;
        }
    }
    std::vector<uint64_t> rel;
    for (SegGroup& g : job->groups) {
        rel.assign(off + g.first, off + g.end + 1);
        for (uint64_t& x : rel) x -= off[g.first];
        int st = gbsort_segmented_plan_create(key_type, vb, desc, rel.data(), g.end - g.first, &g.plan);
        if (st != GBSORT_OK) return st;
        gbsort_segmented_info info{};
        st = gbsort_segmented_plan_info(g.plan, &info);
        if (st != GBSORT_OK) return st;
        g.ws_bytes = size_t(info.workspace_bytes);
        g.image_bytes = segmented_table_bytes(g.plan);
        g.image_off = job->image_total;
        job->image_total += align_up(g.image_bytes, 256);
        job->ws_max = std::max(job->ws_max, g.ws_bytes);
    }
    job->stage_keys = 0;
    job->stage_vals = align_up(size_t(n) * kb, 256);
    job->errs = job->stage_vals + align_up(size_t(n) * vb, 256);
    job->tables = job->errs + align_up(std::max<size_t>(1, job->groups.size()) * 4, 256);
    job->ws = job->tables + align_up(job->image_total, 256);
    job->total = job->ws + align_up(job->ws_max, 256);
    return GBSORT_OK;
}

// Pinned host memory for the groups' table images, kept between calls.
struct PinnedImages {
    std::mutex mu;
    uint8_t* buf = nullptr;
    size_t cap = 0;
};
PinnedImages& pinned_images() {
    static PinnedImages p;
    return p;
}

int sort_segmented_host(int key_type, int desc, uint8_t* h_keys, uint8_t* h_vals, size_t vb, const uint64_t* off,
                        SegHostJob& job, uint8_t* base, cudaStream_t s) {
    const size_t kb = gbsort_key_bytes(key_type);
    const uint64_t off0 = off[0];
    uint8_t* stage_k = base + job.stage_keys;
    uint8_t* stage_v = vb ? base + job.stage_vals : nullptr;
    uint8_t* ws = base + job.ws;
    uint8_t* tables = base + job.tables;
    uint32_t* errs = reinterpret_cast<uint32_t*>(base + job.errs);
    cudaStream_t cin = copy_stream(0), cout = copy_stream(1);
    if (cin == nullptr || cout == nullptr) {
        set_last_error_text("batched host sort: no copy stream");
        return GBSORT_ERR_CUDA;
    }
    PinnedImages& pi = pinned_images();
    std::lock_guard<std::mutex> lk(pi.mu);  // the images stay in use until this call returns
    if (job.image_total > pi.cap) {
        if (pi.buf) cudaFreeHost(pi.buf);
        pi.buf = nullptr;
        pi.cap = 0;
        const cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&pi.buf), job.image_total, cudaHostAllocDefault);
        if (e != cudaSuccess) {
            pi.buf = nullptr;
            set_last_error("batched host sort: table images", e);
            return GBSORT_ERR_CUDA;
        }
        pi.cap = job.image_total;
    }
    for (const SegGroup& g : job.groups)
        if (g.image_bytes) segmented_table_image(g.plan, pi.buf + g.image_off);

    std::vector<cudaEvent_t> evs;
    auto event = [&](cudaEvent_t* ev) {
        const cudaError_t e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        if (e == cudaSuccess) evs.push_back(*ev);
        return e;
    };
    // GBSORT_HOST_TRACE=1: device times of the phases, printed on stderr
    const bool trace = env_u64("GBSORT_HOST_TRACE", 0) == 1;
    std::vector<std::pair<std::string, cudaEvent_t>> marks;
    auto mark = [&](const std::string& label, cudaStream_t st) {
        if (!trace) return;
        cudaEvent_t ev;
        if (cudaEventCreate(&ev) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        evs.push_back(ev);
        cudaEventRecord(ev, st);
        marks.emplace_back(label, ev);
    };
    auto finish = [&](int status) {
        if (trace && !marks.empty()) {
            std::fprintf(stderr, "gbsort-host batched groups=%zu\n", job.groups.size());
            for (const auto& m : marks) {
                float t = 0.f;
                if (cudaEventElapsedTime(&t, marks[0].second, m.second) != cudaSuccess) cudaGetLastError();
                std::fprintf(stderr, "  %-28s %9.3f ms\n", m.first.c_str(), double(t));
            }
        }
        for (cudaEvent_t ev : evs) cudaEventDestroy(ev);
        return status;
    };
    auto fail = [&](const char* what, cudaError_t e, int status) {
        if (e != cudaSuccess) set_last_error(what, e);
        // nothing of this call may still run when it returns
        cudaStreamSynchronize(cin);
        cudaStreamSynchronize(s);
        cudaStreamSynchronize(cout);
        cudaGetLastError();
        return finish(status);
    };
    const size_t G = job.groups.size();
    cudaError_t e = cudaMemsetAsync(errs, 0, G * 4, s);
    cudaEvent_t ev_start;
    if (e == cudaSuccess) e = event(&ev_start);
    if (e == cudaSuccess) e = cudaEventRecord(ev_start, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(cin, ev_start, 0);
    if (e != cudaSuccess) return fail("batched host sort", e, GBSORT_ERR_CUDA);
    mark("start", s);
    // every group's tables first (one small copy), then every group's keys:
    // a group's tables then reach its workspace by a kernel, which cannot
    // queue behind the bulk copies on the copy engine
    cudaEvent_t tables_in;
    if ((e = event(&tables_in)) != cudaSuccess) return fail("batched host sort event", e, GBSORT_ERR_CUDA);
    if (job.image_total) e = cudaMemcpyAsync(tables, pi.buf, job.image_total, cudaMemcpyHostToDevice, cin);
    if (e == cudaSuccess) e = cudaEventRecord(tables_in, cin);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, tables_in, 0);
    if (e != cudaSuccess) return fail("batched host sort tables", e, GBSORT_ERR_CUDA);
    std::vector<cudaEvent_t> in(G), done(G);
    for (size_t i = 0; i < G; ++i) {
        const SegGroup& g = job.groups[i];
        const uint64_t at = off[g.first] - off0, m = off[g.end] - off[g.first];
        if ((e = event(&in[i])) != cudaSuccess) return fail("batched host sort event", e, GBSORT_ERR_CUDA);
        if (m) e = cudaMemcpyAsync(stage_k + at * kb, h_keys + (off0 + at) * kb, m * kb, cudaMemcpyHostToDevice, cin);
        if (e == cudaSuccess && m && vb)
            e = cudaMemcpyAsync(stage_v + at * vb, h_vals + (off0 + at) * vb, m * vb, cudaMemcpyHostToDevice, cin);
        if (e == cudaSuccess) e = cudaEventRecord(in[i], cin);
        if (e != cudaSuccess) return fail("batched host sort copy in", e, GBSORT_ERR_CUDA);
        mark("group " + std::to_string(i) + " in", cin);
    }
    for (size_t i = 0; i < G; ++i) {
        const SegGroup& g = job.groups[i];
        const uint64_t at = off[g.first] - off0;
        if ((e = cudaStreamWaitEvent(s, in[i], 0)) != cudaSuccess)
            return fail("batched host sort", e, GBSORT_ERR_CUDA);
        int st = segmented_bind_image(g.plan, stage_k + at * kb, stage_v ? stage_v + at * vb : nullptr, ws,
                                      job.ws_max, s, tables + g.image_off, true);
        if (st == GBSORT_OK) st = gbsort_segmented_run(g.plan, 0, s);
        if (st != GBSORT_OK) return fail("batched host sort", cudaSuccess, st);
        e = cudaMemcpyAsync(errs + i, segmented_error_word(g.plan), 4, cudaMemcpyDeviceToDevice, s);
        if (e == cudaSuccess) e = event(&done[i]);
        if (e == cudaSuccess) e = cudaEventRecord(done[i], s);
        if (e != cudaSuccess) return fail("batched host sort", e, GBSORT_ERR_CUDA);
        mark("group " + std::to_string(i) + " sorted", s);
    }
    // copies back last: one into pageable memory blocks the host, and every
    // sort must already be queued by then
    for (size_t i = 0; i < G; ++i) {
        const SegGroup& g = job.groups[i];
        const uint64_t at = off[g.first] - off0, m = off[g.end] - off[g.first];
        e = cudaStreamWaitEvent(cout, done[i], 0);
        if (e == cudaSuccess && m)
            e = cudaMemcpyAsync(h_keys + (off0 + at) * kb, stage_k + at * kb, m * kb, cudaMemcpyDeviceToHost, cout);
        if (e == cudaSuccess && m && vb)
            e = cudaMemcpyAsync(h_vals + (off0 + at) * vb, stage_v + at * vb, m * vb, cudaMemcpyDeviceToHost, cout);
        if (e != cudaSuccess) return fail("batched host sort copy out", e, GBSORT_ERR_CUDA);
        mark("group " + std::to_string(i) + " home", cout);
    }
    std::vector<uint32_t> w(G, 0);
    e = cudaStreamSynchronize(cout);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.data(), errs, G * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail("batched host sort finish", e, GBSORT_ERR_CUDA);
    uint32_t all = 0;
    for (uint32_t x : w) all |= x;
    return finish(status_from_error_word(all));
}

}  // namespace
}  // namespace gbsort

using namespace gbsort;

extern "C" {

size_t gbsort_host_buffer_bytes(int key_type, size_t value_bytes, size_t n) {
    Plan plan;
    if (make_plan(key_type, value_bytes, n, &plan) != GBSORT_OK) return 0;
    size_t bytes = plain_bytes(plan, value_bytes);
    SplitLayout L;
    if (plan.passes >= 2 && split_layout(key_type, value_bytes, n, &L) == GBSORT_OK) bytes = std::max(bytes, L.total);
    return bytes;
}

int gbsort_sort_host(int key_type, int descending, void* h_keys, void* h_values, size_t value_bytes, size_t n,
                     void* d_buffer, size_t buffer_bytes, void* stream) {
    Plan plan;
    int st = make_plan(key_type, value_bytes, n, &plan);
    if (st != GBSORT_OK) return st;
    if (n == 0) return GBSORT_OK;
    if (h_keys == nullptr || d_buffer == nullptr || (value_bytes && h_values == nullptr))
        return GBSORT_ERR_INVALID_ARGUMENT;
    if (buffer_bytes < gbsort_host_buffer_bytes(key_type, value_bytes, n)) return GBSORT_ERR_WORKSPACE_TOO_SMALL;
    if (reinterpret_cast<uintptr_t>(d_buffer) % 16) {  // holds a workspace: 16-byte stores clear its status array
        set_last_error_text("the device buffer must be 16-byte aligned");
        return GBSORT_ERR_INVALID_ARGUMENT;
    }
    if (!device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint8_t* base = static_cast<uint8_t*>(d_buffer);
    // the split path overlaps the copies with per-group digit passes; a
    // keys-only sort that goes most significant digit first on the device
    // is short enough that copy, sort, copy wins (2^26 u128: the device sort
    // takes 2 ms of the ~12 the copies take)
    if (plan.passes >= 2 && n >= split_min_keys() && !plan.msd) {
        SplitLayout L;
        st = split_layout(key_type, value_bytes, n, &L);
        if (st != GBSORT_OK) return st;
        return sort_host_split(plan, key_type, descending ? 1 : 0, static_cast<uint8_t*>(h_keys),
                               static_cast<uint8_t*>(h_values), value_bytes, base, L, s);
    }
    const size_t kbytes = n * size_t(plan.kb), vbytes = n * value_bytes;
    uint8_t* d_keys = base;
    uint8_t* d_vals = base + align_up(kbytes, 256);
    uint8_t* d_ws = base + align_up(align_up(kbytes, 256) + vbytes, 256);
    cudaError_t e = cudaMemcpyAsync(d_keys, h_keys, kbytes, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && vbytes) e = cudaMemcpyAsync(d_vals, h_values, vbytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        set_last_error("host to device copy", e);
        return GBSORT_ERR_CUDA;
    }
    st = enqueue_sort(plan, descending ? 1 : 0, d_keys, value_bytes ? d_vals : nullptr, d_ws, s, nullptr, 0,
                      nullptr);
    if (st != GBSORT_OK) return st;
    e = cudaMemcpyAsync(h_keys, d_keys, kbytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && vbytes) e = cudaMemcpyAsync(h_values, d_vals, vbytes, cudaMemcpyDeviceToHost, s);
    uint32_t err = 0;
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&err, d_ws + plan.ctl_off + plan.ctl.err_off, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_last_error("device to host copy", e);
        return GBSORT_ERR_CUDA;
    }
    return status_from_error_word(err);
}

size_t gbsort_segmented_host_buffer_bytes(int key_type, size_t value_bytes, const uint64_t* h_offsets,
                                          size_t num_segments) {
    SegHostJob job;
    if (seg_host_job(key_type, value_bytes, 0, h_offsets, num_segments, &job) != GBSORT_OK) return 0;
    return job.total;
}

int gbsort_segmented_sort_host(int key_type, int descending, void* h_keys, void* h_values, size_t value_bytes,
                               const uint64_t* h_offsets, size_t num_segments, void* d_buffer, size_t buffer_bytes,
                               void* stream) {
    SegHostJob job;
    int st = seg_host_job(key_type, value_bytes, descending ? 1 : 0, h_offsets, num_segments, &job);
    if (st != GBSORT_OK) return st;
    if (num_segments == 0 || h_offsets[num_segments] == h_offsets[0]) return GBSORT_OK;
    if (h_keys == nullptr || d_buffer == nullptr || (value_bytes && h_values == nullptr))
        return GBSORT_ERR_INVALID_ARGUMENT;
    if (buffer_bytes < job.total) return GBSORT_ERR_WORKSPACE_TOO_SMALL;
    if (reinterpret_cast<uintptr_t>(d_buffer) % 16) {  // holds a workspace: 16-byte stores clear its status array
        set_last_error_text("the device buffer must be 16-byte aligned");
        return GBSORT_ERR_INVALID_ARGUMENT;
    }
    if (!device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    return sort_segmented_host(key_type, descending ? 1 : 0, static_cast<uint8_t*>(h_keys),
                               static_cast<uint8_t*>(h_values), value_bytes, h_offsets, job,
                               static_cast<uint8_t*>(d_buffer), static_cast<cudaStream_t>(stream));
}

}  // extern "C"
