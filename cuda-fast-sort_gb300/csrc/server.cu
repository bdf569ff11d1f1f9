// server.cu — continuous-batching sort server.  No counterpart in the
// reference: rsort sorts one array per call and blocks on it
// (include/rsort/detail/radix_kernel.cuh:583-601).
//
// Threads.  Callers submit from any thread.  One scheduler thread forms and
// launches batches.  Completion is signalled by a host function enqueued on
// the batch's stream after its last copy; it only stamps the time and hands
// the batch back to the scheduler (no CUDA call runs in it).
//
// Batching.  Requests of one class (key type, value size, order) that are
// queued when a stream slot frees up are coalesced, in arrival order, into
// one batched segmented sort: each request is one segment of a contiguous
// staging area.  The class of the oldest queued request goes first.  When
// the GPU keeps up, batches are small and latency is one sort; when it falls
// behind, the queue grows and the next batch takes all of it (up to
// max_batch_keys / max_batch_requests), which is what keeps throughput up.
//
// Memory.  One device allocation of pool_bytes is cut into per-batch blocks
// (first fit over a coalescing free list).  A block holds the staging area
// (every request's keys back to back, then their values) followed by the
// batched sort's workspace.  A batch is admitted only when its block fits;
// otherwise it is trimmed to the leading requests that fit, and if not even
// the first fits it waits for a running batch to return its block.  A
// request that could not fit in the empty pool is rejected at submit.
// A lone device-memory request sorted in place (keys_out == keys_in) skips
// the staging copies and is sorted where it lies.

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gbsort.h"
#include "plan.h"
#include "device_common.cuh"
#include "segmented_internal.h"

namespace {

using gbsort::align_up;

uint64_t now_ns() {
    return uint64_t(std::chrono::duration_cast<std::chrono::nanoseconds>(
                        std::chrono::steady_clock::now().time_since_epoch())
                        .count());
}

constexpr size_t POOL_ALIGN = 256;

// First-fit allocator over [0, cap) with coalescing on free.
class Arena {
   public:
    explicit Arena(size_t cap) : cap_(cap) { free_[0] = cap; }
    // offset of a block of `bytes`, or SIZE_MAX
    size_t alloc(size_t bytes) {
        bytes = align_up(std::max<size_t>(bytes, 1), POOL_ALIGN);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const size_t off = it->first, left = it->second - bytes;
            free_.erase(it);
            if (left) free_[off + bytes] = left;
            used_ += bytes;
            peak_ = std::max(peak_, used_);
            return off;
        }
        return SIZE_MAX;
    }
    void release(size_t off, size_t bytes) {
        bytes = align_up(std::max<size_t>(bytes, 1), POOL_ALIGN);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t largest_free() const {
        size_t m = 0;
        for (const auto& f : free_) m = std::max(m, f.second);
        return m;
    }
    size_t peak() const { return peak_; }
    void reset_peak() { peak_ = used_; }

   private:
    size_t cap_;
    size_t used_ = 0, peak_ = 0;
    std::map<size_t, size_t> free_;  // offset -> bytes
};

struct Request {
    uint64_t ticket = 0;
    gbsort_request r{};
    size_t kb = 0;
    uint64_t cls = 0;
    uint64_t t_submit = 0, t_launch = 0, t_done = 0;
    int status = GBSORT_ERR_NOT_READY;
};

struct Batch {
    int slot = -1;
    std::vector<Request*> reqs;
    gbsort_segmented_plan* plan = nullptr;
    size_t block_off = 0, block_bytes = 0;
    uint64_t keys = 0, bytes = 0;
    uint64_t t_done = 0;
    int launch_status = GBSORT_OK;
    struct gbsort_server* server = nullptr;
};

uint64_t class_of(const gbsort_request& r) {
    return (uint64_t(r.key_type) << 40) | (uint64_t(r.value_bytes) << 8) | uint64_t(r.descending ? 1 : 0);
}

bool is_device_ptr(const void* p) {
    if (p == nullptr) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

int status_of_error_word(uint32_t w) {
    if (w & gbsort::ERRBIT_BOUNDS) return GBSORT_ERR_INTERNAL;
    if (w & gbsort::ERRBIT_TIMEOUT) return GBSORT_ERR_TIMEOUT;
    return GBSORT_OK;
}

double percentile_us(std::vector<uint64_t>& v, double q) {
    if (v.empty()) return 0.0;
    const size_t k = std::min(v.size() - 1, size_t(q * double(v.size() - 1) + 0.5));
    std::nth_element(v.begin(), v.begin() + k, v.end());
    return double(v[k]) / 1000.0;
}

}  // namespace

struct gbsort_server {
    gbsort_server_config cfg{};
    int device = 0;
    uint8_t* pool = nullptr;
    std::unique_ptr<Arena> arena;
    std::vector<cudaStream_t> streams;
    std::vector<bool> slot_busy;
    uint32_t* err_words = nullptr;  // pinned, one per slot
    std::vector<uint8_t*> images;   // pinned table images, one per slot
    std::vector<cudaEvent_t> marks; // per slot: start, inputs in, lane free, sorted, outputs out
    std::vector<cudaEvent_t> sorted;  // per slot: this slot's last sort finished
    int last_sort_slot = -1;          // scheduler thread only
    bool trace = false;             // GBSORT_SERVER_TRACE=1: one line per batch on stderr
    uint64_t t_origin = 0;
    std::vector<size_t> image_cap;

    std::mutex mu;
    std::condition_variable cv;       // wakes the scheduler
    std::condition_variable done_cv;  // wakes waiters
    std::deque<Request*> queue;
    std::vector<Batch*> completed;    // handed back by the host functions
    std::unordered_map<uint64_t, Request*> tickets;
    uint64_t next_ticket = 1;
    size_t in_flight = 0;
    size_t outstanding = 0;  // accepted requests not yet finished (queued, being formed or running)
    bool paused = false, stopping = false;
    std::thread worker;

    // stats
    uint64_t submitted = 0, completed_n = 0, failed = 0, rejected = 0, batches = 0, max_batch = 0;
    uint64_t keys_sorted = 0, bytes_sorted = 0, batch_requests_sum = 0;
    uint64_t first_submit = 0, last_done = 0;
    std::vector<uint64_t> latencies, queue_waits;
    uint64_t kernel_launches = 0;
    uint64_t plan_ns = 0, launch_ns = 0, batch_ns = 0;  // scheduler host time; batch launch -> done
    double h2d_ms = 0.0, sort_ms = 0.0, d2h_ms = 0.0;   // device time of the batches' stages
    uint64_t launches_of_last_measure = 0;  // scheduler thread only

    // ---- sizing -------------------------------------------------------
    // Bytes of the block a batch of `reqs` needs (staging + workspace), with
    // the plan it was measured on.  staged: false only for a lone in-place
    // device request.
    int measure(const std::vector<Request*>& reqs, bool staged, gbsort_segmented_plan** plan, size_t* bytes) {
        std::vector<uint64_t> off(reqs.size() + 1, 0);
        for (size_t i = 0; i < reqs.size(); ++i) off[i + 1] = off[i] + reqs[i]->r.n;
        const gbsort_request& r0 = reqs[0]->r;
        int st = gbsort_segmented_plan_create(r0.key_type, r0.value_bytes, r0.descending, off.data(), reqs.size(),
                                              plan);
        if (st != GBSORT_OK) return st;
        gbsort_segmented_info info{};
        gbsort_segmented_plan_info(*plan, &info);
        launches_of_last_measure = info.kernel_launches;
        const uint64_t n = off.back();
        size_t b = info.workspace_bytes;
        if (staged) b += align_up(n * reqs[0]->kb, POOL_ALIGN) + align_up(n * r0.value_bytes, POOL_ALIGN);
        *bytes = align_up(std::max<size_t>(b, 1), POOL_ALIGN);
        return GBSORT_OK;
    }

    static bool in_place_device(const Request* q) {
        const gbsort_request& r = q->r;
        if (r.keys_out != r.keys_in || (r.value_bytes && r.values_out != r.values_in)) return false;
        if (!is_device_ptr(r.keys_in) || (r.value_bytes && !is_device_ptr(r.values_in))) return false;
        return reinterpret_cast<uintptr_t>(r.keys_in) % q->kb == 0 &&
               (r.value_bytes == 0 || reinterpret_cast<uintptr_t>(r.values_in) % r.value_bytes == 0);
    }

    // ---- completion (host function: no CUDA calls) ----------------------
    static void CUDART_CB on_batch_done(void* arg) {
        Batch* b = static_cast<Batch*>(arg);
        b->t_done = now_ns();
        gbsort_server* s = b->server;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->completed.push_back(b);
        }
        s->cv.notify_all();
    }

    // Called by the scheduler with mu held.
    void retire(Batch* b) {
        const uint32_t w = err_words[b->slot];
        if (b->launch_status == GBSORT_OK) {
            float t[4] = {0.f, 0.f, 0.f, 0.f};  // inputs, lane wait, sort, outputs
            cudaEvent_t* m = &marks[size_t(b->slot) * 5];
            for (int i = 0; i < 4; ++i)
                if (cudaEventElapsedTime(&t[i], m[i], m[i + 1]) != cudaSuccess) cudaGetLastError();
            h2d_ms += t[0];
            sort_ms += t[2];
            d2h_ms += t[3];
            if (trace)
                std::fprintf(stderr,
                             "gbsort-server batch slot=%d requests=%zu keys=%llu launch_ms=%.3f done_ms=%.3f "
                             "h2d_ms=%.3f lane_wait_ms=%.3f sort_ms=%.3f d2h_ms=%.3f\n",
                             b->slot, b->reqs.size(), (unsigned long long)b->keys,
                             double(b->reqs[0]->t_launch - t_origin) * 1e-6, double(b->t_done - t_origin) * 1e-6,
                             t[0], t[1], t[2], t[3]);
        }
        const int st = b->launch_status != GBSORT_OK ? b->launch_status : status_of_error_word(w);
        for (Request* q : b->reqs) {
            q->status = st;
            q->t_done = b->t_done;
            if (st == GBSORT_OK) {
                ++completed_n;
                keys_sorted += q->r.n;
                bytes_sorted += q->r.n * (q->kb + q->r.value_bytes);
            } else {
                ++failed;
            }
            latencies.push_back(q->t_done - q->t_submit);
            queue_waits.push_back(q->t_launch - q->t_submit);
            --outstanding;
        }
        last_done = std::max(last_done, b->t_done);
        if (!b->reqs.empty()) batch_ns += b->t_done - b->reqs[0]->t_launch;
        arena->release(b->block_off, b->block_bytes);
        slot_busy[b->slot] = false;
        --in_flight;
    }

    // ---- launch (scheduler thread, mu NOT held) -------------------------
    int launch(Batch* b) {
        cudaStream_t s = streams[b->slot];
        const gbsort_request& r0 = b->reqs[0]->r;
        const size_t kb = b->reqs[0]->kb, vb = r0.value_bytes;
        uint8_t* block = pool + b->block_off;
        const bool staged = !(b->reqs.size() == 1 && in_place_device(b->reqs[0]));
        uint8_t* d_keys = staged ? block : static_cast<uint8_t*>(const_cast<void*>(r0.keys_in));
        uint8_t* d_vals = nullptr;
        size_t stage_bytes = 0;
        if (staged) {
            d_vals = vb ? block + align_up(b->keys * kb, POOL_ALIGN) : nullptr;
            stage_bytes = align_up(b->keys * kb, POOL_ALIGN) + align_up(b->keys * vb, POOL_ALIGN);
        } else if (vb) {
            d_vals = static_cast<uint8_t*>(const_cast<void*>(r0.values_in));
        }
        uint8_t* ws = block + stage_bytes;
        const size_t ws_bytes = b->block_bytes - stage_bytes;
        // the batch's tables go up from this slot's pinned image (the slot's
        // previous batch, the last reader of the image, has finished)
        const size_t tb = gbsort::segmented_table_bytes(b->plan);
        cudaError_t e = cudaSuccess;
        if (tb > image_cap[b->slot]) {
            if (images[b->slot]) cudaFreeHost(images[b->slot]);
            images[b->slot] = nullptr;
            image_cap[b->slot] = 0;
            const size_t cap = std::max<size_t>(tb, size_t(1) << 20);
            e = cudaHostAlloc(reinterpret_cast<void**>(&images[b->slot]), cap, cudaHostAllocDefault);
            if (e != cudaSuccess) {
                gbsort::set_last_error("server table image", e);
                images[b->slot] = nullptr;
                return GBSORT_ERR_CUDA;
            }
            image_cap[b->slot] = cap;
        }
        if (tb) gbsort::segmented_table_image(b->plan, images[b->slot]);
        cudaEvent_t* m = &marks[size_t(b->slot) * 5];
        cudaEventRecord(m[0], s);
        int st = gbsort::segmented_bind_image(b->plan, d_keys, d_vals, ws, ws_bytes, s, images[b->slot]);
        if (st != GBSORT_OK) return st;
        if (staged) {
            size_t at = 0;
            for (Request* q : b->reqs) {
                const size_t n = q->r.n;
                if (n && e == cudaSuccess)
                    e = cudaMemcpyAsync(d_keys + at * kb, q->r.keys_in, n * kb, cudaMemcpyDefault, s);
                if (n && vb && e == cudaSuccess)
                    e = cudaMemcpyAsync(d_vals + at * vb, q->r.values_in, n * vb, cudaMemcpyDefault, s);
                at += n;
            }
        }
        if (e != cudaSuccess) {
            gbsort::set_last_error("server input copy", e);
            return GBSORT_ERR_CUDA;
        }
        // Sorts run one at a time, in launch order ("sort lane"): two onesweep
        // launches sharing the SMs slow each other down far more than they
        // overlap, while copies of other batches overlap a sort for free.
        cudaEventRecord(m[1], s);
        if (last_sort_slot >= 0 && last_sort_slot != b->slot)
            cudaStreamWaitEvent(s, sorted[size_t(last_sort_slot)], 0);
        cudaEventRecord(m[2], s);
        st = gbsort_segmented_run(b->plan, 0, s);
        if (st != GBSORT_OK) return st;
        cudaEventRecord(m[3], s);
        cudaEventRecord(sorted[size_t(b->slot)], s);
        last_sort_slot = b->slot;
        if (staged) {
            size_t at = 0;
            for (Request* q : b->reqs) {
                const size_t n = q->r.n;
                if (n && e == cudaSuccess)
                    e = cudaMemcpyAsync(q->r.keys_out, d_keys + at * kb, n * kb, cudaMemcpyDefault, s);
                if (n && vb && e == cudaSuccess)
                    e = cudaMemcpyAsync(q->r.values_out, d_vals + at * vb, n * vb, cudaMemcpyDefault, s);
                at += n;
            }
        }
        if (e == cudaSuccess) e = cudaEventRecord(m[4], s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&err_words[b->slot], gbsort::segmented_error_word(b->plan), 4,
                                cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaLaunchHostFunc(s, on_batch_done, b);
        if (e != cudaSuccess) {
            gbsort::set_last_error("server launch", e);
            return GBSORT_ERR_CUDA;
        }
        return GBSORT_OK;
    }

    // Takes, with mu held, the requests of the next batch off the queue (the
    // oldest request's class, in arrival order, within the caps).
    std::vector<Request*> take_candidates() {
        std::vector<Request*> out;
        if (queue.empty()) return out;
        const uint64_t cls = queue.front()->cls;
        uint64_t keys = 0;
        for (auto it = queue.begin(); it != queue.end();) {
            Request* q = *it;
            if (q->cls != cls) {
                ++it;
                continue;
            }
            if (!out.empty() && (keys + q->r.n > cfg.max_batch_keys || out.size() >= cfg.max_batch_requests)) break;
            out.push_back(q);
            keys += q->r.n;
            it = queue.erase(it);
        }
        return out;
    }

    void run() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            if (!completed.empty()) {
                std::vector<Batch*> done;
                done.swap(completed);  // host functions may append meanwhile
                lk.unlock();
                for (Batch* b : done) gbsort_segmented_plan_destroy(b->plan);
                lk.lock();
                for (Batch* b : done) {
                    retire(b);
                    delete b;
                }
                done_cv.notify_all();
            }
            int slot = -1;
            for (size_t i = 0; i < slot_busy.size(); ++i)
                if (!slot_busy[i]) {
                    slot = int(i);
                    break;
                }
            if (stopping && outstanding == 0) break;
            if (paused || queue.empty() || slot < 0) {
                if (completed.empty()) cv.wait(lk);
                continue;
            }
            std::vector<Request*> cand = take_candidates();
            // Fit the batch into the pool: measure, and trim from the back
            // until its block fits the largest free range.
            const size_t avail = arena->largest_free();
            lk.unlock();
            gbsort_segmented_plan* plan = nullptr;
            size_t bytes = 0;
            int st = GBSORT_OK;
            size_t keep = cand.size();
            const uint64_t t_plan0 = now_ns();
            for (;;) {
                std::vector<Request*> part(cand.begin(), cand.begin() + keep);
                const bool staged = !(part.size() == 1 && in_place_device(part[0]));
                st = measure(part, staged, &plan, &bytes);
                if (st != GBSORT_OK || bytes <= avail || keep == 1) break;
                gbsort_segmented_plan_destroy(plan);
                plan = nullptr;
                // shrink roughly in proportion, at least by one
                keep = std::max<size_t>(1, std::min(keep - 1, size_t(double(keep) * double(avail) / double(bytes))));
            }
            lk.lock();
            plan_ns += now_ns() - t_plan0;
            if (st == GBSORT_OK && bytes > avail) {
                // not even the first request fits now: put everything back
                // and wait for a running batch to return its block
                gbsort_segmented_plan_destroy(plan);
                queue.insert(queue.begin(), cand.begin(), cand.end());
                if (in_flight == 0) {  // cannot happen: submit checked the empty pool
                    Request* q = queue.front();
                    queue.pop_front();
                    q->status = GBSORT_ERR_BUDGET;
                    q->t_launch = q->t_done = now_ns();
                    ++failed;
                    --outstanding;
                    done_cv.notify_all();
                    continue;
                }
                if (completed.empty()) cv.wait(lk);
                continue;
            }
            // the tail that did not fit goes back to the front, in order
            queue.insert(queue.begin(), cand.begin() + keep, cand.end());
            cand.resize(keep);
            Batch* b = new Batch();
            b->server = this;
            b->slot = slot;
            b->reqs = cand;
            b->plan = plan;
            b->block_bytes = bytes;
            const uint64_t t = now_ns();
            for (Request* q : cand) {
                q->t_launch = t;
                b->keys += q->r.n;
            }
            if (st == GBSORT_OK) {
                b->block_off = arena->alloc(bytes);
                slot_busy[slot] = true;
                ++in_flight;
                ++batches;
                kernel_launches += launches_of_last_measure;
                batch_requests_sum += cand.size();
                max_batch = std::max<uint64_t>(max_batch, cand.size());
                lk.unlock();
                const uint64_t t_l0 = now_ns();
                st = launch(b);
                const uint64_t t_l1 = now_ns();
                if (st != GBSORT_OK) {
                    // nothing of this batch may still run when its block is reused
                    cudaStreamSynchronize(streams[slot]);
                    cudaGetLastError();
                    b->launch_status = st;
                    b->t_done = now_ns();
                    lk.lock();
                    completed.push_back(b);
                } else {
                    lk.lock();
                }
                launch_ns += t_l1 - t_l0;
            } else {
                // the plan itself was refused (invalid request mix)
                for (Request* q : cand) {
                    q->status = st;
                    q->t_done = now_ns();
                    ++failed;
                    --outstanding;
                }
                delete b;
                done_cv.notify_all();
            }
        }
    }
};

extern "C" {

int gbsort_server_create(const gbsort_server_config* cfg, gbsort_server** out) {
    if (out == nullptr) return GBSORT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!gbsort::device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    auto s = std::make_unique<gbsort_server>();
    if (cfg) s->cfg = *cfg;
    if (s->cfg.pool_bytes == 0) s->cfg.pool_bytes = uint64_t(64) << 30;
    if (s->cfg.streams == 0) s->cfg.streams = 6;
    if (s->cfg.streams > 16) return GBSORT_ERR_INVALID_ARGUMENT;
    if (s->cfg.max_batch_keys == 0) s->cfg.max_batch_keys = uint64_t(1) << 26;
    if (s->cfg.max_batch_requests == 0) s->cfg.max_batch_requests = 4096;
    s->cfg.pool_bytes = align_up(s->cfg.pool_bytes, POOL_ALIGN);
    s->paused = s->cfg.paused != 0;
    cudaGetDevice(&s->device);
    cudaError_t e = cudaMalloc(&s->pool, s->cfg.pool_bytes);
    if (e == cudaSuccess) e = cudaHostAlloc(&s->err_words, 16 * sizeof(uint32_t), cudaHostAllocDefault);
    for (uint32_t i = 0; e == cudaSuccess && i < s->cfg.streams; ++i) {
        cudaStream_t st = nullptr;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e == cudaSuccess) s->streams.push_back(st);
    }
    if (e != cudaSuccess) {
        gbsort::set_last_error("server create", e);
        for (cudaStream_t st : s->streams) cudaStreamDestroy(st);
        if (s->err_words) cudaFreeHost(s->err_words);
        if (s->pool) cudaFree(s->pool);
        return GBSORT_ERR_CUDA;
    }
    std::memset(s->err_words, 0, 16 * sizeof(uint32_t));
    s->arena = std::make_unique<Arena>(s->cfg.pool_bytes);
    s->images.assign(s->cfg.streams, nullptr);
    s->marks.assign(size_t(s->cfg.streams) * 5, nullptr);
    for (cudaEvent_t& ev : s->marks) cudaEventCreate(&ev);
    s->sorted.assign(s->cfg.streams, nullptr);
    for (cudaEvent_t& ev : s->sorted) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    const char* tr = std::getenv("GBSORT_SERVER_TRACE");
    s->trace = tr && tr[0] == '1';
    s->t_origin = now_ns();
    s->image_cap.assign(s->cfg.streams, 0);
    s->slot_busy.assign(s->cfg.streams, false);
    gbsort_server* raw = s.release();
    raw->worker = std::thread([raw] { raw->run(); });
    *out = raw;
    return GBSORT_OK;
}

void gbsort_server_destroy(gbsort_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->paused = false;
    }
    s->cv.notify_all();
    s->worker.join();
    for (cudaStream_t st : s->streams) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    cudaFreeHost(s->err_words);
    for (uint8_t* im : s->images)
        if (im) cudaFreeHost(im);
    for (cudaEvent_t ev : s->marks) cudaEventDestroy(ev);
    for (cudaEvent_t ev : s->sorted) cudaEventDestroy(ev);
    cudaFree(s->pool);
    for (auto& kv : s->tickets) delete kv.second;
    delete s;
}

int gbsort_server_submit(gbsort_server* s, const gbsort_request* req, uint64_t* ticket) {
    if (!s || !req || !ticket) return GBSORT_ERR_INVALID_ARGUMENT;
    const size_t kb = gbsort_key_bytes(req->key_type);
    if (kb == 0) return GBSORT_ERR_INVALID_ARGUMENT;
    const size_t vb = req->value_bytes;
    if (vb != 0 && vb != 1 && vb != 2 && vb != 4 && vb != 8 && vb != 16) return GBSORT_ERR_INVALID_ARGUMENT;
    if (req->n && (!req->keys_in || !req->keys_out)) return GBSORT_ERR_INVALID_ARGUMENT;
    if (req->n && vb && (!req->values_in || !req->values_out)) return GBSORT_ERR_INVALID_ARGUMENT;
    auto* q = new Request();
    q->r = *req;
    q->kb = kb;
    q->cls = class_of(*req);
    // admission: the request alone must fit the empty pool
    {
        gbsort_segmented_plan* p = nullptr;
        size_t bytes = 0;
        std::vector<Request*> one{q};
        const int st = s->measure(one, !gbsort_server::in_place_device(q), &p, &bytes);
        gbsort_segmented_plan_destroy(p);
        if (st != GBSORT_OK || bytes > s->cfg.pool_bytes) {
            delete q;
            std::lock_guard<std::mutex> lk(s->mu);
            ++s->rejected;
            return st != GBSORT_OK ? st : GBSORT_ERR_BUDGET;
        }
    }
    q->t_submit = now_ns();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping) {
            delete q;
            return GBSORT_ERR_INVALID_ARGUMENT;
        }
        q->ticket = s->next_ticket++;
        s->tickets[q->ticket] = q;
        ++s->submitted;
        if (s->first_submit == 0) s->first_submit = q->t_submit;
        if (req->n == 0) {  // nothing to sort
            q->status = GBSORT_OK;
            q->t_launch = q->t_done = q->t_submit;
            ++s->completed_n;
        } else {
            s->queue.push_back(q);
            ++s->outstanding;
        }
        *ticket = q->ticket;
    }
    s->cv.notify_all();
    return GBSORT_OK;
}

int gbsort_server_wait(gbsort_server* s, uint64_t ticket, uint64_t timeout_ns) {
    if (!s) return GBSORT_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->tickets.find(ticket);
    if (it == s->tickets.end()) return GBSORT_ERR_INVALID_ARGUMENT;
    Request* q = it->second;
    if (q->status == GBSORT_ERR_NOT_READY && timeout_ns) {
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::nanoseconds(timeout_ns);
        s->done_cv.wait_until(lk, deadline, [q] { return q->status != GBSORT_ERR_NOT_READY; });
    }
    const int st = q->status;
    if (st != GBSORT_ERR_NOT_READY) {
        s->tickets.erase(ticket);
        delete q;
    }
    return st;
}

int gbsort_server_poll(gbsort_server* s, uint64_t ticket) { return gbsort_server_wait(s, ticket, 0); }

int gbsort_server_drain(gbsort_server* s, uint64_t timeout_ns) {
    if (!s) return GBSORT_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::nanoseconds(timeout_ns);
    const bool ok = s->done_cv.wait_until(lk, deadline, [s] { return s->outstanding == 0; });
    return ok ? GBSORT_OK : GBSORT_ERR_NOT_READY;
}

int gbsort_server_pause(gbsort_server* s) {
    if (!s) return GBSORT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    s->paused = true;
    return GBSORT_OK;
}

int gbsort_server_resume(gbsort_server* s) {
    if (!s) return GBSORT_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->paused = false;
    }
    s->cv.notify_all();
    return GBSORT_OK;
}

int gbsort_server_stats_get(gbsort_server* s, gbsort_server_stats* out) {
    if (!s || !out) return GBSORT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted;
    out->completed = s->completed_n;
    out->failed = s->failed;
    out->rejected = s->rejected;
    out->batches = s->batches;
    out->max_batch_requests = s->max_batch;
    out->keys_sorted = s->keys_sorted;
    out->bytes_sorted = s->bytes_sorted;
    out->pool_bytes = s->cfg.pool_bytes;
    out->pool_peak_bytes = s->arena->peak();
    out->kernel_launches = s->kernel_launches;
    std::vector<uint64_t> lat = s->latencies, qw = s->queue_waits;
    out->latency_p50_us = percentile_us(lat, 0.50);
    out->latency_p99_us = percentile_us(lat, 0.99);
    out->queue_p50_us = percentile_us(qw, 0.50);
    out->queue_p99_us = percentile_us(qw, 0.99);
    if (!lat.empty()) {
        double sum = 0.0;
        uint64_t mx = 0;
        for (uint64_t v : lat) {
            sum += double(v);
            mx = std::max(mx, v);
        }
        out->latency_mean_us = sum / double(lat.size()) / 1000.0;
        out->latency_max_us = double(mx) / 1000.0;
    }
    out->mean_batch_requests = s->batches ? double(s->batch_requests_sum) / double(s->batches) : 0.0;
    out->active_seconds = s->last_done > s->first_submit ? double(s->last_done - s->first_submit) * 1e-9 : 0.0;
    out->host_plan_seconds = double(s->plan_ns) * 1e-9;
    out->host_launch_seconds = double(s->launch_ns) * 1e-9;
    out->batch_seconds = double(s->batch_ns) * 1e-9;
    out->h2d_seconds = s->h2d_ms * 1e-3;
    out->sort_seconds = s->sort_ms * 1e-3;
    out->d2h_seconds = s->d2h_ms * 1e-3;
    return GBSORT_OK;
}

int gbsort_server_stats_reset(gbsort_server* s) {
    if (!s) return GBSORT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    s->submitted = s->completed_n = s->failed = s->rejected = s->batches = s->max_batch = 0;
    s->keys_sorted = s->bytes_sorted = s->batch_requests_sum = s->kernel_launches = 0;
    s->plan_ns = s->launch_ns = s->batch_ns = 0;
    s->h2d_ms = s->sort_ms = s->d2h_ms = 0.0;
    s->first_submit = s->last_done = 0;
    s->latencies.clear();
    s->queue_waits.clear();
    s->arena->reset_peak();
    return GBSORT_OK;
}

}  // extern "C"
