// segmented_api.cu — batched (segmented) sort: plan, bind, graph-captured run,
// size-bucket tuning table.  No reference counterpart (rsort sorts one array
// per call); it builds on the same kernels as the plain sort.
//
// A plan classifies every segment by its size bucket (floor(log2 n)) into one
// of three paths, per the tuning table:
//   CTA_S    whole segment in one 256-thread CTA's shared memory
//   CTA_L    whole segment in one 512-thread CTA's shared memory (bigger)
//   ONESWEEP the segment's tiles join one global tile list; one upsweep, one
//            scan, then one persistent launch per digit pass for all of them
// Every launch pulls its work (chunk, segment or tile) from a device counter.
// bind() uploads the tables into the caller's workspace once; run() captures
// the launch sequence into a CUDA graph the first time and replays it after.

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gbsort.h"
#include "plan.h"
#include "device_common.cuh"
#include "sort_params.h"
#include "segmented_internal.h"

namespace gbsort {

const KernelEntry* seg_entries_k1();
const KernelEntry* seg_entries_k2();
const KernelEntry* seg_entries_k4();
const KernelEntry* seg_entries_k8();
const KernelEntry* seg_entries_k16();
const KernelEntry* seg_upsweep_entry_k1();
const KernelEntry* seg_upsweep_entry_k2();
const KernelEntry* seg_upsweep_entry_k4();
const KernelEntry* seg_upsweep_entry_k8();
const KernelEntry* seg_upsweep_entry_k16();

namespace {

const KernelEntry* seg_entries(int kb) {
    switch (kb) {
        case 1: return seg_entries_k1();
        case 2: return seg_entries_k2();
        case 4: return seg_entries_k4();
        case 8: return seg_entries_k8();
        case 16: return seg_entries_k16();
        default: return nullptr;
    }
}
const KernelEntry* seg_upsweep_entry(int kb) {
    switch (kb) {
        case 1: return seg_upsweep_entry_k1();
        case 2: return seg_upsweep_entry_k2();
        case 4: return seg_upsweep_entry_k4();
        case 8: return seg_upsweep_entry_k8();
        case 16: return seg_upsweep_entry_k16();
        default: return nullptr;
    }
}

int width_index(int kb) { return kb == 1 ? 0 : kb == 2 ? 1 : kb == 4 ? 2 : kb == 8 ? 3 : 4; }

constexpr uint64_t UPSWEEP_CHUNK = uint64_t(1) << 18;
constexpr int BUCKETS = 41;  // floor(log2 n) = 0 .. 40

// ---- tuning table: path per (key width, value size, size bucket) ---------
std::mutex g_tune_mu;
int g_tune[5][6][BUCKETS];
bool g_tune_set[5][6];

// floor(log2 len), capped at the last bucket (0 for len 0)
int size_bucket(uint64_t len) { return len ? std::min(BUCKETS - 1, 63 - __builtin_clzll(len)) : 0; }

// The tuning-table row of one (key width, value size) and the CTA-sort
// capacities, read once per plan (one lock, not one per segment).
struct PathRule {
    int table[BUCKETS];
    bool set = false;
    uint64_t s_max = 0, l_max = 0;
};

PathRule path_rule(int kb, int vb, int s_max, int l_max) {
    PathRule r;
    r.s_max = uint64_t(s_max);
    r.l_max = uint64_t(l_max);
    const int wi = width_index(kb), vi = value_index(vb);
    std::lock_guard<std::mutex> lk(g_tune_mu);
    r.set = g_tune_set[wi][vi];
    if (r.set) std::memcpy(r.table, g_tune[wi][vi], sizeof(r.table));
    return r;
}

int path_of(const PathRule& r, uint64_t len) {
    int path = r.set ? r.table[size_bucket(len)] : -1;
    if (path < 0) path = len <= r.s_max ? GBSORT_PATH_CTA_S : len <= r.l_max ? GBSORT_PATH_CTA_L : GBSORT_PATH_ONESWEEP;
    // a path that cannot hold the segment falls through to the next one
    if ((path == GBSORT_PATH_CTA_S || path == GBSORT_PATH_CTA_S4) && len > r.s_max) path = GBSORT_PATH_CTA_L;
    if (path == GBSORT_PATH_CTA_L && len > r.l_max) path = GBSORT_PATH_ONESWEEP;
    return path;
}

int path_for(int kb, int vb, uint64_t len, int s_max, int l_max) {
    return path_of(path_rule(kb, vb, s_max, l_max), len);
}

// Largest first (for the balance of persistent CTAs pulling items in list
// order): a stable counting sort by size bucket, linear in the items.
void order_largest_first(std::vector<SegItem>& v) {
    if (v.size() < 2) return;
    size_t count[BUCKETS] = {};
    for (const SegItem& it : v) ++count[size_bucket(it.end - it.begin)];
    size_t start[BUCKETS];
    size_t at = 0;
    for (int b = BUCKETS - 1; b >= 0; --b) {
        start[b] = at;
        at += count[b];
    }
    std::vector<SegItem> out(v.size());
    for (const SegItem& it : v) out[start[size_bucket(it.end - it.begin)]++] = it;
    v.swap(out);
}

// One CTA (256 threads) per (segment, pass): exclusive scan of the segment's
// digit counts plus the segment's start = where each digit's run begins.
__global__ void __launch_bounds__(256) seg_scan_kernel(SegScanParams p) {
    __shared__ uint32_t tmp[16];
    const uint32_t s = blockIdx.x / p.passes;
    const uint32_t pp = blockIdx.x % p.passes;
    const uint32_t c = p.seg_counts[(size_t(s) * p.passes + pp) * 256 + threadIdx.x];
    uint32_t seg_len = 0;
    const uint32_t excl = block_exclusive_scan_256<uint32_t>(c, tmp, &seg_len);
    p.seg_gofs[(size_t(pp) * p.segments + s) * 256 + threadIdx.x] = uint32_t(p.seg_begin[s]) + excl;
    // the pass must run unless one digit holds this segment (for every segment)
    if (!__syncthreads_or(c == seg_len) && threadIdx.x == 0) atomicOr(p.nonuniform, 1u << pp);
}

// Copies elements [0, bytes) of one range with the CTA's threads (words when
// both ends allow).
__device__ void cta_copy_bytes(uint8_t* dst, const uint8_t* src, uint64_t bytes) {
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 3u) == 0) {
        const uint64_t w = bytes / 4;
        for (uint64_t i = threadIdx.x; i < w; i += blockDim.x)
            reinterpret_cast<uint32_t*>(dst)[i] = reinterpret_cast<const uint32_t*>(src)[i];
        for (uint64_t i = w * 4 + threadIdx.x; i < bytes; i += blockDim.x) dst[i] = src[i];
    } else {
        for (uint64_t i = threadIdx.x; i < bytes; i += blockDim.x) dst[i] = src[i];
    }
}

__global__ void __launch_bounds__(256) seg_fixup_kernel(SegFixupParams f) {
    const uint32_t all = (1u << f.passes) - 1u;
    if ((__popc(*f.nonuniform & all) & 1) == 0) return;  // an even number of passes ran: home already
    for (uint32_t t = blockIdx.x; t < f.num_tiles; t += gridDim.x) {
        const TileRec r = f.tiles[t];
        cta_copy_bytes(static_cast<uint8_t*>(f.keys_a) + r.base * f.key_bytes,
                       static_cast<const uint8_t*>(f.keys_b) + r.base * f.key_bytes, uint64_t(r.cnt) * f.key_bytes);
        if (f.val_bytes)
            cta_copy_bytes(static_cast<uint8_t*>(f.vals_a) + r.base * f.val_bytes,
                           static_cast<const uint8_t*>(f.vals_b) + r.base * f.val_bytes,
                           uint64_t(r.cnt) * f.val_bytes);
    }
}

}  // namespace

struct SegPlan {
    int key_type = 0, kb = 0, vb = 0, kind = 0, passes = 0, desc = 0;
    uint64_t n_total = 0;
    size_t num_segments = 0;
    KernelEntry pass{}, cta_s{}, cta_l{}, cta_s4{}, upsweep{};
    std::vector<SegItem> small_s, small_l, small_s4, up_items;
    std::vector<unsigned long long> large_begin;
    std::vector<TileRec> tiles;
    std::vector<uint8_t> image;  // host copy of the tables for the pageable upload
    uint64_t keys_in_cta = 0, keys_in_onesweep = 0;
    // workspace layout
    size_t alt_keys_off = 0, alt_vals_off = 0, ctl_off = 0, seg_counts_off = 0, zero_bytes = 0;
    size_t seg_gofs_off = 0, seg_begin_off = 0, tiles_off = 0, up_items_off = 0, small_s_off = 0, small_l_off = 0;
    size_t small_s4_off = 0;
    size_t status_off = 0, status_bytes = 0, total_bytes = 0;
    // ctl block: [0..15] tile counters, [16] upsweep items, [17] cta S, [18] cta L, [19] error word,
    // [20] cta S 4-bit
    // bound buffers and the cached graph
    void* keys = nullptr;
    void* vals = nullptr;
    uint8_t* ws = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::mutex mu;
};

namespace {

int build_plan(int key_type, size_t value_bytes, int descending, const uint64_t* off, size_t num, SegPlan* p) {
    const size_t kb = gbsort_key_bytes(key_type);
    const int vi = value_index(int(value_bytes));
    if (kb == 0 || vi < 0 || value_bytes > 16 || (num > 0 && off == nullptr)) return GBSORT_ERR_INVALID_ARGUMENT;
    p->key_type = key_type;
    p->kb = int(kb);
    p->vb = int(value_bytes);
    p->kind = key_type >= GBSORT_KEY_F32 ? KIND_FLOAT : key_type >= GBSORT_KEY_I8 ? KIND_SIGNED : KIND_UNSIGNED;
    p->passes = int(kb);
    p->desc = descending ? 1 : 0;
    p->num_segments = num;
    const KernelEntry* se = seg_entries(p->kb) + vi * 4;
    p->pass = se[0];
    p->cta_s = se[1];
    p->cta_l = se[2];
    p->cta_s4 = se[3];
    p->upsweep = *seg_upsweep_entry(p->kb);
    int lg = 0;
    while ((1 << (lg + 1)) <= p->passes) ++lg;
    const uint64_t seg_value_limit = uint64_t(1) << (30 - lg);  // 32-bit status words
    uint64_t n_total = 0;
    for (size_t s = 0; s < num; ++s) {
        if (off[s + 1] < off[s]) return GBSORT_ERR_INVALID_ARGUMENT;
        n_total = std::max<uint64_t>(n_total, off[s + 1]);
    }
    if (n_total >= 0xFFFFFFFFull) {
        set_last_error_text("segmented sort: the key array must hold fewer than 2^32 elements");
        return GBSORT_ERR_INVALID_ARGUMENT;
    }
    p->n_total = n_total;
    const uint64_t tile = uint64_t(p->pass.tile);
    const PathRule rule = path_rule(p->kb, p->vb, p->cta_s.tile, p->cta_l.tile);
    {  // size the onesweep lists once (their growth dominated planning)
        uint64_t tiles = 0, items = 0, large = 0;
        for (size_t s = 0; s < num; ++s) {
            const uint64_t len = off[s + 1] - off[s];
            if (len > 1 && path_of(rule, len) == GBSORT_PATH_ONESWEEP) {
                tiles += (len + tile - 1) / tile;
                items += (len + UPSWEEP_CHUNK - 1) / UPSWEEP_CHUNK;
                ++large;
            }
        }
        p->tiles.reserve(size_t(std::min<uint64_t>(tiles, 0xFFFFFFFFull)));
        p->up_items.reserve(size_t(items));
        p->large_begin.reserve(size_t(large));
    }
    for (size_t s = 0; s < num; ++s) {
        const uint64_t b = off[s], e = off[s + 1], len = e - b;
        if (len <= 1) continue;  // already sorted
        const int path = path_of(rule, len);
        SegItem it{b, e, 0, 0};
        if (path == GBSORT_PATH_CTA_S) {
            p->small_s.push_back(it);
            p->keys_in_cta += len;
        } else if (path == GBSORT_PATH_CTA_S4) {
            p->small_s4.push_back(it);
            p->keys_in_cta += len;
        } else if (path == GBSORT_PATH_CTA_L) {
            p->small_l.push_back(it);
            p->keys_in_cta += len;
        } else {
            if (len > seg_value_limit) {
                set_last_error_text("segmented sort: a segment exceeds the batched onesweep limit");
                return GBSORT_ERR_INVALID_ARGUMENT;
            }
            const uint32_t idx = uint32_t(p->large_begin.size());
            p->large_begin.push_back(b);
            const uint64_t nt = (len + tile - 1) / tile;
            for (uint64_t t = 0; t < nt; ++t) {
                TileRec r{};
                r.base = b + t * tile;
                r.cnt = uint32_t(std::min<uint64_t>(tile, e - r.base));
                r.seg_flags = (idx << 2) | (t + 1 == nt ? 2u : 0u) | (t == 0 ? 1u : 0u);
                p->tiles.push_back(r);
            }
            for (uint64_t c = b; c < e; c += UPSWEEP_CHUNK)
                p->up_items.push_back(SegItem{c, std::min<uint64_t>(e, c + UPSWEEP_CHUNK), idx, 0});
            p->keys_in_onesweep += len;
        }
    }
    if (p->tiles.size() >= 0xFFFFFFFFull) return GBSORT_ERR_INVALID_ARGUMENT;
    // biggest segments first: better balance for the persistent CTA sorts
    order_largest_first(p->small_s);
    order_largest_first(p->small_l);
    order_largest_first(p->small_s4);
    order_largest_first(p->up_items);

    const size_t L = p->large_begin.size();
    size_t o = 0;
    p->alt_keys_off = o;
    o = align_up(o + (L ? size_t(n_total) * kb : 0), 256);
    p->alt_vals_off = o;
    o = align_up(o + (L ? size_t(n_total) * value_bytes : 0), 256);
    p->ctl_off = o;
    o = align_up(o + 256, 256);
    p->seg_counts_off = o;
    o = align_up(o + L * p->passes * 256 * 4, 256);
    p->zero_bytes = o - p->ctl_off;
    p->seg_gofs_off = o;
    o = align_up(o + L * p->passes * 256 * 4, 256);
    p->seg_begin_off = o;
    o = align_up(o + L * 8, 256);
    p->tiles_off = o;
    o = align_up(o + p->tiles.size() * sizeof(TileRec), 256);
    p->up_items_off = o;
    o = align_up(o + p->up_items.size() * sizeof(SegItem), 256);
    p->small_s_off = o;
    o = align_up(o + p->small_s.size() * sizeof(SegItem), 256);
    p->small_l_off = o;
    o = align_up(o + p->small_l.size() * sizeof(SegItem), 256);
    p->small_s4_off = o;
    o = align_up(o + p->small_s4.size() * sizeof(SegItem), 256);
    p->status_off = o;
    p->status_bytes = p->tiles.size() * 256 * 4;
    o = align_up(o + p->status_bytes, 256);
    p->total_bytes = o;
    return GBSORT_OK;
}

int launch(const KernelEntry& e, uint32_t grid, void* params, cudaStream_t s, const char* what) {
    void* args[] = {params};
    const cudaError_t err = cudaLaunchKernel(e.fn, dim3(grid), dim3(e.threads), args, e.smem, s);
    if (err != cudaSuccess) {
        set_last_error(what, err);
        return GBSORT_ERR_CUDA;
    }
    return GBSORT_OK;
}

uint32_t grid_for(const KernelEntry& e, uint64_t work) {
    const uint64_t cap = uint64_t(device_sm_count()) * uint64_t(std::max(1, resident_ctas(e)));
    return uint32_t(std::max<uint64_t>(1, std::min<uint64_t>(cap, work)));
}

int enqueue_segmented(SegPlan* p, cudaStream_t s) {
    uint8_t* ws = p->ws;
    uint32_t* ctl = reinterpret_cast<uint32_t*>(ws + p->ctl_off);
    uint32_t* err = ctl + 19;
    cudaError_t e = cudaMemsetAsync(ws + p->ctl_off, 0, p->zero_bytes, s);
    if (e != cudaSuccess) {
        set_last_error("segmented memset", e);
        return GBSORT_ERR_CUDA;
    }
    const size_t L = p->large_begin.size();
    const bool odd = (p->passes & 1) != 0;
    const bool skip = gbsort_get_pass_skip() != 0;
    void* alt_keys = ws + p->alt_keys_off;
    void* alt_vals = p->vb ? ws + p->alt_vals_off : nullptr;
    int st;
    if (L) {
        SegUpsweepParams up{};
        up.keys = p->keys;
        up.kind = p->kind;
        up.desc = p->desc;
        up.items = reinterpret_cast<const SegItem*>(ws + p->up_items_off);
        up.num_items = uint32_t(p->up_items.size());
        up.item_counter = ctl + 16;
        up.seg_counts = reinterpret_cast<uint32_t*>(ws + p->seg_counts_off);
        up.status = ws + p->status_off;
        up.status_bytes = p->status_bytes;
        up.mirror_keys = odd ? alt_keys : nullptr;
        up.vals = p->vals;
        up.mirror_vals = (odd && p->vb) ? alt_vals : nullptr;
        up.val_bytes = uint32_t(p->vb);
        if ((st = launch(p->upsweep, grid_for(p->upsweep, p->up_items.size()), &up, s, "segmented upsweep")))
            return st;
        SegScanParams sc{};
        sc.seg_counts = up.seg_counts;
        sc.seg_begin = reinterpret_cast<const unsigned long long*>(ws + p->seg_begin_off);
        sc.seg_gofs = reinterpret_cast<uint32_t*>(ws + p->seg_gofs_off);
        sc.segments = uint32_t(L);
        sc.passes = uint32_t(p->passes);
        sc.nonuniform = ctl + 21;
        void* args[] = {&sc};
        e = cudaLaunchKernel(reinterpret_cast<const void*>(&seg_scan_kernel), dim3(uint32_t(L) * p->passes),
                             dim3(256), args, 0, s);
        if (e != cudaSuccess) {
            set_last_error("segmented scan", e);
            return GBSORT_ERR_CUDA;
        }
    }
    auto cta_launch = [&](const KernelEntry& k, const std::vector<SegItem>& v, size_t off, int ctr) {
        if (v.empty()) return int(GBSORT_OK);
        CtaSortParams cp{};
        cp.keys = p->keys;
        cp.vals = p->vals;
        cp.segs = reinterpret_cast<const SegItem*>(ws + off);
        cp.num_segs = uint32_t(v.size());
        cp.seg_counter = ctl + ctr;
        cp.kind = p->kind;
        cp.desc = p->desc;
        return launch(k, grid_for(k, v.size()), &cp, s, "segmented CTA sort");
    };
    if ((st = cta_launch(p->cta_l, p->small_l, p->small_l_off, 18))) return st;
    if ((st = cta_launch(p->cta_s, p->small_s, p->small_s_off, 17))) return st;
    if ((st = cta_launch(p->cta_s4, p->small_s4, p->small_s4_off, 20))) return st;
    if (L) {
        const uint32_t T = uint32_t(p->tiles.size());
        const uint32_t grid = grid_for(p->pass, T);
        for (int pass = 0; pass < p->passes; ++pass) {
            const bool from_user = ((pass + (odd ? 1 : 0)) & 1) == 0;
            PassParams pp{};
            pp.keys_in = from_user ? p->keys : alt_keys;
            pp.keys_out = from_user ? alt_keys : p->keys;
            pp.vals_in = p->vb ? (from_user ? p->vals : alt_vals) : nullptr;
            pp.vals_out = p->vb ? (from_user ? alt_vals : p->vals) : nullptr;
            pp.n = p->n_total;
            pp.num_tiles = T;
            pp.pass = pass;
            pp.kind = p->kind;
            pp.desc = p->desc;
            pp.twiddle_load = pass == 0;
            pp.twiddle_store = pass == p->passes - 1;
            pp.tma_keys = 1;
            pp.tma_vals = p->vb ? 1 : 0;
            pp.gp_counts = nullptr;
            pp.status = ws + p->status_off;
            pp.tile_counter = ctl + pass;
            pp.err = err;
            pp.wait_limit_ns = wait_limit_ns();
            pp.tiles = reinterpret_cast<const TileRec*>(ws + p->tiles_off);
            pp.seg_gofs = reinterpret_cast<const uint32_t*>(ws + p->seg_gofs_off) + size_t(pass) * L * 256;
            pp.skip = skip ? 1 : 0;
            pp.passes = p->passes;
            pp.start_alt = odd ? 1 : 0;
            pp.nonuniform_mask = ctl + 21;
            pp.keys_a = p->keys;
            pp.vals_a = p->vals;
            pp.keys_b = alt_keys;
            pp.vals_b = alt_vals;
            if ((st = launch(p->pass, grid, &pp, s, "segmented pass"))) return st;
        }
        if (skip && !odd) {  // odd pass counts start mirrored and always end at home
            SegFixupParams fp{};
            fp.tiles = reinterpret_cast<const TileRec*>(ws + p->tiles_off);
            fp.num_tiles = T;
            fp.passes = p->passes;
            fp.nonuniform = ctl + 21;
            fp.key_bytes = uint32_t(p->kb);
            fp.val_bytes = uint32_t(p->vb);
            fp.keys_b = alt_keys;
            fp.keys_a = p->keys;
            fp.vals_b = alt_vals;
            fp.vals_a = p->vals;
            void* args[] = {&fp};
            e = cudaLaunchKernel(reinterpret_cast<const void*>(&seg_fixup_kernel),
                                 dim3(std::max<uint32_t>(1, std::min<uint32_t>(T, uint32_t(device_sm_count()) * 4))),
                                 dim3(256), args, 0, s);
            if (e != cudaSuccess) {
                set_last_error("segmented fixup", e);
                return GBSORT_ERR_CUDA;
            }
        }
    }
    return GBSORT_OK;
}

int prepare_all(SegPlan* p) {
    int st;
    if (!device_is_sm103()) return GBSORT_ERR_UNSUPPORTED;
    if (!p->large_begin.empty()) {
        if ((st = prepare_kernel(p->pass))) return st;
        if ((st = prepare_kernel(p->upsweep))) return st;
    }
    if (!p->small_s.empty() && (st = prepare_kernel(p->cta_s))) return st;
    if (!p->small_l.empty() && (st = prepare_kernel(p->cta_l))) return st;
    if (!p->small_s4.empty() && (st = prepare_kernel(p->cta_s4))) return st;
    return GBSORT_OK;
}

void drop_graph(SegPlan* p) {
    if (p->exec) {
        cudaGraphExecDestroy(p->exec);
        p->exec = nullptr;
    }
}

}  // namespace
}  // namespace gbsort

using namespace gbsort;

struct gbsort_segmented_plan : SegPlan {};

extern "C" {

int gbsort_segmented_plan_create(int key_type, size_t value_bytes, int descending, const uint64_t* h_offsets,
                                 size_t num_segments, gbsort_segmented_plan** out) {
    if (out == nullptr) return GBSORT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    auto* p = new gbsort_segmented_plan();
    const int st = build_plan(key_type, value_bytes, descending, h_offsets, num_segments, p);
    if (st != GBSORT_OK) {
        delete p;
        return st;
    }
    *out = p;
    return GBSORT_OK;
}

void gbsort_segmented_plan_destroy(gbsort_segmented_plan* plan) {
    if (!plan) return;
    drop_graph(plan);
    delete plan;
}

int gbsort_segmented_plan_info(const gbsort_segmented_plan* p, gbsort_segmented_info* out) {
    if (!p || !out) return GBSORT_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->num_segments = p->num_segments;
    out->cta_small_segments = p->small_s.size();
    out->cta_large_segments = p->small_l.size();
    out->cta_small4_segments = p->small_s4.size();
    out->onesweep_segments = p->large_begin.size();
    out->onesweep_tiles = p->tiles.size();
    out->keys_in_cta = p->keys_in_cta;
    out->keys_in_onesweep = p->keys_in_onesweep;
    out->cta_small_max = uint32_t(p->cta_s.tile);
    out->cta_large_max = uint32_t(p->cta_l.tile);
    out->onesweep_tile = uint32_t(p->pass.tile);
    out->workspace_bytes = p->total_bytes;
    out->kernel_launches = (p->large_begin.empty()
                                ? 0
                                : 2 + uint64_t(p->passes) + ((gbsort_get_pass_skip() && (p->passes & 1) == 0) ? 1 : 0)) +
                           !p->small_l.empty() + !p->small_s.empty() + !p->small_s4.empty();
    return GBSORT_OK;
}

}  // extern "C"

namespace gbsort {

size_t segmented_table_bytes(const gbsort_segmented_plan* p) { return p->status_off - p->seg_begin_off; }

// Host image of the workspace range [seg_begin_off, status_off): segment
// begins, tile list, upsweep items, CTA segment lists.
void segmented_table_image(const gbsort_segmented_plan* p, uint8_t* dst) {
    std::memset(dst, 0, segmented_table_bytes(p));
    auto put = [&](size_t off, const void* src, size_t bytes) {
        if (bytes) std::memcpy(dst + (off - p->seg_begin_off), src, bytes);
    };
    put(p->seg_begin_off, p->large_begin.data(), p->large_begin.size() * 8);
    put(p->tiles_off, p->tiles.data(), p->tiles.size() * sizeof(TileRec));
    put(p->up_items_off, p->up_items.data(), p->up_items.size() * sizeof(SegItem));
    put(p->small_s_off, p->small_s.data(), p->small_s.size() * sizeof(SegItem));
    put(p->small_l_off, p->small_l.data(), p->small_l.size() * sizeof(SegItem));
    put(p->small_s4_off, p->small_s4.data(), p->small_s4.size() * sizeof(SegItem));
}

// bind with the table image taken from `image` (pinned memory lets the
// upload run asynchronously); image == nullptr builds it in pageable memory.
namespace {
// Copies a table image that is already in device memory into a workspace
// (a kernel, not a copy engine: it cannot queue behind bulk transfers).
__global__ void __launch_bounds__(256) table_copy_kernel(uint8_t* dst, const uint8_t* src, size_t bytes) {
    const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x, stride = size_t(gridDim.x) * blockDim.x;
    size_t done = 0;
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0) {
        const size_t nv = bytes >> 4;
        for (size_t i = t; i < nv; i += stride) reinterpret_cast<uint4*>(dst)[i] = reinterpret_cast<const uint4*>(src)[i];
        done = nv << 4;
    }
    for (size_t i = done + t; i < bytes; i += stride) dst[i] = src[i];
}
}  // namespace

// image_on_device: `image` is a device copy of segmented_table_image(p),
// moved into the workspace by a kernel; otherwise host memory (pinned, or
// nullptr for the plan's own pageable image) uploaded on `stream`.
int segmented_bind_image(gbsort_segmented_plan* p, void* d_keys, void* d_values, void* d_workspace,
                         size_t workspace_bytes, void* stream, const uint8_t* image, bool image_on_device) {
    if (!p || (p->num_segments && !d_keys) || (p->vb && p->num_segments && !d_values)) return GBSORT_ERR_INVALID_ARGUMENT;
    if (d_workspace == nullptr || workspace_bytes < p->total_bytes) return GBSORT_ERR_WORKSPACE_TOO_SMALL;
    if (reinterpret_cast<uintptr_t>(d_workspace) % 16) {  // the status array is cleared by 16-byte stores
        set_last_error_text("the workspace must be 16-byte aligned");
        return GBSORT_ERR_INVALID_ARGUMENT;
    }
    if ((reinterpret_cast<uintptr_t>(d_keys) % p->kb) || (p->vb && reinterpret_cast<uintptr_t>(d_values) % p->vb))
        return GBSORT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(p->mu);
    const int st = prepare_all(p);
    if (st != GBSORT_OK) return st;
    if (p->keys != d_keys || p->vals != d_values || p->ws != d_workspace) drop_graph(p);
    p->keys = d_keys;
    p->vals = d_values;
    p->ws = static_cast<uint8_t*>(d_workspace);
    // the tables sit back to back in the workspace: upload them as one image
    const size_t bytes = segmented_table_bytes(p);
    if (bytes == 0) return GBSORT_OK;
    if (image_on_device) {
        const uint32_t grid = uint32_t(std::min<size_t>((bytes + 4095) / 4096, 1024));
        table_copy_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(p->ws + p->seg_begin_off, image,
                                                                              bytes);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_last_error("segmented table copy", e);
            return GBSORT_ERR_CUDA;
        }
        return GBSORT_OK;
    }
    const uint8_t* src = image;
    if (src == nullptr) {  // kept with the plan: the copy may read it later
        p->image.resize(bytes);
        segmented_table_image(p, p->image.data());
        src = p->image.data();
    }
    const cudaError_t e = cudaMemcpyAsync(p->ws + p->seg_begin_off, src, bytes, cudaMemcpyHostToDevice,
                                          static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) {
        set_last_error("segmented table upload", e);
        return GBSORT_ERR_CUDA;
    }
    return GBSORT_OK;
}

}  // namespace gbsort

extern "C" {

int gbsort_segmented_bind(gbsort_segmented_plan* p, void* d_keys, void* d_values, void* d_workspace,
                          size_t workspace_bytes, void* stream) {
    return gbsort::segmented_bind_image(p, d_keys, d_values, d_workspace, workspace_bytes, stream, nullptr);
}

// Runs the bound plan.  use_graph != 0: the first run captures the launch
// sequence into a CUDA graph (the stream must be capturable: not the legacy
// default stream) and later runs replay it; 0: plain launches every time.
int gbsort_segmented_run(gbsort_segmented_plan* p, int use_graph, void* stream) {
    if (!p || !p->ws) return GBSORT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(p->mu);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!use_graph || s == nullptr) return enqueue_segmented(p, s);
    if (!p->exec) {
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            set_last_error("segmented graph capture", e);
            return GBSORT_ERR_CUDA;
        }
        const int st = enqueue_segmented(p, s);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(s, &g);
        if (st != GBSORT_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) set_last_error("segmented graph capture", e);
            return st != GBSORT_OK ? st : GBSORT_ERR_CUDA;
        }
        e = cudaGraphInstantiate(&p->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            p->exec = nullptr;
            set_last_error("segmented graph instantiate", e);
            return GBSORT_ERR_CUDA;
        }
    }
    const cudaError_t e = cudaGraphLaunch(p->exec, s);
    if (e != cudaSuccess) {
        set_last_error("segmented graph launch", e);
        return GBSORT_ERR_CUDA;
    }
    return GBSORT_OK;
}

int gbsort_segmented_status(gbsort_segmented_plan* p, void* stream) {
    if (!p || !p->ws) return GBSORT_ERR_INVALID_ARGUMENT;
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    uint32_t err = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&err, p->ws + p->ctl_off + 19 * 4, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        set_last_error("segmented status", e);
        return GBSORT_ERR_CUDA;
    }
    if (err & ERRBIT_BOUNDS) return GBSORT_ERR_INTERNAL;
    if (err & ERRBIT_TIMEOUT) return GBSORT_ERR_TIMEOUT;
    return GBSORT_OK;
}

int gbsort_segmented_sort(int key_type, int descending, void* d_keys, void* d_values, size_t value_bytes,
                          const uint64_t* h_offsets, size_t num_segments, size_t* temp_bytes, void* d_workspace,
                          void* stream) {
    if (temp_bytes == nullptr) return GBSORT_ERR_INVALID_ARGUMENT;
    gbsort_segmented_plan* p = nullptr;
    int st = gbsort_segmented_plan_create(key_type, value_bytes, descending, h_offsets, num_segments, &p);
    if (st != GBSORT_OK) return st;
    if (d_workspace == nullptr) {
        *temp_bytes = p->total_bytes;
        gbsort_segmented_plan_destroy(p);
        return GBSORT_OK;
    }
    st = gbsort_segmented_bind(p, d_keys, d_values, d_workspace, *temp_bytes, stream);
    if (st == GBSORT_OK) st = gbsort_segmented_run(p, 0, stream);
    // the tables were uploaded from the plan's host memory: keep it alive
    // until the copies have been consumed
    if (st == GBSORT_OK) {
        const cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
        if (e != cudaSuccess) {
            set_last_error("segmented sort", e);
            st = GBSORT_ERR_CUDA;
        }
    }
    gbsort_segmented_plan_destroy(p);
    return st;
}

int gbsort_set_segmented_path(int key_type, size_t value_bytes, int size_log2, int path) {
    const size_t kb = gbsort_key_bytes(key_type);
    const int vi = value_index(int(value_bytes));
    if (kb == 0 || vi < 0 || size_log2 < -1 || size_log2 >= BUCKETS || path < -1)
        return GBSORT_ERR_INVALID_ARGUMENT;
    if (path > GBSORT_PATH_CTA_S4) return GBSORT_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const int wi = width_index(int(kb));
    if (!g_tune_set[wi][vi]) {
        for (int b = 0; b < BUCKETS; ++b) g_tune[wi][vi][b] = -1;
        g_tune_set[wi][vi] = true;
    }
    if (size_log2 < 0) {
        for (int b = 0; b < BUCKETS; ++b) g_tune[wi][vi][b] = path;
    } else {
        g_tune[wi][vi][size_log2] = path;
    }
    return GBSORT_OK;
}

int gbsort_segmented_path_override(int key_type, size_t value_bytes, int size_log2) {
    const size_t kb = gbsort_key_bytes(key_type);
    const int vi = value_index(int(value_bytes));
    if (kb == 0 || vi < 0 || size_log2 < 0 || size_log2 >= BUCKETS) return -1;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    const int wi = width_index(int(kb));
    return g_tune_set[wi][vi] ? g_tune[wi][vi][size_log2] : -1;
}

int gbsort_get_segmented_path(int key_type, size_t value_bytes, int size_log2) {
    const size_t kb = gbsort_key_bytes(key_type);
    const int vi = value_index(int(value_bytes));
    if (kb == 0 || vi < 0 || size_log2 < 0 || size_log2 >= BUCKETS) return -2;
    const uint64_t len = uint64_t(1) << size_log2;
    const KernelEntry* se = seg_entries(int(kb)) + vi * 4;
    return path_for(int(kb), int(value_bytes), len, se[1].tile, se[2].tile);
}

}  // extern "C"

namespace gbsort {
// Device address of a bound plan's error word (the sort server copies it to
// pinned host memory at the end of each batch instead of synchronizing).
const void* segmented_error_word(const gbsort_segmented_plan* p) {
    return (p && p->ws) ? p->ws + p->ctl_off + 19 * 4 : nullptr;
}
}  // namespace gbsort
