/*
 * gbsort.h — C ABI of the GB300 (sm_103a) onesweep LSD radix sort.
 *
 * Every entry point is a plain C function over raw device pointers and sizes,
 * so any FFI (ctypes, cgo, JNI, N-API) and the header-only C++ shim in
 * include/rsort/rsort.cuh can bind it.  No CUDA type appears in a signature:
 * streams are passed as `void*` (a cudaStream_t, or NULL for the legacy
 * default stream).
 *
 * Reference interface replaced (AwardOfSky/CUDA-Fast-Sort, "rsort" v0.4.0):
 *   include/rsort/rsort.cuh:13-30   rsort::sort                  -> gbsort_sort_keys
 *   include/rsort/rsort.cuh:33-50   rsort::sort_descending       -> gbsort_sort_keys(descending=1)
 *   include/rsort/rsort.cuh:53-71   rsort::sort_pairs            -> gbsort_sort_pairs
 *   include/rsort/rsort.cuh:74-92   rsort::sort_pairs_descending -> gbsort_sort_pairs(descending=1)
 *   include/rsort/detail/radix_kernel.cuh:486-507  size query (workspace == NULL
 *       writes the required bytes to *temp_bytes and returns, no device work)
 *
 * Protocol (same as rsort): call once with workspace == NULL to learn
 * *temp_bytes, allocate that many device bytes, call again with the
 * workspace; keys (and values) are sorted in place, ping-ponging through the
 * workspace.  The library allocates no device memory on this path.  The
 * workspace must be 16-byte aligned (cudaMalloc returns 256-byte aligned
 * memory); an unaligned one is refused with GBSORT_ERR_INVALID_ARGUMENT.
 *
 * Deliberate differences from rsort, all in the caller's favour:
 *   - the stream argument is honoured (rsort replaces it by a private stream
 *     and replays a graph on the legacy stream, radix_kernel.cuh:583-601);
 *   - n == 0 is a no-op (rsort underflows, radix_kernel.cuh:385);
 *   - errors come back as a gbsort_status instead of being dropped;
 *   - device-side waits are bounded: a stalled lookback sets an error word
 *     in the workspace (read with gbsort_workspace_status) instead of hanging.
 */
#ifndef GBSORT_H
#define GBSORT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Key types.  The 13 types rsort validates (benchmark/validate_sort.cuh:36-40).
 * GBSORT_KEY_F128 is `long double` on platforms where it is 16 bytes: the key
 * is ordered as a raw 128-bit pattern with the float twiddle applied at bit
 * 127, exactly as rsort does (detail/radix_kernel.cuh:351-356 reinterprets the
 * buffer as unsigned __int128; detail/tuning.cuh:356-357 twiddles it). */
typedef enum gbsort_key_type {
    GBSORT_KEY_U8 = 0,
    GBSORT_KEY_U16 = 1,
    GBSORT_KEY_U32 = 2,
    GBSORT_KEY_U64 = 3,
    GBSORT_KEY_U128 = 4,
    GBSORT_KEY_I8 = 5,
    GBSORT_KEY_I16 = 6,
    GBSORT_KEY_I32 = 7,
    GBSORT_KEY_I64 = 8,
    GBSORT_KEY_I128 = 9,
    GBSORT_KEY_F32 = 10,
    GBSORT_KEY_F64 = 11,
    GBSORT_KEY_F128 = 12,
    GBSORT_KEY_COUNT = 13
} gbsort_key_type;

typedef enum gbsort_status {
    GBSORT_OK = 0,
    GBSORT_ERR_INVALID_ARGUMENT = 1,   /* bad key type, value size, null pointer */
    GBSORT_ERR_WORKSPACE_TOO_SMALL = 2,/* *temp_bytes smaller than required     */
    GBSORT_ERR_CUDA = 3,               /* a CUDA runtime call or launch failed  */
    GBSORT_ERR_TIMEOUT = 4,            /* a bounded device wait ran out         */
    GBSORT_ERR_UNSUPPORTED = 5,        /* no device of compute capability 10.3  */
    GBSORT_ERR_BUDGET = 6,             /* server: request exceeds memory budget */
    GBSORT_ERR_NOT_READY = 7,          /* server: result not yet available      */
    GBSORT_ERR_INTERNAL = 8            /* a device-side bounds check fired      */
} gbsort_status;

/* Bytes of one key of the given type (0 for an unknown type). */
size_t gbsort_key_bytes(int key_type);

/* Human-readable text for a status code (static storage). */
const char* gbsort_status_string(int status);

/* Library version string, e.g. "gbsort 1.0 sm_103a". */
const char* gbsort_version(void);

/* Text of the last CUDA failure seen by this thread ("" if none). */
const char* gbsort_last_error(void);

/* ------------------------------------------------------------------------ */
/* Plain sort: the drop-in for rsort::sort / sort_descending /              */
/* sort_pairs / sort_pairs_descending (include/rsort/rsort.cuh:13-92).       */
/* ------------------------------------------------------------------------ */

/* Keys-only sort, in place.  workspace == NULL: writes the required bytes to
 * *temp_bytes and returns GBSORT_OK without touching the device.  Otherwise
 * *temp_bytes must hold the workspace size (>= the required bytes). */
int gbsort_sort_keys(int key_type, int descending, void* d_keys,
                     size_t* temp_bytes, void* d_workspace, size_t n,
                     void* stream);

/* Key-value sort, in place.  value_bytes is the size of one value: 1, 2, 4,
 * 8 or 16 (values are moved as raw bytes, so any trivially copyable type of
 * those sizes works).  Equal keys keep their input order (stable). */
int gbsort_sort_pairs(int key_type, int descending, void* d_keys,
                      void* d_values, size_t value_bytes, size_t* temp_bytes,
                      void* d_workspace, size_t n, void* stream);

/* Input-preserving ("DoubleBuffer") forms, like the reference's CUB
 * comparator (benchmark/cub_radix_double.cu:82-111): keys_in / values_in are
 * only read and the sorted result is written to keys_out / values_out; the
 * passes ping-pong between the output and the workspace, arranged on the
 * device so the last one lands in the output (no extra copy).  Same size
 * query and workspace size as the in-place form.  Identical input and output
 * pointers sort in place; any other overlap is GBSORT_ERR_INVALID_ARGUMENT. */
int gbsort_sort_keys_copy(int key_type, int descending, const void* d_keys_in,
                          void* d_keys_out, size_t* temp_bytes,
                          void* d_workspace, size_t n, void* stream);
int gbsort_sort_pairs_copy(int key_type, int descending, const void* d_keys_in,
                           void* d_keys_out, const void* d_values_in,
                           void* d_values_out, size_t value_bytes,
                           size_t* temp_bytes, void* d_workspace, size_t n,
                           void* stream);

/* DoubleBuffer forms, as cub::DoubleBuffer in the reference's CUB comparator
 * (benchmark/cub_radix_double.cu:79-111): the caller owns two key buffers
 * (and two value buffers) of n elements; *selector (0 or 1) names the one
 * holding the input and, on return, the one holding the sorted result (it
 * flips only for 1-byte keys, whose sort is a single pass).  The passes ping-pong between the caller's buffers, so the
 * workspace holds only control words and lookback status, not n-sized
 * alternate buffers (2^28 u32 keys: ~30 MB instead of ~1.1 GB).  The other
 * buffer is clobbered.  d_workspace == NULL writes the required bytes to
 * *temp_bytes (no device work).  The buffers of a pair must not overlap. */
int gbsort_sort_keys_double_buffer(int key_type, int descending, void* d_keys0,
                                   void* d_keys1, int* selector,
                                   size_t* temp_bytes, void* d_workspace,
                                   size_t n, void* stream);
int gbsort_sort_pairs_double_buffer(int key_type, int descending,
                                    void* d_keys0, void* d_keys1,
                                    void* d_values0, void* d_values1,
                                    size_t value_bytes, int* selector,
                                    size_t* temp_bytes, void* d_workspace,
                                    size_t n, void* stream);
/* gbsort_workspace_status for a DoubleBuffer workspace (its control block
 * sits at the start): synchronizes `stream`, then reports a timed-out wait
 * or a failed bounds check of the last sort that used it. */
int gbsort_double_buffer_status(int key_type, size_t value_bytes, size_t n,
                                void* d_workspace, void* stream);

/* Typed convenience entry points (same semantics as above). */
#define GBSORT_DECLARE_TYPED(name)                                              \
    int gbsort_sort_##name(void* d_keys, size_t* temp_bytes, void* d_workspace, \
                           size_t n, void* stream);                             \
    int gbsort_sort_##name##_desc(void* d_keys, size_t* temp_bytes,             \
                                  void* d_workspace, size_t n, void* stream);   \
    int gbsort_sort_pairs_##name(void* d_keys, void* d_values,                  \
                                 size_t value_bytes, size_t* temp_bytes,        \
                                 void* d_workspace, size_t n, void* stream);    \
    int gbsort_sort_pairs_##name##_desc(void* d_keys, void* d_values,           \
                                        size_t value_bytes, size_t* temp_bytes, \
                                        void* d_workspace, size_t n,            \
                                        void* stream);
GBSORT_DECLARE_TYPED(u8)
GBSORT_DECLARE_TYPED(u16)
GBSORT_DECLARE_TYPED(u32)
GBSORT_DECLARE_TYPED(u64)
GBSORT_DECLARE_TYPED(u128)
GBSORT_DECLARE_TYPED(i8)
GBSORT_DECLARE_TYPED(i16)
GBSORT_DECLARE_TYPED(i32)
GBSORT_DECLARE_TYPED(i64)
GBSORT_DECLARE_TYPED(i128)
GBSORT_DECLARE_TYPED(f32)
GBSORT_DECLARE_TYPED(f64)
GBSORT_DECLARE_TYPED(f128)
#undef GBSORT_DECLARE_TYPED

/* Keys-only sort that allocates nothing and takes no workspace.  No
 * counterpart in the reference (rsort always needs a caller workspace).  For
 * callers that may not allocate device memory where they sort — cudaMalloc /
 * cudaFree can block or synchronize the device, and some hosts own every
 * device byte or give a library a fixed budget.  The scratch is a 16 MiB
 * static device array inside the library, held by every GPU that loads it
 * until exit.  Limit: the sort fits when the size query reports <= 16 MiB
 * (about 4.0 M 4-byte, 2.0 M 8-byte or 1.0 M 16-byte keys); larger n returns
 * GBSORT_ERR_WORKSPACE_TOO_SMALL with no device work.  The first call on a
 * device looks up the array's address on that device: make it before any
 * stream capture there.  All calls share the array (the sort re-clears what
 * must start at zero); calls that overlap on the GPU race, so order them. */
int gbsort_sort_keys_noalloc(int key_type, int descending, void* d_keys,
                             size_t n, void* stream);

/* Device-side status of the last gbsort_sort_keys_noalloc call of this
 * (key_type, n): synchronizes `stream`, then reads the error word the sort's
 * kernels left in the static scratch (GBSORT_OK, GBSORT_ERR_TIMEOUT when a
 * bounded device wait ran out, GBSORT_ERR_INTERNAL for a failed bounds
 * check).  Call it before the next noalloc call, which clears the word.  No
 * counterpart in the reference (like the noalloc sort itself); allocates
 * nothing. */
int gbsort_noalloc_status(int key_type, size_t n, void* stream);

/* Sort from HOST buffers: copies n keys (and values) from host memory into
 * the caller's device buffer d_buffer (16-byte aligned), sorts them there and
 * copies the result back, then synchronizes.  d_buffer must hold
 * gbsort_host_buffer_bytes(...) bytes (twice the keys and values, plus
 * control words); pinned host memory gives full copy bandwidth.  No
 * allocation happens inside.  Arrays of >= GBSORT_HOST_SPLIT_MIN keys
 * (environment, default 2^25; keys of 2 bytes or more) are partitioned by
 * their top digit first and sorted in groups of consecutive buckets of
 * ~2^24 keys (2 to 16; GBSORT_HOST_SPLIT_GROUPS overrides), each copied
 * back on a library-owned copy stream while the next ones sort; the work is
 * ordered after what `stream` already holds.  Smaller arrays are copied in,
 * sorted and copied back on `stream`.  Either way the result is the in-place
 * sort's.  Calls from several threads are safe; their split-path copies share
 * the copy stream and so run one after another. */
size_t gbsort_host_buffer_bytes(int key_type, size_t value_bytes, size_t n);
int gbsort_sort_host(int key_type, int descending, void* h_keys,
                     void* h_values, size_t value_bytes, size_t n,
                     void* d_buffer, size_t buffer_bytes, void* stream);

/* ------------------------------------------------------------------------ */
/* Batched (segmented) sort — no counterpart in the reference (one array per */
/* rsort call).  Thousands of independent sorts of uneven sizes run in a     */
/* few persistent launches: small segments sorted whole in one CTA's shared  */
/* memory, large ones through onesweep passes over one global tile list.     */
/* Segment i is elements [offsets[i], offsets[i+1]) of the key (and value)   */
/* arrays; the arrays must hold fewer than 2^32 elements.                    */
/* ------------------------------------------------------------------------ */

/* Paths a size bucket can take (see gbsort_set_segmented_path). */
enum {
    GBSORT_PATH_CTA_S = 0,    /* whole segment in a 256-thread CTA          */
    GBSORT_PATH_CTA_L = 1,    /* whole segment in a 512-thread CTA          */
    GBSORT_PATH_ONESWEEP = 2, /* onesweep passes over the global tile list  */
    GBSORT_PATH_CTA_S4 = 3    /* as CTA_S with 4-bit digits (16 bins)       */
};

typedef struct gbsort_segmented_plan gbsort_segmented_plan;

typedef struct gbsort_segmented_info {
    uint64_t num_segments;
    uint64_t cta_small_segments;
    uint64_t cta_large_segments;
    uint64_t onesweep_segments;
    uint64_t onesweep_tiles;
    uint64_t keys_in_cta;
    uint64_t keys_in_onesweep;
    uint32_t cta_small_max;   /* largest segment the 256-thread CTA sort takes */
    uint32_t cta_large_max;   /* largest segment the 512-thread CTA sort takes */
    uint32_t onesweep_tile;   /* keys per onesweep tile                        */
    uint32_t pad;
    uint64_t cta_small4_segments; /* segments on the 4-bit-digit CTA sort      */
    uint64_t workspace_bytes;
    uint64_t kernel_launches; /* kernels one run launches (plus one memset)  */
} gbsort_segmented_info;

/* Plan from HOST offsets (num_segments + 1 entries, non-decreasing). */
int gbsort_segmented_plan_create(int key_type, size_t value_bytes,
                                 int descending, const uint64_t* h_offsets,
                                 size_t num_segments,
                                 gbsort_segmented_plan** out);
void gbsort_segmented_plan_destroy(gbsort_segmented_plan* plan);
int gbsort_segmented_plan_info(const gbsort_segmented_plan* plan,
                               gbsort_segmented_info* out);
/* Bind device keys/values and a workspace of >= info.workspace_bytes; uploads
 * the plan's tables into the workspace on `stream`. */
int gbsort_segmented_bind(gbsort_segmented_plan* plan, void* d_keys,
                          void* d_values, void* d_workspace,
                          size_t workspace_bytes, void* stream);
/* Sort every segment in place.  use_graph: the first run captures the launch
 * sequence into a CUDA graph on `stream` (must not be the legacy default
 * stream), later runs replay it; rebinding other buffers drops the graph. */
int gbsort_segmented_run(gbsort_segmented_plan* plan, int use_graph,
                         void* stream);
/* Synchronizes `stream` and reads the plan's device error word. */
int gbsort_segmented_status(gbsort_segmented_plan* plan, void* stream);
/* One-shot form with rsort's protocol: d_workspace == NULL writes the bytes
 * needed to *temp_bytes.  Synchronizes `stream` before returning. */
int gbsort_segmented_sort(int key_type, int descending, void* d_keys,
                          void* d_values, size_t value_bytes,
                          const uint64_t* h_offsets, size_t num_segments,
                          size_t* temp_bytes, void* d_workspace, void* stream);
/* Batched sort of segments in HOST memory (keys, values and offsets on the
 * host; segment i is [h_offsets[i], h_offsets[i+1]) of h_keys): copies in,
 * sorts every segment, copies back, then synchronizes.  Consecutive segments
 * form groups of ~2^24 keys (2 to 16; GBSORT_HOST_SPLIT_GROUPS overrides);
 * a group's keys
 * come in on one library-owned copy stream while the previous group sorts on
 * `stream` and the one before goes back on a second copy stream, so both
 * directions of the host link work at once (pinned memory for full speed).
 * d_buffer (16-byte aligned) holds gbsort_segmented_host_buffer_bytes(...)
 * bytes: the keys and values once plus one group's workspace.  Calls from
 * several threads are safe and run one at a time (they share the library's
 * pinned staging of the groups' tables). */
size_t gbsort_segmented_host_buffer_bytes(int key_type, size_t value_bytes,
                                          const uint64_t* h_offsets,
                                          size_t num_segments);
int gbsort_segmented_sort_host(int key_type, int descending, void* h_keys,
                               void* h_values, size_t value_bytes,
                               const uint64_t* h_offsets, size_t num_segments,
                               void* d_buffer, size_t buffer_bytes,
                               void* stream);
/* Tuning table: the path segments of size [2^size_log2, 2^(size_log2+1))
 * take for this key type and value size (size_log2 = -1: every bucket;
 * path = -1: back to the built-in size thresholds).  A path too small for a
 * segment falls through to the next bigger one.  Plans made afterwards use
 * it. */
int gbsort_set_segmented_path(int key_type, size_t value_bytes, int size_log2,
                              int path);
/* Path a segment of exactly 2^size_log2 keys would take now. */
int gbsort_get_segmented_path(int key_type, size_t value_bytes, int size_log2);
/* The table's explicit entry for the bucket (-1: none, built-in thresholds). */
int gbsort_segmented_path_override(int key_type, size_t value_bytes,
                                   int size_log2);

/* Autotuner: for each size bucket min_log2..max_log2 times every path that
 * can hold segments of that size (4-bit and 8-bit CTA sorts of two tile
 * shapes, onesweep) on synthetic batches built in the caller's device scratch
 * (no allocation; ~(key + value bytes) * 12 MiB covers every bucket up to
 * 2^22), and installs the fastest in the tuning table.  A per-bucket report
 * is written to `report`. */
int gbsort_autotune_segmented(int key_type, size_t value_bytes, int descending,
                              int min_log2, int max_log2, void* d_scratch,
                              size_t scratch_bytes, void* stream, char* report,
                              size_t report_cap);
/* Tuning table as text ("key_type value_bytes size_log2 path" per line);
 * returns the text length.  _load applies such text. */
int gbsort_segmented_tuning_text(char* buf, size_t cap);
int gbsort_segmented_tuning_load(const char* text);

/* ------------------------------------------------------------------------ */
/* Sort server — continuous batching of independent sort requests.  No      */
/* counterpart in the reference.  Requests arrive from any thread; one      */
/* scheduler thread coalesces queued requests of one class (key type, value */
/* size, order) into a batched sort over a contiguous staging area carved   */
/* from one pooled device allocation, admits a batch only when its bytes    */
/* fit the pool, and keeps up to `streams` batches in flight, so the copies */
/* of one batch overlap the sort of another.  A request's buffers may be    */
/* host (pinned for overlap) or device memory; results land in keys_out /   */
/* values_out (which may equal the inputs).                                 */
/* ------------------------------------------------------------------------ */

typedef struct gbsort_server gbsort_server;

typedef struct gbsort_server_config {
    uint64_t pool_bytes;      /* device pool = admission budget (0: 64 GiB)  */
    uint32_t streams;         /* batches in flight (0: 6)                    */
    uint32_t paused;          /* start paused (see gbsort_server_resume)     */
    uint64_t max_batch_keys;  /* keys coalesced into one launch (0: 2^26)    */
    uint64_t max_batch_requests; /* requests per launch (0: 4096)            */
} gbsort_server_config;

typedef struct gbsort_request {
    int key_type;
    int descending;
    size_t value_bytes;       /* 0: keys only                                */
    size_t n;
    const void* keys_in;      /* host or device memory                       */
    const void* values_in;
    void* keys_out;           /* may equal keys_in                           */
    void* values_out;
} gbsort_request;

typedef struct gbsort_server_stats {
    uint64_t submitted, completed, failed, rejected;
    uint64_t batches;
    uint64_t max_batch_requests;
    uint64_t keys_sorted;     /* keys of completed requests                  */
    uint64_t bytes_sorted;    /* key + value bytes of completed requests     */
    uint64_t pool_bytes;
    uint64_t pool_peak_bytes; /* high-water mark of the pool in use          */
    uint64_t kernel_launches; /* kernels launched by the batches             */
    double latency_p50_us, latency_p99_us, latency_mean_us, latency_max_us;
    double queue_p50_us, queue_p99_us; /* submit -> batch launch             */
    double mean_batch_requests;
    double active_seconds;    /* first submit -> last completion             */
    double host_plan_seconds; /* scheduler time forming and sizing batches   */
    double host_launch_seconds; /* scheduler time enqueuing batches          */
    double batch_seconds;     /* sum over batches of launch -> completion    */
    double h2d_seconds;       /* device time of the batches' input copies    */
    double sort_seconds;      /* device time of the batches' sorts           */
    double d2h_seconds;       /* device time of the batches' output copies   */
} gbsort_server_stats;

/* cfg may be NULL (defaults).  Allocates the pool and the streams on the
 * current device. */
int gbsort_server_create(const gbsort_server_config* cfg, gbsort_server** out);
/* Drains every queued and running request, then frees everything. */
void gbsort_server_destroy(gbsort_server* server);
/* Queues one request; *ticket identifies it.  GBSORT_ERR_BUDGET when the
 * request alone needs more device bytes than the pool holds. */
int gbsort_server_submit(gbsort_server* server, const gbsort_request* req,
                         uint64_t* ticket);
/* GBSORT_ERR_NOT_READY while queued or running; otherwise the request's final
 * status, after which the ticket is retired (a second call returns
 * GBSORT_ERR_INVALID_ARGUMENT). */
int gbsort_server_poll(gbsort_server* server, uint64_t ticket);
/* As poll, waiting up to timeout_ns for the request to finish. */
int gbsort_server_wait(gbsort_server* server, uint64_t ticket,
                       uint64_t timeout_ns);
/* Waits until nothing is queued or running (GBSORT_ERR_NOT_READY on timeout). */
int gbsort_server_drain(gbsort_server* server, uint64_t timeout_ns);
/* While paused, requests queue but no batch is launched. */
int gbsort_server_pause(gbsort_server* server);
int gbsort_server_resume(gbsort_server* server);
int gbsort_server_stats_get(gbsort_server* server, gbsort_server_stats* out);
int gbsort_server_stats_reset(gbsort_server* server);

/* ------------------------------------------------------------------------ */
/* Multi-GPU sharding of independent work — no counterpart in the reference */
/* (one GPU).  Segments and requests are independent, so they are split     */
/* across ranks by bytes with no collective and no data exchange: every     */
/* rank computes the same assignment from the same host sizes and sorts only */
/* what it owns.  Greedy longest-processing-time: items by decreasing       */
/* weight, each to the least-loaded rank (ties: lowest index, lowest rank). */
/* Host only; needs no GPU.                                                  */
/* ------------------------------------------------------------------------ */

/* owner_out[i] = rank of item i (num_items entries); rank_load_out (may be
 * NULL) receives the total weight per rank (world entries). */
int gbsort_partition_weights(const uint64_t* weights, size_t num_items,
                             int world, int32_t* owner_out,
                             uint64_t* rank_load_out);
/* Same over the segments of a batched sort: weight of segment i =
 * (offsets[i+1] - offsets[i]) * (key_bytes + value_bytes). */
int gbsort_partition_segments(const uint64_t* h_offsets, size_t num_segments,
                              int world, size_t key_bytes, size_t value_bytes,
                              int32_t* owner_out, uint64_t* rank_bytes_out);

/* ------------------------------------------------------------------------ */
/* Workspace status and bounded waits                                       */
/* ------------------------------------------------------------------------ */

/* Clears the control block (error word, tile counters) of a workspace laid
 * out for (key type, value size, n) on `stream`.  Every sort clears it itself
 * before it starts; this only forgets a recorded error. */
int gbsort_workspace_reset(int key_type, size_t value_bytes, size_t n,
                           void* d_workspace, void* stream);

/* Synchronizes `stream`, then reads the error word the last sort on this
 * workspace left (GBSORT_OK or GBSORT_ERR_TIMEOUT).  Needs the n, key type and
 * value size of that sort to locate the word. */
int gbsort_workspace_status(int key_type, size_t value_bytes, size_t n,
                            void* d_workspace, void* stream);

/* Uniform-digit pass skipping (default on; GBSORT_PASS_SKIP=0 in the
 * environment turns it off at load).  A digit pass in which every key has
 * the same digit leaves the order unchanged, so the sort runs only the other
 * passes: each pass kernel reads the upsweep's digit counts on the device
 * and exits when its digit is uniform, and a final copy kernel moves the
 * result home when an odd number of passes ran.  Nothing synchronizes with
 * the host.  The reference's optional form (EXIT_EARLY_OPT,
 * include/rsort/detail/radix_kernel.cuh:298-323) copies the counts to the
 * host first. */
void gbsort_set_pass_skip(int enable);
int gbsort_get_pass_skip(void);

/* One-launch sort of short keys-only arrays (n <= 2^21, 2^20 for 16-byte
 * keys; no values; plain,
 * input-preserving and DoubleBuffer forms): the digit counts, every pass and
 * the pass-skip fix-up run in one cooperative launch with a grid barrier
 * (bounded wait, GBSORT_ERR_TIMEOUT) between them, instead of one launch per
 * kernel.  The reference's short mode (radix_kernel.cuh:525-559) still
 * launches every kernel.  On by default; GBSORT_SHORT_FUSED=0 in the
 * environment or gbsort_set_short_fused(0) selects the separate launches.
 * Results are identical either way. */
void gbsort_set_short_fused(int enable);
int gbsort_get_short_fused(void);

/* Inside the one-launch short sort (keys of 2 bytes or more): when the
 * top-digit regions fit a CTA's local sort (gbsort_plan_info.msd_region_keys
 * != 0), every tile partitions its keys into them by the most significant
 * digit and each CTA then sorts whole buckets in shared memory — one
 * grid-wide exchange instead of one per digit.  Otherwise (or when switched
 * off: GBSORT_SHORT_MSD=0, gbsort_set_short_msd(0)) every digit takes a
 * pass.  Keys only, so the result is the same bytes either way. */
void gbsort_set_short_msd(int enable);
int gbsort_get_short_msd(void);

/* Keys-only sorts of 8- and 16-byte keys above the short range (1.5 x 2^24
 * to 2^28 keys of 8 bytes, 1.5 x 2^20 to 2^27 of 16): most significant digit
 * first —
 * a split by the top digit, a count of (top, second) digit pairs, a split by
 * the second digit into the 65536 pairs' ranges, and in-place local sorts
 * of those groups in shared memory — instead of one stable pass per key
 * byte (gbsort_plan_info.msd_stages = 6).  When a group outgrows a local
 * sort (skewed or repeated keys), the digit passes sort instead, decided on
 * the device.  The size query reserves the path's ~1 MB either way.  On by
 * default; GBSORT_MSD=0 in the environment or gbsort_set_msd(0) turns it
 * off.  Keys only, so the result is the same bytes either way. */
void gbsort_set_msd(int enable);
int gbsort_get_msd(void);

/* Graph replay of repeated calls (default on; GBSORT_GRAPH_CACHE=0 turns it
 * off at load).  The second call of gbsort_sort_keys / _pairs / _copy with
 * the same buffers, size, key type, order, stream and settings is captured
 * into a CUDA graph, and later identical calls replay it, which removes the
 * gaps between the sort's kernels (what the reference does on every call,
 * include/rsort/detail/radix_kernel.cuh:583-601, without its per-call
 * capture cost).  Nothing is captured on the legacy stream or on a stream
 * the caller is capturing.  The 32 most recently used calls are tracked per
 * process; a new one replaces the least recently used (and its graph).
 * gbsort_graph_cache_clear synchronizes the device and frees them.
 * gbsort_graph_cache_stats: tracked calls, of those the ones holding a graph,
 * and graphs captured and replays launched since load (any pointer may be
 * NULL). */
void gbsort_set_graph_cache(int enable);
int gbsort_get_graph_cache(void);
int gbsort_graph_cache_clear(void);
void gbsort_graph_cache_stats(uint64_t* calls, uint64_t* graphs, uint64_t* captures, uint64_t* replays);

/* Upper bound, in nanoseconds, on any single device-side wait (lookback spin
 * or TMA barrier) of later launches.  Default 2e9 (2 s).  Process-wide. */
void gbsort_set_wait_limit_ns(uint64_t ns);
uint64_t gbsort_get_wait_limit_ns(void);

/* Runs one bounded wait, on the device, on a status word that nothing ever
 * publishes, with the given limit; returns GBSORT_ERR_TIMEOUT when the wait
 * gave up (the expected outcome) and GBSORT_OK otherwise.  d_scratch must
 * point to 64 bytes of device memory.  Exercises the failure path of the
 * lookback without stalling any sort. */
int gbsort_probe_wait_timeout(void* d_scratch, uint64_t limit_ns,
                              void* stream);

/* Runs the grid barrier of the one-launch short sort, on the device, where
 * the second arrival it waits for never comes, with the given limit; returns
 * GBSORT_ERR_TIMEOUT when the wait gave up (the expected outcome) and
 * GBSORT_OK otherwise.  d_scratch must point to 64 bytes of device memory.
 * Exercises that barrier's failure path without stalling any sort. */
int gbsort_probe_barrier_timeout(void* d_scratch, uint64_t limit_ns,
                                 void* stream);

/* ------------------------------------------------------------------------ */
/* Result checks on the device (the reference's post-sort checks,           */
/* benchmark/benchmark_sort.cuh:26-175: order, counts, pairs).  Each runs on */
/* `stream`, synchronizes it and allocates 8 device bytes stream-ordered.   */
/* ------------------------------------------------------------------------ */

/* Adjacent pairs out of order, compared as the sort orders keys. */
int gbsort_check_order(int key_type, int descending, const void* d_keys,
                       size_t n, void* stream, uint64_t* violations);
/* Order-independent 64-bit checksum of n keys: equal for any permutation. */
int gbsort_checksum(int key_type, const void* d_keys, size_t n, void* stream,
                    uint64_t* sum);
/* Values that hold each key's original index (4 or 8 bytes): counts output
 * positions i whose d_keys_in[index[i]] differs from d_keys_out[i]. */
int gbsort_check_pairs(int key_type, const void* d_keys_in,
                       const void* d_keys_out, const void* d_index_values,
                       size_t value_bytes, size_t n, void* stream,
                       uint64_t* violations);

/* ------------------------------------------------------------------------ */
/* Introspection used by the benchmark                                      */
/* ------------------------------------------------------------------------ */

/* Geometry the plain sort picks for (key type, value size, n). */
typedef struct gbsort_plan_info {
    uint32_t passes;          /* digit passes (key bytes)                    */
    uint32_t radix_bits;      /* bits per digit (8)                          */
    uint32_t tile_items;      /* keys per tile                               */
    uint32_t threads;         /* threads per CTA of the pass kernel          */
    uint32_t items_per_thread;
    uint32_t num_tiles;
    uint32_t pass_ctas;       /* persistent CTAs of the pass kernel          */
    uint32_t hist_ctas;       /* CTAs of the histogram kernel                */
    uint32_t status_word_bytes; /* 4 or 8                                    */
    uint32_t kernel_launches; /* launches (plus one memset node) per sort;
                                 1 when a short array sorts in one launch     */
    uint64_t workspace_bytes;
    uint32_t msd_region_keys; /* one-launch sort, most significant digit
                                 first: keys per top-digit region of its
                                 partition (each key read and written twice);
                                 0: every digit takes a pass                  */
    uint32_t msd_stages;      /* keys-only sorts of 8- and 16-byte keys above
                                 the short range, most significant digit
                                 first: 6 kernels (top split, pair count,
                                 scan, second split, local sorts, and the
                                 histogram of the other digits) run after the
                                 top digit's histogram kernel and before the
                                 digit passes; those and the last histogram
                                 exit at once unless a group was too big;
                                 0: not planned                              */
} gbsort_plan_info;

int gbsort_plan(int key_type, size_t value_bytes, size_t n,
                gbsort_plan_info* out);

/* Same as gbsort_sort_pairs (d_values may be NULL with value_bytes 0), but
 * records a CUDA event around every kernel on `stream` and, after
 * synchronizing, writes the per-kernel device milliseconds to ms_out:
 * ms_out[0] = histogram kernel, then with the MSD path planned
 * (gbsort_plan_info.msd_stages = S = 6) ms_out[1 .. S] = its kernels (top
 * split, pair count, scan, second split, local sorts, histogram of the other
 * digits), then
 * ms_out[1 + S + p] = digit pass p (S = 0 otherwise), and with pass skipping
 * on and an even pass count P, ms_out[1 + S + P] = the fix-up copy.  A short
 * array sorted in one launch (gbsort_set_short_fused) writes one entry, the
 * whole sort.  ms_cap is the capacity of ms_out; *n_ms receives the number
 * of entries written. */
int gbsort_sort_timed(int key_type, int descending, void* d_keys,
                      void* d_values, size_t value_bytes, void* d_workspace,
                      size_t temp_bytes, size_t n, void* stream,
                      float* ms_out, int ms_cap, int* n_ms);

/* Fills d_out with n synthetic keys on the device (seeded, deterministic):
 *   dist 0: splitmix64 stream, full-range bits of the key width
 *   dist 1: float32 N(0,1) with 1% -0.0, 0.1% +/-inf, 0.01% quiet NaN
 *   dist 2: uint64, upper 32 bits from 256 distinct values, lower uniform
 *   dist 3: ascending index values (key i = i)
 *   dist 4: rsort init_keys "random" mode (mix32 of i ^ seed)
 *   dist 5: rsort init_keys "byte_skip" mode
 * key_bytes is the width written (1, 2, 4, 8 or 16). */
int gbsort_generate(int dist, size_t key_bytes, void* d_out, size_t n,
                    uint64_t seed, void* stream);

/* Number of SMs of the current device, 0 without a device. */
int gbsort_device_sm_count(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* GBSORT_H */
