/*
 * rmq.h -- C ABI of the GB300 batch range-minimum-query engine.
 *
 * One data-parallel path: answer q inclusive, 0-based queries (l, r) over a
 * float32 array A[0..n) with
 *     val = min A[l..r]                      (bit pattern of A[idx])
 *     idx = smallest i in [l, r] with A[i] == val   (float `<`, leftmost tie)
 * which is the semantics of the reference's CPU/GPU BASE oracles
 * (src/cpu_methods.h:42-53, src/cuda_methods.cuh:23-42) and of its
 * block-decomposition ray-tracing path RTX_blocks (alg 5 / 105,
 * src/rtx_kernels.cu:85-193 and 350-465).
 *
 * Conventions
 *  - Every pointer named d_* is device memory, h_* is host memory.
 *  - Queries are int32 pairs {l, r} (the reference's int2), 8-byte aligned.
 *  - All calls are stream ordered; none synchronises the device unless its
 *    comment says so. rmq_query never allocates.
 *  - Every call returns RMQ_OK (0) or a negative status; nothing exits or
 *    prints. rmq_last_error_string() describes the last failure of the
 *    calling thread.
 *  - NaN is outside the supported input domain. NaN elements order above
 *    +inf and are returned (as a canonical quiet NaN) only when a range holds
 *    nothing else; -0.0 and +0.0 compare equal, as with float `<`.
 */
#ifndef RTXRMQ_GB300_RMQ_H
#define RTXRMQ_GB300_RMQ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same type as cudaStream_t; NULL means the legacy default stream. */
typedef struct CUstream_st *rmq_stream_t;

/* status codes */
#define RMQ_OK        0
#define RMQ_EINVAL   (-1)  /* bad argument (size, alignment, null pointer) */
#define RMQ_ENOMEM   (-2)  /* device or host allocation failed            */
#define RMQ_ECUDA    (-3)  /* a CUDA runtime call failed                  */
#define RMQ_ENOTSUP  (-5)  /* algorithm or mode not available             */
/* (-4) is not used: no call of this library waits on the device with a
 * time limit (the batched kernel's phase barriers are grid syncs of a
 * cooperative launch, whose CTAs are all resident). */

/* Default block size when bs <= 0: 2^15, as the reference CLI
 * (src/tools.h:96). */
#define RMQ_DEFAULT_BS (1 << 15)

typedef struct rmq_handle rmq_handle_t;

typedef struct rmq_info {
    int64_t n;            /* elements                                   */
    int64_t bs;           /* block size                                 */
    int64_t nb;           /* blocks = ceil(n / bs)  (src/rtx.h:42)      */
    int32_t levels;       /* sparse-table levels over the block minima  */
    int32_t aligned;      /* 1 when d_vals is 16-byte aligned           */
    int64_t table_bytes;  /* sparse table (block minima and levels)     */
    int64_t struct_bytes; /* all device memory owned by the handle      */
    int32_t micro_levels; /* levels of the sub-block table (0 = none)   */
    int32_t light;        /* 1: light index (RMQ_BUILD_LIGHT)           */
    int64_t micro_table_bytes; /* micro-block minima + table offsets     */
    int32_t is_max;       /* 1: range maximum (RMQ_BUILD_MAX)           */
    int32_t is_int32;     /* 1: int32 elements (RMQ_BUILD_INT32)        */
} rmq_info_t;

/* rmq_build_ex flags */
#define RMQ_BUILD_NO_MICRO 1u  /* no sub-block level: same-block queries are
                                  answered by warp-cooperative scans */
#define RMQ_BUILD_MAX      2u  /* range MAXIMUM (leftmost on ties) instead of
                                  minimum; NaN still never wins */
#define RMQ_BUILD_INT32    4u  /* d_vals holds int32 elements (pass the int32
                                  buffer cast to const float *); the value
                                  outputs of rmq_query then receive the int32
                                  bits (pass an int32 buffer cast to float *).
                                  The role of HRMQ's integer constructors,
                                  hrmq/includes/RMQRMM64.h:175-178 */
#define RMQ_BUILD_LIGHT    8u  /* light index: the block and micro-block
                                  tables only, no per-element prefix /
                                  suffix entries (about 1.3 instead of 32
                                  bytes per element, a build that reads the
                                  values once and writes ~1/25 as much); a
                                  query the table probe leaves open scans
                                  one 128-byte line of values per end
                                  instead of reading an entry. Needs the
                                  sub-block level and bs a multiple of 32,
                                  >= 64 (bs > n is rounded up to one block).
                                  No counterpart in the reference. */

/*
 * Build the index over d_vals[0..n) with block size bs (bs <= 0: default).
 * Replaces the construction half of rtx_rmq<T>() (src/rtx.h:24-99): the
 * per-block minimum (kernel_min_blocks, src/device_tools.cuh:243-253), the
 * per-block leftmost argmin (compute_min_blocks, src/rtx.h:3-22) and the
 * geometry + BVH build (src/device_tools.cuh:139-169, 378-389,
 * src/rtx_functions.h:289-379) become in-block prefix/suffix minima and a
 * sparse table over the block minima.
 * The handle owns its structure memory; it does not own or copy d_vals,
 * which must stay valid and unchanged while the handle is used.
 * Allocates (cudaMalloc); not for use under stream capture.
 */
int rmq_build(const float *d_vals, int64_t n, int64_t bs, rmq_stream_t stream,
              rmq_handle_t **out);

/*
 * rmq_build with options. When bs >= 64 the index
 * also gets a sub-block level -- prefix and suffix minima inside 32-element
 * micro-blocks (16 more bytes per element) and a sparse table over the
 * micro-block minima, truncated to windows no longer than one block and
 * stored as 1-4 byte offsets to each window's best micro-block (small
 * enough to stay in L2). A query spanning at most about two blocks is then
 * answered from that table: usually from its table words alone, otherwise
 * with one or two per-element entries (one 128-byte line of values if it
 * lies inside one micro-block), never by scanning A[l..r].
 * RMQ_BUILD_NO_MICRO leaves it out.
 * rmq_build(...) is rmq_build_ex(..., 0, ...).
 */
int rmq_build_ex(const float *d_vals, int64_t n, int64_t bs, uint32_t flags,
                 rmq_stream_t stream, rmq_handle_t **out);

/*
 * Answer q queries d_queries[2*i] = l, d_queries[2*i+1] = r.
 * d_val (float[q]) and d_idx (int32[q]) may each be NULL, not both:
 * value mode is alg 5, index mode is alg 105 (src/main.cu:132-137,
 * src/rtx.h:150-159); both may be requested in one call.
 * Replaces the timed optixLaunch loop body (src/rtx.h:150-154) and the ray
 * programs __raygen__rmq_blocks / __closesthit__rmq_blocks
 * (src/rtx_kernels.cu:85-193) and their _idx variants (350-465).
 * An invalid query (l < 0, r >= n or l > r) yields idx = -1, val = NaN
 * and is counted (rmq_invalid_count). No allocation; the handle is not
 * modified except for that counter, so concurrent calls on different
 * streams are safe.
 */
int rmq_query(const rmq_handle_t *h, const int32_t *d_queries, int64_t q,
              float *d_val, int32_t *d_idx, rmq_stream_t stream);

/*
 * rmq_query with host-side buffers (h_queries, h_val, h_idx in host memory;
 * device pointers are used as they are). When the GPU can address every
 * buffer -- page-locked memory (cudaHostAlloc, cudaHostRegister), or any
 * host memory on systems where the device reads pageable memory
 * (Grace-Blackwell) -- the query kernel reads the queries and writes the
 * results in place over the host link (NVLink-C2C on GB300), with no staging
 * copies and no allocation. Otherwise the work is staged through device
 * memory in 4 Mi-query chunks on three internal streams (queries copied in,
 * chunk kernels, results copied out while later chunks run; addressable
 * buffers stay in place); that path allocates its staging (192 MB), streams
 * and events on its first call on a handle, all or nothing.
 * Stream ordered with respect to `stream`: the results are in the host
 * buffers once `stream` has been synchronised. Calls on one handle from
 * several threads or streams are safe: on the staged path their enqueueing
 * is serialised and a staging slot is reused only after the kernel and the
 * copies of its previous chunk, whichever call and stream that was on. This
 * is the end-to-end
 * form of the reference's timed loop plus its copy-out (src/rtx.h:150-159).
 *
 * Environment switches read by the library:
 *   RTXRMQ_HOST_STAGED=1  every rmq_query_host buffer through staging
 *   RTXRMQ_HOST_MODE=<m>  addressable host buffers through staging anyway:
 *                         bit 0 the results, bit 1 the queries
 *   RTXRMQ_FAIL_ALLOC=1   every device allocation of the library fails as
 *                         out-of-memory (host-side fault injection for tests)
 *   RTXRMQ_NVML_LIBRARY   path of the NVML library the power sampler opens
 */
int rmq_query_host(const rmq_handle_t *h, const int32_t *h_queries, int64_t q,
                   float *h_val, int32_t *h_idx, rmq_stream_t stream);

/*
 * Build + query of one array in one call that allocates nothing. No
 * counterpart in the reference: it exists for callers that may not allocate
 * device memory (a host framework that owns all device memory through its
 * own pool, or a latency-critical loop that cannot take the implicit
 * device-wide synchronisation of cudaMalloc / cudaFree). The index is built
 * into a fixed device array inside this library (RMQ_NOALLOC_SCRATCH_BYTES,
 * held on every GPU that loads the library until the process exits) and the
 * queries are answered from it; the caller passes inputs and outputs as for
 * rmq_build + rmq_query, with the same results. Sizes whose index does not
 * fit are rejected with RMQ_EINVAL (any n <= 2^20 fits for bs >= 16).
 * The first call on a device, and the first after the device's context was
 * reset (cudaDeviceReset), looks up the array's device address (set-up),
 * so make that call before any stream capture. All calls share the
 * array: calls whose work overlaps on the GPU race.
 */
#define RMQ_NOALLOC_SCRATCH_BYTES (32u << 20)
int rmq_query_noalloc(const float *d_vals, int64_t n, int64_t bs,
                      const int32_t *d_queries, int64_t q, float *d_val,
                      int32_t *d_idx, rmq_stream_t stream);

/*
 * Persisted index, the role of HRMQ's saveDS / loadDS
 * (hrmq/RMQRMM64.cpp:1471-1659). rmq_save writes a header (layout sizes and
 * a 64-bit fingerprint of all the values, computed on the GPU) and the
 * handle's device structure to `path`; the values themselves are not stored.
 * rmq_load recreates the handle for d_vals[0..n), which must be the values
 * the index was built from: a different length, layout or fingerprint, a
 * truncated or foreign file give RMQ_EINVAL. Both synchronise `stream` and
 * use a temporary device word for the fingerprint.
 */
int rmq_save(const rmq_handle_t *h, const char *path, rmq_stream_t stream);
int rmq_load(const float *d_vals, int64_t n, const char *path,
             rmq_stream_t stream, rmq_handle_t **out);

/* Release everything the handle owns. NULL is accepted. */
int rmq_free(rmq_handle_t *h);

/* Describe a built handle. */
int rmq_info(const rmq_handle_t *h, rmq_info_t *info);

/* Number of invalid queries seen by this handle so far. Synchronises
 * `stream` before reading. */
int rmq_invalid_count(const rmq_handle_t *h, rmq_stream_t stream,
                      int64_t *count);

/* Message for the last failing call on this thread ("" when none). */
const char *rmq_last_error_string(void);

/* Library version string. */
const char *rmq_version(void);

/*
 * Block size from a block count, as the reference's --nb flag
 * (src/tools.h:129-132): bs = n / min(n, nb) with integer division; the
 * block count actually used is then ceil(n / bs) (src/rtx.h:42).
 */
int rmq_bs_from_nb(int64_t n, int64_t nb, int64_t *bs);

/*
 * GPU brute force, one thread per query scanning A[l..r] with strict `<`
 * (alg 2 / 102). Replaces kernel_rmq_basic / kernel_rmq_basic_idx and
 * gpu_rmq_basic (src/cuda_methods.cuh:3-66, 137-169), which the reference
 * uses as its --check oracle (src/main.cu:140-167).
 */
int rmq_query_scan(const float *d_vals, int64_t n, const int32_t *d_queries,
                   int64_t q, float *d_val, int32_t *d_idx,
                   rmq_stream_t stream);

/*
 * Measurement helper, no reference counterpart: the random-access ceiling
 * of rmq_query on this index. One launch with rmq_query's grid, query
 * stream and output stores, but per query only the two random 8-byte
 * lookups of its cross-block case (suffix minimum at l, prefix minimum at r)
 * and no other work. The outputs are better(suf[l], pre[r]), which is the
 * range minimum only when l and r lie in the same or in adjacent blocks;
 * out-of-range l / r are clamped into the array. A benchmark times it
 * beside rmq_query to state the fraction of this ceiling a query reaches.
 */
int rmq_probe_gather(const rmq_handle_t *h, const int32_t *d_queries, int64_t q,
                     float *d_val, int32_t *d_idx, rmq_stream_t stream);

/*
 * Measurement helper, no reference counterpart: rmq_query (same arguments,
 * same results; d_val and d_idx may both be NULL here) through an
 * instantiation of the query kernel that also counts how every query was
 * settled and what it read, into h_counts[RMQ_QUERY_STATS_FIELDS]:
 *   [0] settled by the probe of the small table over every unit (block or
 *       32-element micro-block) the query touches: the best of that
 *       superset lay inside [l, r]
 *   [1] settled by a narrower probe plus one per-element entry
 *   [2] the three-part decomposition (two entries, probe of the middle)
 *   [3] inside one micro-block: one thread scans it
 *   [4] inside one block without the sub-block level: an edge entry
 *   [5] inside one block without the sub-block level: warp scan
 *   [6] per-element entries read (random 8-byte HBM lookups)
 *   [7] small-table words read (L2-resident probes)
 *   [8] 32-byte sectors of the values read by scans
 *   [9] invalid queries
 * Synchronises `stream`. Uses the handle's counter block, so concurrent
 * rmq_query_stats calls on one handle race (rmq_query does not).
 */
#define RMQ_QUERY_STATS_FIELDS 10
int rmq_query_stats(const rmq_handle_t *h, const int32_t *d_queries, int64_t q,
                    float *d_val, int32_t *d_idx, int64_t *h_counts,
                    rmq_stream_t stream);

/*
 * Measurement helper, no reference counterpart: the random-access rate of
 * the GPU for this query stream, independent of any index layout. One
 * launch with rmq_query's grid, query stream and output stores, and per
 * query two 8-byte loads at positions hashed from (query number, l, r),
 * uniform over d_buf[0 .. words). The outputs carry the loaded words, not
 * range minima. Queries are read but not validated.
 */
int rmq_probe_random(const uint64_t *d_buf, int64_t words, const int32_t *d_queries,
                     int64_t q, float *d_val, int32_t *d_idx, rmq_stream_t stream);

/*
 * Checked builds only, no reference counterpart (the library compiled with
 * -DRMQ_CHECKED=1, a stand-in for a memory sanitizer): the number of
 * out-of-range global accesses the kernels caught and skipped since the
 * library was loaded. RMQ_ENOTSUP (count 0) in normal builds.
 */
int rmq_checked_violations(int64_t *count);

/* ------------------------------------------------------------------------
 * Batched ragged form: many independent arrays of uneven length, each with
 * its own queries, built and answered by ONE persistent cooperative kernel
 * launch (no allocation per run, so a run can be captured in a CUDA graph).
 * The reference has no batched form: rtx_rmq<T> (src/rtx.h:24-177) serves
 * one array per call; rmq_batch_run_per_array is that plain path, one build
 * and one query launch sequence per array, over the same plan.
 *
 * Array i holds d_vals[h_starts[i] .. h_starts[i] + h_lengths[i]) and owns
 * the queries d_queries[h_qstarts[i] .. h_qstarts[i] + h_qcounts[i]) (int32
 * pairs in array-local coordinates); outputs are written at the queries'
 * positions, indices array-local. Arrays and query ranges may sit anywhere
 * in their buffers (gaps allowed). An array may be empty (length 0): it has
 * no structure, and every query it owns is invalid (index -1, value NaN,
 * the bits 0x7fc00000 in an int32 plan, counted by rmq_batch_invalid_count).
 * Arrays are grouped into size buckets floor(log2 length);
 * h_bucket_bs[bucket] (RMQ_BATCH_BUCKETS entries, or NULL; <= 0 means the
 * default: 64 below 2^17 elements, 256 above; 4096 for a light plan) is
 * the block size of that bucket, as chosen by rmq_batch_autotune.
 * ---------------------------------------------------------------------- */
#define RMQ_BATCH_BUCKETS 32

typedef struct rmq_batch rmq_batch_t;

typedef struct rmq_batch_info {
    int32_t narrays;
    int32_t max_levels;
    int64_t values_span;      /* one past the last value any array uses   */
    int64_t queries_span;     /* one past the last query any array owns   */
    int64_t workspace_bytes;  /* prefix/suffix minima and sparse tables   */
    int64_t device_bytes;     /* all device memory owned by the plan      */
    int32_t build_items;
    int32_t query_items;
    int32_t bucket_bs[RMQ_BATCH_BUCKETS];
    int32_t flags;            /* the plan's rmq_batch_create_ex flags     */
} rmq_batch_info_t;

/* Plan a batch (host metadata in, device workspace allocated here). */
int rmq_batch_create(int32_t narrays, const int64_t *h_starts,
                     const int64_t *h_lengths, const int64_t *h_qstarts,
                     const int64_t *h_qcounts, const int32_t *h_bucket_bs,
                     rmq_batch_t **out);

/*
 * Block size and tile schedule of one size bucket: the plan cuts each array
 * of the bucket into query items of query_chunk queries (the unit of work a
 * CTA takes in the query phase) and each sparse-table level into items of
 * level_chunk entries (the unit of the table phase). Values <= 0 mean the
 * defaults (bs as rmq_batch_create, 2048 queries, 4096 entries). The
 * reference has no batched form, so no counterpart.
 */
typedef struct rmq_batch_tile {
    int32_t bs;
    int32_t query_chunk;
    int32_t level_chunk;
    int32_t reserved;
} rmq_batch_tile_t;

/* rmq_batch_create with a tile per bucket (h_bucket_tiles: RMQ_BATCH_BUCKETS
 * entries, or NULL for the defaults) and build flags for every array of the
 * plan: RMQ_BUILD_INT32 (d_vals holds int32 and the value outputs are int32),
 * RMQ_BUILD_MAX (range maximum), RMQ_BUILD_LIGHT (light index per array:
 * block and micro-block tables only; block sizes multiples of 32 and >= 64,
 * default 4096; an array shorter than its block size gets one block of its
 * length rounded up to a multiple of 32, at least 64). Other flags:
 * RMQ_EINVAL. rmq_batch_create(..., bs, out) is this call with tiles
 * {bs[b], 0, 0, 0} and flags 0. */
int rmq_batch_create_ex(int32_t narrays, const int64_t *h_starts,
                        const int64_t *h_lengths, const int64_t *h_qstarts,
                        const int64_t *h_qcounts,
                        const rmq_batch_tile_t *h_bucket_tiles, uint32_t flags,
                        rmq_batch_t **out);

/* The plan's tile per bucket (RMQ_BATCH_BUCKETS entries, defaults filled in). */
int rmq_batch_tiles(const rmq_batch_t *b, rmq_batch_tile_t *h_bucket_tiles);

/* Build every array and answer every query: one cooperative launch. */
int rmq_batch_run(rmq_batch_t *b, const float *d_vals,
                  const int32_t *d_queries, float *d_val, int32_t *d_idx,
                  rmq_stream_t stream);

/*
 * The two halves of rmq_batch_run, for arrays that stay the same while the
 * queries change: rmq_batch_build builds every array's index in the plan's
 * workspace (one cooperative launch, phases build + tables);
 * rmq_batch_query answers the plan's queries from that index (one
 * cooperative launch, query phase only). rmq_batch_query needs a build
 * (rmq_batch_build or rmq_batch_run) enqueued earlier on the same d_vals
 * (RMQ_EINVAL otherwise); the values must not change in between. Both
 * allocate nothing and can be captured in a CUDA graph.
 */
int rmq_batch_build(rmq_batch_t *b, const float *d_vals, rmq_stream_t stream);
int rmq_batch_query(rmq_batch_t *b, const float *d_vals, const int32_t *d_queries,
                    float *d_val, int32_t *d_idx, rmq_stream_t stream);

/* The same results through the plain path: per array one rmq_build-style
 * launch sequence and one rmq_query-style launch (comparison baseline). */
int rmq_batch_run_per_array(rmq_batch_t *b, const float *d_vals,
                            const int32_t *d_queries, float *d_val,
                            int32_t *d_idx, rmq_stream_t stream);

/*
 * Backward of the batched range-min: d_grad_vals[start(i) + d_idx[q]] +=
 * d_grad_out[q] for every query q of array i (fp32 atomics, so the order of
 * additions is not deterministic). accumulate == 0 zeroes
 * d_grad_vals[0 .. values_span) first. Indices < 0 (invalid queries) are
 * skipped. No allocation. RMQ_EINVAL for a plan of int32 values.
 */
int rmq_batch_scatter_grad(const rmq_batch_t *b, const int32_t *d_idx,
                           const float *d_grad_out, float *d_grad_vals,
                           int32_t accumulate, rmq_stream_t stream);

int rmq_batch_info(const rmq_batch_t *b, rmq_batch_info_t *info);
/* Invalid queries seen by this plan; synchronises `stream`. */
int rmq_batch_invalid_count(const rmq_batch_t *b, rmq_stream_t stream,
                            int64_t *count);
int rmq_batch_free(rmq_batch_t *b);

/*
 * Per-size-bucket block-size autotuner: for every bucket present, times a
 * batch of that bucket's arrays and queries with each candidate block size
 * (64 .. 65536, up to twice the bucket's largest length) over `reps` runs
 * and writes the fastest to h_bucket_bs[bucket] (0 for absent buckets).
 * Uses d_val / d_idx as scratch outputs; allocates and frees temporary plans.
 */
int rmq_batch_autotune(int32_t narrays, const int64_t *h_starts,
                       const int64_t *h_lengths, const int64_t *h_qstarts,
                       const int64_t *h_qcounts, const float *d_vals,
                       const int32_t *d_queries, float *d_val, int32_t *d_idx,
                       int32_t reps, rmq_stream_t stream,
                       int32_t *h_bucket_bs);

/*
 * rmq_batch_autotune over the whole tile: per bucket present, first the
 * block size (as rmq_batch_autotune; for a light plan 4096, 1024 or 16384,
 * another than 4096 only when it is more than 3% faster), then with it the
 * query-item size
 * (512 .. 8192 queries) and then the level-item size (1024 .. 16384
 * entries), each the fastest over `reps` runs of a plan holding only that
 * bucket's arrays, built with `flags` (as rmq_batch_create_ex); absent
 * buckets get {0, 0, 0, 0}. Allocates and frees temporary plans; d_val /
 * d_idx are scratch outputs.
 */
int rmq_batch_autotune_ex(int32_t narrays, const int64_t *h_starts,
                          const int64_t *h_lengths, const int64_t *h_qstarts,
                          const int64_t *h_qcounts, const float *d_vals,
                          const int32_t *d_queries, float *d_val,
                          int32_t *d_idx, int32_t reps, rmq_stream_t stream,
                          uint32_t flags, rmq_batch_tile_t *h_bucket_tiles);

/*
 * GPU power sampling around a timed region, the role of the reference's
 * GPUPowerBegin / GPUPowerEnd (common/nvmlPower.cpp:91-167, used around the
 * timed loop at src/rtx.h:148-158). A thread reads the board power of CUDA
 * device `device` through NVML every sample_ms and, when `path` is given,
 * writes the reference's table (#timestep power acc-energy avg-power dt
 * acc-time). cooldown_ms is slept after starting / before stopping (the
 * reference uses 1000 ms). NVML is loaded at run time and only read;
 * RMQ_ENOTSUP when it is not available. One sampler at a time.
 */
int rmq_power_begin(int32_t device, int32_t sample_ms, int32_t cooldown_ms,
                    const char *path);
int rmq_power_end(int32_t cooldown_ms, double *avg_watts, double *energy_joules,
                  double *seconds);

/*
 * Host-side synthetic inputs (OpenMP; the output does not depend on the
 * thread count, unlike the reference's per-thread mt19937(seed*tid)
 * streams, src/rand.cuh:120-173).
 *
 * rmq_gen_values_uniform: h_out[i] uniform in [0,1) with 24-bit resolution,
 *   the role of create_random_array_dev (src/rand.cuh:23-43).
 * rmq_gen_values_normal: h_out[i] ~ N(mean, stddev), rounded to float32.
 * rmq_gen_values_int: h_out[i] = integer uniform in [0, range) as float.
 * rmq_gen_queries: q pairs {l, r} over [0, n) with the reference's length
 *   modes (src/rand.cuh:179-201): lr > 0 fixed length lr; -1 uniform length
 *   in [1, n]; -2 lognormal(mu = 0.6 ln n, 0.3); -3 lognormal(0.3 ln n, 0.3);
 *   -4 lognormal(ln max(1, n/2^8), 0.3); -5 lognormal(ln max(1, n/2^15), 0.3).
 *   Lognormal lengths are rounded to nearest and clamped to [1, n];
 *   l is uniform in [0, n - len], r = l + len - 1.
 * rmq_gen_queries_lognormal: the same with explicit mu and sigma.
 */
int rmq_gen_values_uniform(float *h_out, int64_t n, uint64_t seed);
int rmq_gen_values_normal(float *h_out, int64_t n, double mean, double stddev,
                          uint64_t seed);
int rmq_gen_values_int(float *h_out, int64_t n, int32_t range, uint64_t seed);
int rmq_gen_queries(int32_t *h_out, int64_t q, int64_t n, int32_t lr,
                    uint64_t seed);
int rmq_gen_queries_lognormal(int32_t *h_out, int64_t q, int64_t n, double mu,
                              double sigma, uint64_t seed);

#ifdef __cplusplus
}
#endif
#endif /* RTXRMQ_GB300_RMQ_H */
