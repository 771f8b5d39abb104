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
#define RMQ_ETIMEOUT (-4)  /* a bounded device wait expired               */
#define RMQ_ENOTSUP  (-5)  /* algorithm or mode not available             */

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
} rmq_info_t;

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
