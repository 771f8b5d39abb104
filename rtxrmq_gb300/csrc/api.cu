// api.cu -- the exported C ABI (include/rmq.h): argument checks, memory
// ownership and error reporting around the kernels in build.cu / query.cu.
//
// Error behaviour differs from the reference on purpose: its CUDA_CHECK /
// OPTIX_CHECK print and carry on (common/common.h:57-69) and HRMQ calls
// exit() (hrmq/RMQRMM64.cpp:237-240); here every failure is a status code
// plus a per-thread message.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "../../include/rmq.h"
#include "engine.h"

struct rmq_handle {
    rmq::BuildPlan plan;
    int device;
    void *mem;                      // single allocation holding everything below
    size_t mem_bytes;
    unsigned long long *invalid;    // device counter of rejected queries
    int64_t table_bytes;
    // rmq_query_host pipeline, created on its first call: device staging for
    // kHostStreams chunks (queries in, values and indices out), its streams
    // and events, and a lock that keeps concurrent calls from interleaving
    // their chunks on the shared staging buffers
    std::mutex *host_mu;
    void *stage;
    cudaStream_t hs;           // query copies into staging
    cudaStream_t ks;           // chunk kernels, in order
    cudaStream_t cs;           // result copies, each after its chunk's kernel
    cudaEvent_t ev_start;
    cudaEvent_t h_done[3];     // per staging slot: queries copied in
    cudaEvent_t k_done[3];     // per staging slot: kernel finished
    cudaEvent_t c_done[3];     // per staging slot: results copied out
    cudaEvent_t ev_end;
    // per staging slot: used by an earlier chunk (of this call or an earlier
    // one, whatever stream it was on), so its next use waits for that
    // chunk's kernel and copy-out
    bool slot_used[3];
};

namespace {
constexpr int kHostStreams = 3;
static_assert(sizeof(rmq_handle::slot_used) / sizeof(bool) == kHostStreams,
              "one slot flag per staging slot");
constexpr int64_t kHostChunk = int64_t(1) << 22;  // queries per staged chunk (64 MB of staging)
// rmq_query_stats' counters: words kStatsSlot .. kStatsSlot + RMQ_QUERY_STATS_FIELDS
// of the handle's 256-byte counter block (word 0 counts invalid queries)
constexpr int kStatsSlot = 8;
static_assert((kStatsSlot + RMQ_QUERY_STATS_FIELDS) * 8 <= 256, "stats fit the counter block");
}  // namespace

namespace rmq {

static thread_local char g_err[512] = "";

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t err, const char *what) {
    return set_error(err == cudaErrorMemoryAllocation ? RMQ_ENOMEM : RMQ_ECUDA, "%s: %s (%s)",
                     what, cudaGetErrorName(err), cudaGetErrorString(err));
}

int device_info(DeviceInfo *out) {
    static std::mutex mu;
    static DeviceInfo cache[64];
    static bool have[64] = {false};
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return cuda_fail(err, "cudaGetDevice");
    if (dev < 0 || dev >= 64) return set_error(RMQ_ENOTSUP, "device ordinal %d unsupported", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!have[dev]) {
        DeviceInfo d;
        d.device = dev;
        int v = 0;
        err = cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        if (err != cudaSuccess) return cuda_fail(err, "cudaDeviceGetAttribute(SMs)");
        d.sms = v;
        err = cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev);
        if (err != cudaSuccess) return cuda_fail(err, "cudaDeviceGetAttribute(L2)");
        d.l2_bytes = static_cast<size_t>(v);
        cache[dev] = d;
        have[dev] = true;
    }
    *out = cache[dev];
    return RMQ_OK;
}

}  // namespace rmq

using namespace rmq;

namespace rmq {

int handle_view(const rmq_handle *h, BuildPlan *plan, void **mem, size_t *bytes) {
    if (!h) return set_error(RMQ_EINVAL, "handle is NULL");
    *plan = h->plan;
    *mem = h->mem;
    *bytes = h->mem_bytes;
    return RMQ_OK;
}

int handle_adopt(BuildPlan plan, void *mem, size_t bytes, cudaStream_t stream, rmq_handle **out) {
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    rmq_handle_t *h = new (std::nothrow) rmq_handle_t;
    if (!h) return set_error(RMQ_ENOMEM, "host allocation failed");
    std::memset(h, 0, sizeof(*h));
    h->host_mu = new (std::nothrow) std::mutex;
    if (!h->host_mu) {
        delete h;
        return set_error(RMQ_ENOMEM, "host allocation failed");
    }
    h->device = dev.device;
    h->mem = mem;
    h->mem_bytes = bytes;
    h->invalid = place_index(plan, mem);
    h->table_bytes = static_cast<int64_t>(sizeof(Entry) * static_cast<size_t>(plan.nb) * plan.levels);
    h->plan = plan;
    cudaError_t err = cudaMemsetAsync(h->invalid, 0, sizeof(unsigned long long), stream);
    if (err != cudaSuccess) {
        delete h->host_mu;
        delete h;
        return cuda_fail(err, "clear counter");
    }
    *out = h;
    return RMQ_OK;
}

}  // namespace rmq

extern "C" {

const char *rmq_last_error_string(void) { return g_err; }

const char *rmq_version(void) { return "rtxrmq_gb300 0.1 (sm_103a)"; }

int rmq_bs_from_nb(int64_t n, int64_t nb, int64_t *bs) {
    g_err[0] = '\0';
    if (!bs) return set_error(RMQ_EINVAL, "rmq_bs_from_nb: bs is NULL");
    if (n <= 0 || nb <= 0) return set_error(RMQ_EINVAL, "rmq_bs_from_nb: n=%lld nb=%lld must be > 0",
                                            (long long)n, (long long)nb);
    const int64_t k = nb < n ? nb : n;
    *bs = n / k;
    return RMQ_OK;
}

int rmq_build(const float *d_vals, int64_t n, int64_t bs, rmq_stream_t stream,
              rmq_handle_t **out) {
    return rmq_build_ex(d_vals, n, bs, 0, stream, out);
}

int rmq_build_ex(const float *d_vals, int64_t n, int64_t bs, uint32_t flags, rmq_stream_t stream,
                 rmq_handle_t **out) {
    NvtxRange nvtx_range("rmq_build_ex");
    g_err[0] = '\0';
    if (!out) return set_error(RMQ_EINVAL, "rmq_build: out is NULL");
    if (flags & ~static_cast<uint32_t>(RMQ_BUILD_NO_MICRO | RMQ_BUILD_MAX | RMQ_BUILD_INT32 |
                                       RMQ_BUILD_LIGHT))
        return set_error(RMQ_EINVAL, "rmq_build_ex: unknown flags 0x%x", flags);
    *out = nullptr;
    if (n <= 0 || n > 0x7fffffffLL)
        return set_error(RMQ_EINVAL, "rmq_build: n=%lld outside [1, 2^31-1]", (long long)n);
    if (!d_vals) return set_error(RMQ_EINVAL, "rmq_build: d_vals is NULL");
    if (reinterpret_cast<uintptr_t>(d_vals) % 4 != 0)
        return set_error(RMQ_EINVAL, "rmq_build: d_vals not 4-byte aligned");
    if (bs <= 0) bs = RMQ_DEFAULT_BS;
    const bool light = (flags & RMQ_BUILD_LIGHT) != 0;
    if (light) {
        // blocks on micro-block boundaries; one block of the array rounded up
        if (bs > n) bs = (n + 31) / 32 * 32;
        if ((flags & RMQ_BUILD_NO_MICRO) || bs < 64 || bs % 32 != 0)
            return set_error(RMQ_EINVAL,
                             "rmq_build_ex: a light index needs the sub-block level and a block "
                             "size that is a multiple of 32 and at least 64 (bs=%lld)",
                             (long long)bs);
    } else if (bs > n) {
        bs = n;
    }

    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;

    BuildPlan p;
    std::memset(&p, 0, sizeof(p));
    p.A = d_vals;
    p.n = static_cast<uint32_t>(n);
    p.bs = static_cast<uint32_t>(bs);
    p.light = light;
    p.kmode = ((flags & RMQ_BUILD_INT32) ? kIntMin : kFloatMin) + ((flags & RMQ_BUILD_MAX) ? 1u : 0u);
    const size_t total = plan_index(p, (flags & RMQ_BUILD_NO_MICRO) != 0);

    rmq_handle_t *h = new (std::nothrow) rmq_handle_t;
    if (!h) return set_error(RMQ_ENOMEM, "rmq_build: host allocation failed");
    std::memset(h, 0, sizeof(*h));
    h->host_mu = new (std::nothrow) std::mutex;
    if (!h->host_mu) {
        delete h;
        return set_error(RMQ_ENOMEM, "rmq_build: host allocation failed");
    }
    h->device = dev.device;
    cudaError_t err = dev_malloc(&h->mem, total);
    if (err != cudaSuccess) {
        delete h->host_mu;
        delete h;
        cudaGetLastError();
        return set_error(RMQ_ENOMEM, "rmq_build: cudaMalloc(%zu bytes) failed: %s", total,
                         cudaGetErrorString(err));
    }
    h->invalid = place_index(p, h->mem);
    h->mem_bytes = total;
    h->table_bytes = static_cast<int64_t>(sizeof(Entry) * static_cast<size_t>(p.nb) * p.levels);
    h->plan = p;

    err = cudaMemsetAsync(h->invalid, 0, sizeof(unsigned long long), stream);
    if (err == cudaSuccess) err = launch_build(p, dev, stream);
    if (err != cudaSuccess) {
        rc = cuda_fail(err, "rmq_build: launch");
        cudaFree(h->mem);
        delete h->host_mu;
        delete h;
        return rc;
    }
    *out = h;
    return RMQ_OK;
}

int rmq_query(const rmq_handle_t *h, const int32_t *d_queries, int64_t q, float *d_val,
              int32_t *d_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_query");
    g_err[0] = '\0';
    if (!h) return set_error(RMQ_EINVAL, "rmq_query: handle is NULL");
    if (q < 0) return set_error(RMQ_EINVAL, "rmq_query: q=%lld < 0", (long long)q);
    if (q == 0) return RMQ_OK;
    if (!d_queries) return set_error(RMQ_EINVAL, "rmq_query: d_queries is NULL");
    if (reinterpret_cast<uintptr_t>(d_queries) % 8 != 0)
        return set_error(RMQ_EINVAL, "rmq_query: d_queries not 8-byte aligned");
    if (!d_val && !d_idx) return set_error(RMQ_EINVAL, "rmq_query: both outputs are NULL");
    if ((d_val && reinterpret_cast<uintptr_t>(d_val) % 4) ||
        (d_idx && reinterpret_cast<uintptr_t>(d_idx) % 4))
        return set_error(RMQ_EINVAL, "rmq_query: outputs not 4-byte aligned");
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    if (dev.device != h->device)
        return set_error(RMQ_EINVAL, "rmq_query: handle built on device %d, current is %d",
                         h->device, dev.device);
    QueryArgs a;
    a.Q = reinterpret_cast<const int2 *>(d_queries);
    a.q = q;
    a.val = d_val;
    a.idx = d_idx;
    a.invalid = h->invalid;
    cudaError_t err = launch_query(h->plan, a, dev, stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_query: launch");
    return RMQ_OK;
}

int rmq_probe_gather(const rmq_handle_t *h, const int32_t *d_queries, int64_t q, float *d_val,
                     int32_t *d_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_probe_gather");
    g_err[0] = '\0';
    if (!h) return set_error(RMQ_EINVAL, "rmq_probe_gather: handle is NULL");
    if (q < 0) return set_error(RMQ_EINVAL, "rmq_probe_gather: q=%lld < 0", (long long)q);
    if (q == 0) return RMQ_OK;
    if (!d_queries || reinterpret_cast<uintptr_t>(d_queries) % 8 != 0)
        return set_error(RMQ_EINVAL, "rmq_probe_gather: d_queries NULL or not 8-byte aligned");
    if (!d_val && !d_idx) return set_error(RMQ_EINVAL, "rmq_probe_gather: both outputs are NULL");
    if ((d_val && reinterpret_cast<uintptr_t>(d_val) % 4) ||
        (d_idx && reinterpret_cast<uintptr_t>(d_idx) % 4))
        return set_error(RMQ_EINVAL, "rmq_probe_gather: outputs not 4-byte aligned");
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    if (dev.device != h->device)
        return set_error(RMQ_EINVAL, "rmq_probe_gather: handle built on device %d, current is %d",
                         h->device, dev.device);
    QueryArgs a;
    a.Q = reinterpret_cast<const int2 *>(d_queries);
    a.q = q;
    a.val = d_val;
    a.idx = d_idx;
    a.invalid = nullptr;
    cudaError_t err = launch_probe_gather(h->plan, a, dev, stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_probe_gather: launch");
    return RMQ_OK;
}

int rmq_query_stats(const rmq_handle_t *h, const int32_t *d_queries, int64_t q, float *d_val,
                    int32_t *d_idx, int64_t *h_counts, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_query_stats");
    g_err[0] = '\0';
    if (!h || !h_counts) return set_error(RMQ_EINVAL, "rmq_query_stats: NULL argument");
    if (q < 0) return set_error(RMQ_EINVAL, "rmq_query_stats: q=%lld < 0", (long long)q);
    for (int c = 0; c < RMQ_QUERY_STATS_FIELDS; ++c) h_counts[c] = 0;
    if (q == 0) return RMQ_OK;
    if (!d_queries || reinterpret_cast<uintptr_t>(d_queries) % 8 != 0)
        return set_error(RMQ_EINVAL, "rmq_query_stats: d_queries NULL or not 8-byte aligned");
    if ((d_val && reinterpret_cast<uintptr_t>(d_val) % 4) ||
        (d_idx && reinterpret_cast<uintptr_t>(d_idx) % 4))
        return set_error(RMQ_EINVAL, "rmq_query_stats: outputs not 4-byte aligned");
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    if (dev.device != h->device)
        return set_error(RMQ_EINVAL, "rmq_query_stats: handle built on device %d, current is %d",
                         h->device, dev.device);
    // the counters sit in the handle's counter block, after the invalid-query
    // counter (kStatsSlot words in, RMQ_QUERY_STATS_FIELDS words)
    unsigned long long *dst = h->invalid + kStatsSlot;
    QueryArgs a;
    a.Q = reinterpret_cast<const int2 *>(d_queries);
    a.q = q;
    a.val = d_val;
    a.idx = d_idx;
    a.invalid = h->invalid;
    a.stats = dst;
    unsigned long long host[RMQ_QUERY_STATS_FIELDS];
    cudaError_t err = cudaMemsetAsync(dst, 0, sizeof(host), stream);
    if (err == cudaSuccess) err = launch_query(h->plan, a, dev, stream);
    if (err == cudaSuccess) err = cudaMemcpyAsync(host, dst, sizeof(host), cudaMemcpyDeviceToHost, stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_query_stats");
    for (int c = 0; c < RMQ_QUERY_STATS_FIELDS; ++c) h_counts[c] = static_cast<int64_t>(host[c]);
    return RMQ_OK;
}

int rmq_probe_random(const uint64_t *d_buf, int64_t words, const int32_t *d_queries, int64_t q,
                     float *d_val, int32_t *d_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_probe_random");
    g_err[0] = '\0';
    if (!d_buf || words <= 0 || reinterpret_cast<uintptr_t>(d_buf) % 8 != 0)
        return set_error(RMQ_EINVAL, "rmq_probe_random: d_buf NULL, unaligned or words <= 0");
    if (q < 0) return set_error(RMQ_EINVAL, "rmq_probe_random: q=%lld < 0", (long long)q);
    if (q == 0) return RMQ_OK;
    if (!d_queries || reinterpret_cast<uintptr_t>(d_queries) % 8 != 0)
        return set_error(RMQ_EINVAL, "rmq_probe_random: d_queries NULL or not 8-byte aligned");
    if (!d_val && !d_idx) return set_error(RMQ_EINVAL, "rmq_probe_random: both outputs are NULL");
    if ((d_val && reinterpret_cast<uintptr_t>(d_val) % 4) ||
        (d_idx && reinterpret_cast<uintptr_t>(d_idx) % 4))
        return set_error(RMQ_EINVAL, "rmq_probe_random: outputs not 4-byte aligned");
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    QueryArgs a;
    a.Q = reinterpret_cast<const int2 *>(d_queries);
    a.q = q;
    a.val = d_val;
    a.idx = d_idx;
    a.invalid = nullptr;
    cudaError_t err = launch_probe_random(reinterpret_cast<const unsigned long long *>(d_buf),
                                          static_cast<uint64_t>(words), a, dev, stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_probe_random: launch");
    return RMQ_OK;
}

// Streams, events and buffer of the rmq_query_host pipeline, whatever part
// of them exists (after waiting for their work); the handle then has none.
static cudaError_t release_staging(rmq_handle_t *h) {
    cudaStream_t *streams[] = {&h->hs, &h->ks, &h->cs};
    for (cudaStream_t *st : streams)
        if (*st) {
            cudaStreamSynchronize(*st);
            cudaStreamDestroy(*st);
            *st = nullptr;
        }
    for (int s = 0; s < kHostStreams; ++s) {
        cudaEvent_t *evs[] = {&h->h_done[s], &h->k_done[s], &h->c_done[s]};
        for (cudaEvent_t *e : evs)
            if (*e) {
                cudaEventDestroy(*e);
                *e = nullptr;
            }
    }
    cudaEvent_t *evs[] = {&h->ev_start, &h->ev_end};
    for (cudaEvent_t *e : evs)
        if (*e) {
            cudaEventDestroy(*e);
            *e = nullptr;
        }
    for (bool &u : h->slot_used) u = false;
    cudaError_t err = cudaSuccess;
    if (h->stage) err = cudaFree(h->stage);
    h->stage = nullptr;
    return err;
}

// True when p is device (or managed) memory of the current context.
static bool is_device_memory(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Device-usable address of host memory the GPU can read in place
// (page-locked and mapped, or any memory where the device reads pageable
// memory), or null.
static const void *device_address(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return p;
    if (at.type == cudaMemoryTypeHost && at.devicePointer) return at.devicePointer;
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
        pageable)
        return p;
    cudaGetLastError();
    return nullptr;
}

int rmq_query_host(const rmq_handle_t *h, const int32_t *h_queries, int64_t q, float *h_val,
                   int32_t *h_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_query_host");
    g_err[0] = '\0';
    if (!h) return set_error(RMQ_EINVAL, "rmq_query_host: handle is NULL");
    if (q < 0) return set_error(RMQ_EINVAL, "rmq_query_host: q=%lld < 0", (long long)q);
    if (q == 0) return RMQ_OK;
    if (!h_queries) return set_error(RMQ_EINVAL, "rmq_query_host: h_queries is NULL");
    if (!h_val && !h_idx) return set_error(RMQ_EINVAL, "rmq_query_host: both outputs are NULL");
    // RTXRMQ_HOST_STAGED=1 takes the staged path for every buffer, as on a
    // system where the device cannot address host memory (the tests use it
    // to cover that path everywhere). RTXRMQ_HOST_MODE=<m> moves addressable
    // host buffers to staging anyway: bit 0 the results, bit 1 the queries.
    const char *force = std::getenv("RTXRMQ_HOST_STAGED");
    const bool forced = force && force[0] == '1';
    const char *mode_s = std::getenv("RTXRMQ_HOST_MODE");
    const int mode = mode_s ? std::atoi(mode_s) : 0;
    // device memory, page-locked host memory, or host memory on a system
    // where the device reads pageable memory: the kernel reads / writes it
    // in place
    const int2 *qdev = forced ? nullptr : static_cast<const int2 *>(device_address(h_queries));
    float *vdev = (forced || !h_val) ? nullptr
                  : static_cast<float *>(const_cast<void *>(device_address(h_val)));
    int32_t *idev = (forced || !h_idx) ? nullptr
                    : static_cast<int32_t *>(const_cast<void *>(device_address(h_idx)));
    if ((mode & 2) && !is_device_memory(h_queries)) qdev = nullptr;
    if ((mode & 1) && h_val && !is_device_memory(h_val)) vdev = nullptr;
    if ((mode & 1) && h_idx && !is_device_memory(h_idx)) idev = nullptr;
    const bool v_stage = h_val && !vdev;
    const bool i_stage = h_idx && !idev;
    if (qdev && !v_stage && !i_stage)
        return rmq_query(h, reinterpret_cast<const int32_t *>(qdev), q, vdev, idev, stream);

    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    if (dev.device != h->device)
        return set_error(RMQ_EINVAL, "rmq_query_host: handle built on device %d, current is %d",
                         h->device, dev.device);
    rmq_handle_t *hm = const_cast<rmq_handle_t *>(h);
    std::lock_guard<std::mutex> lock(*hm->host_mu);
    cudaError_t err = cudaSuccess;
    if (!hm->stage) {
        // streams and events first, the staging buffer last: `stage` set
        // means the whole pipeline exists; a failure leaves none of it
        err = cudaStreamCreateWithFlags(&hm->hs, cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&hm->ks, cudaStreamNonBlocking);
        if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&hm->cs, cudaStreamNonBlocking);
        for (int s = 0; s < kHostStreams && err == cudaSuccess; ++s) {
            err = cudaEventCreateWithFlags(&hm->h_done[s], cudaEventDisableTiming);
            if (err == cudaSuccess) err = cudaEventCreateWithFlags(&hm->k_done[s], cudaEventDisableTiming);
            if (err == cudaSuccess) err = cudaEventCreateWithFlags(&hm->c_done[s], cudaEventDisableTiming);
        }
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&hm->ev_start, cudaEventDisableTiming);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&hm->ev_end, cudaEventDisableTiming);
        if (err == cudaSuccess) err = dev_malloc(&hm->stage, kHostStreams * kHostChunk * 16);
        if (err != cudaSuccess) {
            release_staging(hm);
            return cuda_fail(err, "rmq_query_host: staging set-up");
        }
    }
    err = cudaEventRecord(hm->ev_start, stream);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(hm->hs, hm->ev_start, 0);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(hm->ks, hm->ev_start, 0);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(hm->cs, hm->ev_start, 0);
    // Chunks of kHostChunk queries over kHostStreams staging slots, three
    // streams: query copies in (hs), the chunk kernels in order (ks), result
    // copies out (cs), each chunk's steps ordered by per-slot events; a slot
    // is reused only when the kernel has read its queries and the copy-out
    // has read its results, including a slot last used by an earlier call
    // on another stream.
    for (int64_t c = 0, i = 0; c < q && err == cudaSuccess; c += kHostChunk, ++i) {
        const int b = static_cast<int>(i % kHostStreams);
        const int64_t m = q - c < kHostChunk ? q - c : kHostChunk;
        char *base = static_cast<char *>(hm->stage) + b * kHostChunk * 16;
        QueryArgs a;
        if (qdev) {
            a.Q = qdev + c;
        } else {
            int32_t *dq = reinterpret_cast<int32_t *>(base);
            if (hm->slot_used[b]) err = cudaStreamWaitEvent(hm->hs, hm->k_done[b], 0);
            if (err == cudaSuccess)
                err = cudaMemcpyAsync(dq, h_queries + 2 * c, m * 8, cudaMemcpyHostToDevice, hm->hs);
            if (err == cudaSuccess) err = cudaEventRecord(hm->h_done[b], hm->hs);
            if (err == cudaSuccess) err = cudaStreamWaitEvent(hm->ks, hm->h_done[b], 0);
            if (err != cudaSuccess) break;
            a.Q = reinterpret_cast<const int2 *>(dq);
        }
        if ((v_stage || i_stage) && hm->slot_used[b])
            err = cudaStreamWaitEvent(hm->ks, hm->c_done[b], 0);
        if (err != cudaSuccess) break;
        float *dv = !h_val ? nullptr : v_stage ? reinterpret_cast<float *>(base + kHostChunk * 8) : vdev + c;
        int32_t *di = !h_idx ? nullptr
                      : i_stage ? reinterpret_cast<int32_t *>(base + kHostChunk * 12) : idev + c;
        a.q = m;
        a.val = dv;
        a.idx = di;
        a.invalid = h->invalid;
        err = launch_query(h->plan, a, dev, hm->ks);
        if (err == cudaSuccess) err = cudaEventRecord(hm->k_done[b], hm->ks);
        if (err == cudaSuccess && (v_stage || i_stage)) {
            err = cudaStreamWaitEvent(hm->cs, hm->k_done[b], 0);
            if (err == cudaSuccess && v_stage)
                err = cudaMemcpyAsync(h_val + c, dv, m * 4, cudaMemcpyDeviceToHost, hm->cs);
            if (err == cudaSuccess && i_stage)
                err = cudaMemcpyAsync(h_idx + c, di, m * 4, cudaMemcpyDeviceToHost, hm->cs);
            if (err == cudaSuccess) err = cudaEventRecord(hm->c_done[b], hm->cs);
        }
        if (err == cudaSuccess) hm->slot_used[b] = true;
    }
    // `stream` continues when the kernel and copy-out streams are done (the
    // query copies precede their kernels)
    if (err == cudaSuccess) err = cudaEventRecord(hm->ev_end, hm->ks);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(stream, hm->ev_end, 0);
    if (err == cudaSuccess) err = cudaEventRecord(hm->ev_end, hm->cs);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(stream, hm->ev_end, 0);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_query_host");
    return RMQ_OK;
}

int rmq_free(rmq_handle_t *h) {
    g_err[0] = '\0';
    if (!h) return RMQ_OK;
    cudaError_t err = release_staging(h);
    cudaError_t e2 = cudaFree(h->mem);
    if (err == cudaSuccess) err = e2;
    delete h->host_mu;
    delete h;
    if (err != cudaSuccess) return cuda_fail(err, "rmq_free: cudaFree");
    return RMQ_OK;
}

int rmq_info(const rmq_handle_t *h, rmq_info_t *info) {
    g_err[0] = '\0';
    if (!h || !info) return set_error(RMQ_EINVAL, "rmq_info: NULL argument");
    info->n = h->plan.n;
    info->bs = h->plan.bs;
    info->nb = h->plan.nb;
    info->levels = static_cast<int32_t>(h->plan.levels);
    info->aligned = h->plan.aligned ? 1 : 0;
    info->table_bytes = h->table_bytes;
    info->struct_bytes = static_cast<int64_t>(h->mem_bytes);
    info->micro_levels = static_cast<int32_t>(h->plan.mlevels);
    info->light = h->plan.light ? 1 : 0;
    info->micro_table_bytes =
        h->plan.micro ? static_cast<int64_t>(static_cast<size_t>(h->plan.nmicro) *
                                             (sizeof(Entry) + static_cast<size_t>(h->plan.moff_bytes) *
                                                                  (h->plan.mlevels - 1)))
                      : 0;
    info->is_max = (h->plan.kmode & 1u) ? 1 : 0;
    info->is_int32 = (h->plan.kmode >= kIntMin) ? 1 : 0;
    return RMQ_OK;
}

int rmq_invalid_count(const rmq_handle_t *h, rmq_stream_t stream, int64_t *count) {
    g_err[0] = '\0';
    if (!h || !count) return set_error(RMQ_EINVAL, "rmq_invalid_count: NULL argument");
    unsigned long long v = 0;
    cudaError_t err = cudaMemcpyAsync(&v, h->invalid, sizeof(v), cudaMemcpyDeviceToHost, stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_invalid_count");
    *count = static_cast<int64_t>(v);
    return RMQ_OK;
}

int rmq_checked_violations(int64_t *count) {
    g_err[0] = '\0';
    if (!count) return set_error(RMQ_EINVAL, "rmq_checked_violations: count is NULL");
    *count = 0;
    if (!RMQ_CHECKED)
        return set_error(RMQ_ENOTSUP, "rmq_checked_violations: not a checked build (RMQ_CHECKED=1)");
    const unsigned long long parts[] = {violations_build(), violations_query(), violations_batch(),
                                        violations_batch_light(), violations_persist()};
    for (unsigned long long v : parts) {
        if (v == ~0ull) return set_error(RMQ_ECUDA, "rmq_checked_violations: counter read failed");
        *count += static_cast<int64_t>(v);
    }
    return RMQ_OK;
}

int rmq_query_scan(const float *d_vals, int64_t n, const int32_t *d_queries, int64_t q,
                   float *d_val, int32_t *d_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_query_scan");
    g_err[0] = '\0';
    if (n <= 0 || n > 0x7fffffffLL)
        return set_error(RMQ_EINVAL, "rmq_query_scan: n=%lld outside [1, 2^31-1]", (long long)n);
    if (!d_vals) return set_error(RMQ_EINVAL, "rmq_query_scan: d_vals is NULL");
    if (q < 0) return set_error(RMQ_EINVAL, "rmq_query_scan: q < 0");
    if (q == 0) return RMQ_OK;
    if (!d_queries || reinterpret_cast<uintptr_t>(d_queries) % 8 != 0)
        return set_error(RMQ_EINVAL, "rmq_query_scan: d_queries NULL or not 8-byte aligned");
    if (!d_val && !d_idx) return set_error(RMQ_EINVAL, "rmq_query_scan: both outputs are NULL");
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    QueryArgs a;
    a.Q = reinterpret_cast<const int2 *>(d_queries);
    a.q = q;
    a.val = d_val;
    a.idx = d_idx;
    a.invalid = nullptr;
    cudaError_t err = launch_query_scan(d_vals, static_cast<uint32_t>(n), a, dev, stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_query_scan: launch");
    return RMQ_OK;
}

}  // extern "C"
