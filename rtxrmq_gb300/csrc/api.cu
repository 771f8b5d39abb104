// api.cu -- the exported C ABI (include/rmq.h): argument checks, memory
// ownership and error reporting around the kernels in build.cu / query.cu.
//
// Error behaviour differs from the reference on purpose: its CUDA_CHECK /
// OPTIX_CHECK print and carry on (common/common.h:57-69) and HRMQ calls
// exit() (hrmq/RMQRMM64.cpp:237-240); here every failure is a status code
// plus a per-thread message.
#include <cstdarg>
#include <cstdio>
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
};

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
    return set_error(RMQ_ECUDA, "%s: %s (%s)", what, cudaGetErrorName(err),
                     cudaGetErrorString(err));
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

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace rmq

using namespace rmq;

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
    g_err[0] = '\0';
    if (!out) return set_error(RMQ_EINVAL, "rmq_build: out is NULL");
    if (flags & ~static_cast<uint32_t>(RMQ_BUILD_NO_MICRO))
        return set_error(RMQ_EINVAL, "rmq_build_ex: unknown flags 0x%x", flags);
    *out = nullptr;
    if (n <= 0 || n > 0x7fffffffLL)
        return set_error(RMQ_EINVAL, "rmq_build: n=%lld outside [1, 2^31-1]", (long long)n);
    if (!d_vals) return set_error(RMQ_EINVAL, "rmq_build: d_vals is NULL");
    if (reinterpret_cast<uintptr_t>(d_vals) % 4 != 0)
        return set_error(RMQ_EINVAL, "rmq_build: d_vals not 4-byte aligned");
    if (bs <= 0) bs = RMQ_DEFAULT_BS;
    if (bs > n) bs = n;

    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;

    BuildPlan p;
    std::memset(&p, 0, sizeof(p));
    p.A = d_vals;
    p.n = static_cast<uint32_t>(n);
    p.bs = static_cast<uint32_t>(bs);
    const size_t total = plan_index(p, (flags & RMQ_BUILD_NO_MICRO) != 0);

    rmq_handle_t *h = new (std::nothrow) rmq_handle_t;
    if (!h) return set_error(RMQ_ENOMEM, "rmq_build: host allocation failed");
    std::memset(h, 0, sizeof(*h));
    h->device = dev.device;
    cudaError_t err = cudaMalloc(&h->mem, total);
    if (err != cudaSuccess) {
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
        delete h;
        return rc;
    }
    *out = h;
    return RMQ_OK;
}

int rmq_query(const rmq_handle_t *h, const int32_t *d_queries, int64_t q, float *d_val,
              int32_t *d_idx, rmq_stream_t stream) {
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

// Device-usable address of a buffer the caller calls "host" memory, or null
// if the current device cannot address it.
static const void *device_view(const void *p, bool *ok) {
    *ok = false;
    if (!p) {
        *ok = true;
        return nullptr;
    }
    cudaPointerAttributes at;
    cudaError_t err = cudaPointerGetAttributes(&at, p);
    if (err != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        *ok = true;
        return p;
    }
    if (at.type == cudaMemoryTypeHost && at.devicePointer) {
        *ok = true;
        return at.devicePointer;
    }
    int dev = 0, pageable = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess &&
        pageable) {
        *ok = true;
        return p;
    }
    cudaGetLastError();
    return nullptr;
}

int rmq_query_host(const rmq_handle_t *h, const int32_t *h_queries, int64_t q, float *h_val,
                   int32_t *h_idx, rmq_stream_t stream) {
    g_err[0] = '\0';
    if (!h) return set_error(RMQ_EINVAL, "rmq_query_host: handle is NULL");
    if (q < 0) return set_error(RMQ_EINVAL, "rmq_query_host: q=%lld < 0", (long long)q);
    if (q == 0) return RMQ_OK;
    if (!h_queries) return set_error(RMQ_EINVAL, "rmq_query_host: h_queries is NULL");
    if (!h_val && !h_idx) return set_error(RMQ_EINVAL, "rmq_query_host: both outputs are NULL");
    bool okq, okv, oki;
    const void *dq = device_view(h_queries, &okq);
    void *dv = const_cast<void *>(device_view(h_val, &okv));
    void *di = const_cast<void *>(device_view(h_idx, &oki));
    if (!okq || !okv || !oki)
        return set_error(RMQ_EINVAL,
                         "rmq_query_host: a buffer is not addressable by the device "
                         "(page-lock it with cudaHostRegister or allocate it with cudaHostAlloc)");
    return rmq_query(h, static_cast<const int32_t *>(dq), q, static_cast<float *>(dv),
                     static_cast<int32_t *>(di), stream);
}

int rmq_free(rmq_handle_t *h) {
    g_err[0] = '\0';
    if (!h) return RMQ_OK;
    cudaError_t err = cudaFree(h->mem);
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
    info->reserved = 0;
    info->micro_table_bytes =
        static_cast<int64_t>(sizeof(Entry) * static_cast<size_t>(h->plan.nmicro) * h->plan.mlevels);
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

int rmq_query_scan(const float *d_vals, int64_t n, const int32_t *d_queries, int64_t q,
                   float *d_val, int32_t *d_idx, rmq_stream_t stream) {
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
