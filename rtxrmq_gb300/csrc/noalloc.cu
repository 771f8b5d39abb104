// noalloc.cu -- build + query of one array in a single call that allocates
// nothing: the index lives in a fixed device array owned by this library.
//
// Who needs it: callers that are not allowed to allocate device memory
// themselves or through a library -- a host framework that accounts for all
// device memory through its own pool and forbids third-party cudaMalloc, or
// a latency-critical loop that cannot take cudaMalloc / cudaFree's implicit
// device-wide synchronisation. They pass their own input and output buffers;
// the prefix/suffix minima, sparse tables and invalid-query counter are
// written into g_noalloc_scratch below instead of memory from rmq_build.
//
// The array is a file-scope __device__ variable of kNoallocScratchBytes, so
// every GPU that loads this library holds it until the process exits. In
// host code its name is only a host-side stand-in, never a device address:
// the device address comes from cudaGetSymbolAddress, called with that
// device current on the first call of rmq_query_noalloc on the device and
// again whenever the device's context has changed since (a device reset
// ends the context, and the next one may place the array elsewhere).
// All calls share the array and it keeps the last call's contents; the
// counter is cleared by every call and everything else is rewritten before
// it is read. Calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array.
#include <cstring>
#include <mutex>

#include <cuda.h>  // driver types only; the driver is reached through the runtime

#include "../../include/rmq.h"
#include "engine.h"

static __device__ __align__(256) unsigned char g_noalloc_scratch[RMQ_NOALLOC_SCRATCH_BYTES];

namespace rmq {
namespace {

constexpr size_t kNoallocScratchBytes = static_cast<size_t>(RMQ_NOALLOC_SCRATCH_BYTES);

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[kMaxDevices] = {nullptr};
unsigned long long g_noalloc_ctx[kMaxDevices] = {0};

// Unique id of the calling thread's current context (cuCtxGetId), 0 when
// there is none or the driver cannot tell. Context handles may be reused
// after a reset; the ids are not.
unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static std::once_flag once;
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult st;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &st) ==
                cudaSuccess && st == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &st) ==
                cudaSuccess && st == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
        cudaGetLastError();
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c ||
        get_id(c, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of the scratch array on the current device (set-up on the
// first call per device, repeated when the context is not the one the
// address was taken in, or cannot be identified).
int scratch_address(int device, void **out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_noalloc_ptr[device] || ctx == 0 || ctx != g_noalloc_ctx[device]) {
        void *p = nullptr;
        cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (err != cudaSuccess || !p) {
            cudaGetLastError();
            g_noalloc_ptr[device] = nullptr;
            return set_error(RMQ_ECUDA, "rmq_query_noalloc: cudaGetSymbolAddress failed: %s",
                             cudaGetErrorString(err));
        }
        g_noalloc_ptr[device] = p;
        // taken after the lookup, which makes the device's context current
        g_noalloc_ctx[device] = current_context_id();
    }
    *out = g_noalloc_ptr[device];
    return RMQ_OK;
}

}  // namespace
}  // namespace rmq

using namespace rmq;

extern "C" int rmq_query_noalloc(const float *d_vals, int64_t n, int64_t bs,
                                 const int32_t *d_queries, int64_t q, float *d_val,
                                 int32_t *d_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_query_noalloc");
    if (n <= 0 || n > 0x7fffffffLL)
        return set_error(RMQ_EINVAL, "rmq_query_noalloc: n=%lld outside [1, 2^31-1]", (long long)n);
    if (!d_vals || reinterpret_cast<uintptr_t>(d_vals) % 4)
        return set_error(RMQ_EINVAL, "rmq_query_noalloc: d_vals NULL or not 4-byte aligned");
    if (q < 0) return set_error(RMQ_EINVAL, "rmq_query_noalloc: q=%lld < 0", (long long)q);
    if (q > 0 && (!d_queries || reinterpret_cast<uintptr_t>(d_queries) % 8))
        return set_error(RMQ_EINVAL, "rmq_query_noalloc: d_queries NULL or not 8-byte aligned");
    if (q > 0 && !d_val && !d_idx)
        return set_error(RMQ_EINVAL, "rmq_query_noalloc: both outputs are NULL");
    if ((d_val && reinterpret_cast<uintptr_t>(d_val) % 4) ||
        (d_idx && reinterpret_cast<uintptr_t>(d_idx) % 4))
        return set_error(RMQ_EINVAL, "rmq_query_noalloc: outputs not 4-byte aligned");
    if (bs <= 0) bs = RMQ_DEFAULT_BS;
    if (bs > n) bs = n;

    BuildPlan p;
    std::memset(&p, 0, sizeof(p));
    p.A = d_vals;
    p.n = static_cast<uint32_t>(n);
    p.bs = static_cast<uint32_t>(bs);
    // the sub-block level when it fits, otherwise the plain index (same results)
    size_t need = plan_index(p, false);
    if (need > kNoallocScratchBytes) need = plan_index(p, true);
    if (need > kNoallocScratchBytes)
        return set_error(RMQ_EINVAL,
                         "rmq_query_noalloc: n=%lld with bs=%lld needs %zu bytes of scratch; the "
                         "static scratch holds %zu bytes (use rmq_build / rmq_query)",
                         (long long)n, (long long)bs, need, kNoallocScratchBytes);

    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    if (dev.device >= kMaxDevices)
        return set_error(RMQ_ENOTSUP, "rmq_query_noalloc: device %d unsupported", dev.device);
    void *base = nullptr;
    rc = scratch_address(dev.device, &base);
    if (rc) return rc;
    unsigned long long *invalid = place_index(p, base);

    cudaError_t err = cudaMemsetAsync(invalid, 0, sizeof(unsigned long long), stream);
    if (err == cudaSuccess) err = launch_build(p, dev, stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_query_noalloc: build");
    if (q == 0) return RMQ_OK;
    QueryArgs a;
    a.Q = reinterpret_cast<const int2 *>(d_queries);
    a.q = q;
    a.val = d_val;
    a.idx = d_idx;
    a.invalid = invalid;
    err = launch_query(p, a, dev, stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_query_noalloc: query");
    return RMQ_OK;
}
