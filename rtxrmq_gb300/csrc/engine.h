// engine.h -- internal interface between the C ABI (api.cu) and the kernel
// translation units. Nothing here is exported.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdlib>
#include <cstdint>
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"

namespace rmq {

// Records a message for rmq_last_error_string() and returns `code`.
int set_error(int code, const char *fmt, ...);
// Converts a CUDA error into RMQ_ECUDA (RMQ_ENOMEM for an allocation
// failure) with the call site in the message.
int cuda_fail(cudaError_t err, const char *what);

// Device properties the launchers need, cached per device.
struct DeviceInfo {
    int device;
    int sms;
    size_t l2_bytes;
};
int device_info(DeviceInfo *out);

// NVTX range over one C-ABI call (named after it), visible to profilers
// and tracers; nearly free when none is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Every device allocation of the library goes through here. Fault
// injection for tests: with RTXRMQ_FAIL_ALLOC=1 in the environment it
// fails as an out-of-memory would, without touching the device.
inline cudaError_t dev_malloc(void **p, size_t bytes) {
    const char *f = std::getenv("RTXRMQ_FAIL_ALLOC");
    if (f && f[0] == '1') {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

// Resident CTAs per SM of `kernel` at `threads` threads and `dynamic_smem`
// bytes of dynamic shared memory, computed once per cache slot; concurrent
// first callers compute and store the same value.
template <class K>
cudaError_t occupancy_cached(K kernel, int threads, std::atomic<int> &cache, int &per_sm,
                             size_t dynamic_smem = 0) {
    int v = cache.load(std::memory_order_relaxed);
    if (v == 0) {
        const cudaError_t err =
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, threads, dynamic_smem);
        if (err != cudaSuccess) return err;
        cache.store(v, std::memory_order_relaxed);
    }
    per_sm = v;
    return cudaSuccess;
}

// Checked builds: out-of-range accesses caught per translation unit.
unsigned long long violations_build();
unsigned long long violations_query();
unsigned long long violations_batch();
unsigned long long violations_batch_light();
unsigned long long violations_persist();

// ---- plain index (build.cu) ----
struct BuildPlan {
    const float *A;
    uint32_t n;
    uint32_t bs;
    uint32_t nb;
    uint32_t levels;
    bool aligned;
    Entry *pre;   // [n]
    Entry *suf;   // [n]
    Entry *st;    // [levels * nb], level 0 = block minima
    // sub-block level (every bs >= 64): minima of the 32-element
    // micro-blocks and a sparse table over them truncated to the window
    // lengths a same-block query can need. Level 0 holds the micro-block
    // minima as entries; level k >= 1 holds, for the window of 2^k
    // micro-blocks starting at j, the offset (< 2^k) of its leftmost best
    // micro-block in moff_bytes = 1, 2 or 4 bytes: 1/8 to 1/2 of the bytes
    // of entries, so that the table stays in L2
    bool micro;
    uint32_t nmicro;   // ceil(n / 32)
    uint32_t mlevels;
    Entry *mst;        // [nmicro] micro-block minima (table level 0)
    void *moff;        // [(mlevels - 1) * nmicro] offsets of levels 1 ..
    uint32_t moff_bytes;
    Entry *mpre;       // [n] leftmost minimum of A[microstart(i) .. i]
    Entry *msuf;       // [n] leftmost minimum of A[i .. microend(i)]
    uint32_t kmode;    // KeyMode: float32 / int32 elements, minimum / maximum
    // light index (RMQ_BUILD_LIGHT): the tables only, no per-element entries
    // (pre, suf, mpre, msuf are null); needs the sub-block level and blocks
    // on micro-block boundaries (bs a multiple of 32)
    bool light;
};
constexpr uint32_t kMicro = 32;
// levels of the micro table for block size bs (0 when not applicable)
uint32_t micro_levels(uint32_t bs);
// bytes of one micro-table offset for a table of `mlevels` levels: the
// largest offset is 2^(mlevels - 1) - 1
inline uint32_t micro_offset_bytes(uint32_t mlevels) {
    return mlevels <= 9 ? 1u : (mlevels <= 17 ? 2u : 4u);
}

// Fill the size fields of a plan (A, n, bs and light given; micro level on
// unless `no_micro`); returns the bytes of the single allocation holding the
// index and its invalid-query counter.
size_t plan_index(BuildPlan &p, bool no_micro);
// Point the plan's arrays into that allocation; returns the counter.
unsigned long long *place_index(BuildPlan &p, void *base);
uint32_t st_levels(uint32_t nb);
cudaError_t launch_build(const BuildPlan &p, const DeviceInfo &dev, cudaStream_t s);

// ---- handles (api.cu) ----
}  // namespace rmq
struct rmq_handle;
namespace rmq {
// The plan (with its device pointers), allocation and size of a handle.
int handle_view(const rmq_handle *h, BuildPlan *plan, void **mem, size_t *bytes);
// A new handle owning `mem` (laid out by place_index for `plan`), with its
// invalid-query counter cleared on `stream`.
int handle_adopt(BuildPlan plan, void *mem, size_t bytes, cudaStream_t stream, rmq_handle **out);

// ---- queries (query.cu) ----
struct QueryArgs {
    const int2 *Q;
    int64_t q;
    float *val;
    int32_t *idx;
    unsigned long long *invalid;  // device counter, may be null
    // measurement launches only (rmq_query_stats): kStatCount device
    // counters of how each query was settled; null for every other launch
    unsigned long long *stats = nullptr;
};
cudaError_t launch_query(const BuildPlan &p, const QueryArgs &a, const DeviceInfo &dev,
                         cudaStream_t s);
struct V1View;
V1View view_of(const BuildPlan &p);
cudaError_t launch_probe_gather(const BuildPlan &p, const QueryArgs &a, const DeviceInfo &dev,
                                cudaStream_t s);
// Random 8-byte loads from buf[0 .. words), query_kernel's grid (rmq_probe_random).
cudaError_t launch_probe_random(const unsigned long long *buf, uint64_t words, const QueryArgs &a,
                                const DeviceInfo &dev, cudaStream_t s);
cudaError_t launch_query_scan(const float *A, uint32_t n, const QueryArgs &a,
                              const DeviceInfo &dev, cudaStream_t s);

}  // namespace rmq
