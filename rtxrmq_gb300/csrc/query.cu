// query.cu -- plain query kernels.
//
// query_kernel: one CTA answers 256 * QPT consecutive queries at a time with
// the shared body of query_impl.cuh (RTX_blocks' three-ray decomposition
// answered from pre/suf/sparse-table lookups, src/rtx_kernels.cu:85-193 and
// 350-465). Queries and outputs may live in device memory or in pinned host
// memory mapped into the device address space: on a Grace-Blackwell node the
// kernel then streams them over NVLink-C2C while its random lookups hit HBM.
//
// scan_kernel is the GPU brute force of alg 2 / 102
// (src/cuda_methods.cuh:3-66): one thread per query, strict `<` from A[l].
#include "engine.h"
#include "query_impl.cuh"

namespace rmq {
namespace {

constexpr int kThreads = 256;
#ifndef RMQ_QUERY_QPT
#define RMQ_QUERY_QPT 2  // queries per thread per step (independent lookups in flight)
#endif
constexpr int kQPT = RMQ_QUERY_QPT;

// Grid-stride over steps of 256 * kQPT queries; the next step's queries are
// loaded before the current step is answered, so their latency (host memory
// over the host link when called through rmq_query_host) overlaps the
// current step's lookups.
template <bool ALIGNED>
__global__ void __launch_bounds__(kThreads)
query_kernel(V1View v, QueryOut o, int64_t q) {
    const int64_t chunk = static_cast<int64_t>(kThreads) * kQPT;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * chunk;
    int64_t c0 = static_cast<int64_t>(blockIdx.x) * chunk;
    if (c0 >= q) return;
    int2 cur[kQPT];
    load_queries<kQPT>(o, c0, c0 + chunk < q ? c0 + chunk : q, cur);
    for (; c0 < q; c0 += stride) {
        const int64_t c1 = c0 + stride;
        int2 nxt[kQPT];
        if (c1 < q) load_queries<kQPT>(o, c1, c1 + chunk < q ? c1 + chunk : q, nxt);
        answer_step<ALIGNED, kQPT>(v, o, c0, c0 + chunk < q ? c0 + chunk : q, cur);
#pragma unroll
        for (int k = 0; k < kQPT; ++k) cur[k] = nxt[k];
    }
}

// Random-access ceiling of query_kernel (rmq_probe_gather): the same grid,
// query stream and output stores, but per query only the two random
// 8-byte lookups suf[l] and pre[r] (no block decision, no table probe, no
// scan). Its rate bounds what any two-lookup query kernel reaches on this
// index; its answers are not range minima.
__global__ void __launch_bounds__(kThreads)
gather_kernel(V1View v, QueryOut o, int64_t q) {
    const int64_t chunk = static_cast<int64_t>(kThreads) * kQPT;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * chunk;
    for (int64_t c0 = static_cast<int64_t>(blockIdx.x) * chunk; c0 < q; c0 += stride) {
        int2 qq[kQPT];
        load_queries<kQPT>(o, c0, c0 + chunk < q ? c0 + chunk : q, qq);
        Entry e[kQPT];
#pragma unroll
        for (int k = 0; k < kQPT; ++k) {
            // clamped into the array: the probe never reads out of bounds
            const uint32_t l = min(static_cast<uint32_t>(max(qq[k].x, 0)), v.n - 1u);
            const uint32_t r = min(static_cast<uint32_t>(max(qq[k].y, 0)), v.n - 1u);
            e[k] = better(v.suf[l], v.pre[r]);
        }
#pragma unroll
        for (int k = 0; k < kQPT; ++k) {
            const int64_t i = c0 + threadIdx.x + static_cast<int64_t>(k) * kThreads;
            if (i < q) put_result(o, i, e[k], v.kmode);
        }
    }
}

__global__ void __launch_bounds__(kThreads)
scan_kernel(const float *__restrict__ A, uint32_t n, QueryOut o, int64_t q) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * kThreads;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x; i < q;
         i += stride) {
        const int2 qq = o.Q[i];
        if (qq.x < 0 || qq.x > qq.y || static_cast<uint32_t>(qq.y) >= n) {
            put_invalid(o, i);
            continue;
        }
        float m = A[qq.x];
        uint32_t mi = static_cast<uint32_t>(qq.x);
        for (uint32_t j = static_cast<uint32_t>(qq.x); j <= static_cast<uint32_t>(qq.y); ++j) {
            const float x = A[j];
            if (x < m) {
                m = x;
                mi = j;
            }
        }
        put_bits_idx(o, i, __float_as_uint(m), mi);
    }
}

std::atomic<int> g_query_per_sm[2];
std::atomic<int> g_gather_per_sm{0};
std::atomic<int> g_scan_per_sm{0};

template <typename K>
cudaError_t occupancy(K kernel, std::atomic<int> *cache, int *per_sm) {
    const cudaError_t err = occupancy_cached(kernel, kThreads, *cache, *per_sm);
    if (*per_sm < 1) *per_sm = 1;
    return err;
}

uint32_t grid_size(int64_t q, int64_t per_block, int per_sm, const DeviceInfo &dev) {
    const int64_t need = (q + per_block - 1) / per_block;
    const int64_t cap = static_cast<int64_t>(dev.sms) * per_sm;
    return static_cast<uint32_t>(need < cap ? need : cap);
}

}  // namespace

V1View view_of(const BuildPlan &p) {
    V1View v;
    v.A = p.A;
    v.off = 0;
    v.limit = p.n;
    v.n = p.n;
    v.bs = p.bs;
    v.nb = p.nb;
    v.dv = make_div31(p.bs);
    v.pre = p.pre;
    v.suf = p.suf;
    v.st = p.st;
    v.mst = p.micro ? p.mst : nullptr;
    v.moff = p.micro ? p.moff : nullptr;
    v.moff_bytes = p.micro ? p.moff_bytes : 0u;
    v.nmicro = p.micro ? p.nmicro : 0u;
    v.mpre = p.micro ? p.mpre : nullptr;
    v.msuf = p.micro ? p.msuf : nullptr;
    v.kmode = p.kmode;
    v.levels = p.levels;
    v.mlevels = p.micro ? p.mlevels : 0u;
    return v;
}

cudaError_t launch_query(const BuildPlan &p, const QueryArgs &a, const DeviceInfo &dev,
                         cudaStream_t s) {
    if (a.q <= 0) return cudaSuccess;
    const V1View v = view_of(p);
    QueryOut o;
    o.Q = a.Q;
    o.val = a.val;
    o.idx = a.idx;
    o.invalid = a.invalid;
    o.span = a.q;
    cudaError_t err;
    if (p.aligned) {
        int per_sm;
        err = occupancy(query_kernel<true>, &g_query_per_sm[1], &per_sm);
        if (err != cudaSuccess) return err;
        query_kernel<true><<<grid_size(a.q, kThreads * kQPT, per_sm, dev), kThreads, 0, s>>>(
            v, o, a.q);
    } else {
        int per_sm;
        err = occupancy(query_kernel<false>, &g_query_per_sm[0], &per_sm);
        if (err != cudaSuccess) return err;
        query_kernel<false><<<grid_size(a.q, kThreads * kQPT, per_sm, dev), kThreads, 0, s>>>(
            v, o, a.q);
    }
    return cudaGetLastError();
}

cudaError_t launch_probe_gather(const BuildPlan &p, const QueryArgs &a, const DeviceInfo &dev,
                                cudaStream_t s) {
    if (a.q <= 0) return cudaSuccess;
    const V1View v = view_of(p);
    QueryOut o;
    o.Q = a.Q;
    o.val = a.val;
    o.idx = a.idx;
    o.invalid = nullptr;
    o.span = a.q;
    int per_sm;
    cudaError_t err = occupancy(gather_kernel, &g_gather_per_sm, &per_sm);
    if (err != cudaSuccess) return err;
    gather_kernel<<<grid_size(a.q, kThreads * kQPT, per_sm, dev), kThreads, 0, s>>>(v, o, a.q);
    return cudaGetLastError();
}

cudaError_t launch_query_scan(const float *A, uint32_t n, const QueryArgs &a,
                              const DeviceInfo &dev, cudaStream_t s) {
    if (a.q <= 0) return cudaSuccess;
    int per_sm;
    cudaError_t err = occupancy(scan_kernel, &g_scan_per_sm, &per_sm);
    if (err != cudaSuccess) return err;
    QueryOut o;
    o.Q = a.Q;
    o.val = a.val;
    o.idx = a.idx;
    o.invalid = a.invalid;
    o.span = a.q;
    scan_kernel<<<grid_size(a.q, kThreads, per_sm, dev), kThreads, 0, s>>>(A, n, o, a.q);
    return cudaGetLastError();
}

RMQ_VIOLATIONS_READER(violations_query)

}  // namespace rmq
