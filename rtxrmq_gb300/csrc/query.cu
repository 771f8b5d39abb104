// query.cu -- plain query kernels.
//
// query_kernel: one CTA answers 256 * QPT consecutive queries at a time with
// the queued body of query_impl.cuh (RTX_blocks' three-ray decomposition,
// src/rtx_kernels.cu:85-193 and 350-465, needed only for the queries a
// probe of the small tables over a superset of [l, r] does not settle). Queries and outputs may live in device memory or in pinned host
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
#ifndef RMQ_QUERY_MINB
#define RMQ_QUERY_MINB 1  // CTAs per SM the query kernel is compiled for (a register bound)
#endif
#ifndef RMQ_QUERY_LIGHT_MINB
#define RMQ_QUERY_LIGHT_MINB 3  // the same for the light-index instantiations (68 registers)
#endif

// Queries base + t + k * kThreads (k < kQPT) of a full step, no bounds checks.
__device__ __forceinline__ void load_full(const QueryOut &o, int64_t base, int2 (&qq)[kQPT]) {
    const int2 *Qs = o.Q + base;
#pragma unroll
    for (int k = 0; k < kQPT; ++k) qq[k] = __ldcs(Qs + threadIdx.x + k * kThreads);
}

// Grid-stride over steps of 256 * kQPT queries (answer_step_queued); the
// next step's queries are loaded before the current step is answered, so
// their latency (host memory over the host link when called through
// rmq_query_host) overlaps the current step's lookups. Specialised on the
// key mode and on whether the index has the sub-block level. STATS: the
// measurement instantiation (rmq_query_stats), which also counts how each
// query was settled and what it read into stats[kStatCount].
template <bool ALIGNED, bool MICRO, bool LIGHT, uint32_t MODE, bool STATS>
__global__ void __launch_bounds__(kThreads, LIGHT ? RMQ_QUERY_LIGHT_MINB : RMQ_QUERY_MINB)
query_kernel(V1View v, QueryOut o, int64_t q, unsigned long long *stats) {
    __shared__ MissQueue s_mq[kThreads / 32];
    // light index only: each thread's slot for the line copies of its
    // misses (dynamic shared memory; none is given to other launches, so
    // they keep the whole L1)
    extern __shared__ uint4 s_lines[];
    uint4 *const lines = LIGHT ? s_lines : nullptr;
    constexpr int64_t chunk = static_cast<int64_t>(kThreads) * kQPT;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * chunk;
    int64_t c0 = static_cast<int64_t>(blockIdx.x) * chunk;
    if (c0 >= q) return;
    const int64_t last_full = q - chunk;  // steps starting at or before it are full
    QStats s;
    if constexpr (STATS)
        for (int c = 0; c < kStatCount; ++c) s.c[c] = 0u;
    MissQueue &mq = s_mq[threadIdx.x >> 5];
    uint32_t waiting = 0;  // the warp's queue length (warp-uniform)
    int2 cur[kQPT];
    if (c0 <= last_full)
        load_full(o, c0, cur);
    else
        load_queries<kQPT>(o, c0, q, cur);
    for (; c0 < q; c0 += stride) {
        const int64_t c1 = c0 + stride;
        int2 nxt[kQPT];
        if (c1 <= last_full)
            load_full(o, c1, nxt);
        else if (c1 < q)
            load_queries<kQPT>(o, c1, q, nxt);
        if (c0 <= last_full)
            answer_step_queued<ALIGNED, MICRO, LIGHT, MODE, kThreads, kQPT, STATS, true>(
                v, o, c0, static_cast<uint32_t>(chunk), cur, s, mq, waiting, lines);
        else
            answer_step_queued<ALIGNED, MICRO, LIGHT, MODE, kThreads, kQPT, STATS, false>(
                v, o, c0, static_cast<uint32_t>(q - c0), cur, s, mq, waiting, lines);
#pragma unroll
        for (int k = 0; k < kQPT; ++k) cur[k] = nxt[k];
    }
    if (waiting) drain_misses<ALIGNED, MICRO, LIGHT, MODE, STATS>(v, o, mq, waiting, l2_keep_policy(), s, lines);
    if constexpr (STATS) flush_stats(s, stats);
}

// Random-access ceiling of the un-pruned query on this index
// (rmq_probe_gather): query_kernel's grid, query stream and output stores,
// but per query only the two random 8-byte lookups suf[l] and pre[r] (no
// block decision, no table probe, no scan). Its answers are not range minima.
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

// 64-bit finaliser of SplitMix64 (Steele, Lea, Flood, OOPSLA 2014).
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Random-access rate of this GPU, independent of any index layout
// (rmq_probe_random): query_kernel's grid, query stream and output stores,
// and per query two 8-byte loads at positions hashed from (i, l, r),
// uniform over buf[0 .. words).
__global__ void __launch_bounds__(kThreads)
random_gather_kernel(const unsigned long long *__restrict__ buf, uint64_t words, QueryOut o,
                     int64_t q) {
    const int64_t chunk = static_cast<int64_t>(kThreads) * kQPT;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * chunk;
    for (int64_t c0 = static_cast<int64_t>(blockIdx.x) * chunk; c0 < q; c0 += stride) {
        int2 qq[kQPT];
        load_queries<kQPT>(o, c0, c0 + chunk < q ? c0 + chunk : q, qq);
        Entry e[kQPT];
#pragma unroll
        for (int k = 0; k < kQPT; ++k) {
            const int64_t i = c0 + threadIdx.x + static_cast<int64_t>(k) * kThreads;
            const uint64_t h1 = mix64((static_cast<uint64_t>(i) << 32) ^ static_cast<uint32_t>(qq[k].x));
            const uint64_t h2 = mix64(h1 ^ static_cast<uint32_t>(qq[k].y));
            const uint64_t p1 = __umul64hi(h1, words), p2 = __umul64hi(h2, words);
            e[k] = better(__ldg(buf + p1), __ldg(buf + p2));
        }
#pragma unroll
        for (int k = 0; k < kQPT; ++k) {
            const int64_t i = c0 + threadIdx.x + static_cast<int64_t>(k) * kThreads;
            if (i < q) put_bits_idx(o, i, static_cast<uint32_t>(e[k] >> 32), static_cast<uint32_t>(e[k]));
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

std::atomic<int> g_gather_per_sm{0};
std::atomic<int> g_random_per_sm{0};
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
    v.micro_span = p.micro ? (1u << p.mlevels) - 1u : 0u;
    return v;
}

constexpr size_t kLineBytes = sizeof(uint4) * kLineChunks * kThreads;  // light launches

template <bool ALIGNED, bool MICRO, bool LIGHT, uint32_t MODE, bool STATS>
cudaError_t launch_query_t(const V1View &v, const QueryOut &o, int64_t q,
                           unsigned long long *stats, const DeviceInfo &dev, cudaStream_t s) {
    static std::atomic<int> per_sm_cache{0};
    auto kern = query_kernel<ALIGNED, MICRO, LIGHT, MODE, STATS>;
    const size_t smem = LIGHT ? kLineBytes : 0;
    int per_sm = per_sm_cache.load(std::memory_order_relaxed);
    if (per_sm == 0) {
        cudaError_t err;
        if (LIGHT) {
            // the line slots exceed the 48 KB default of dynamic shared memory
            err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(smem));
            if (err != cudaSuccess) return err;
        }
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
        if (err != cudaSuccess) return err;
        if (per_sm < 1) per_sm = 1;
        per_sm_cache.store(per_sm, std::memory_order_relaxed);
    }
    kern<<<grid_size(q, kThreads * kQPT, per_sm, dev), kThreads, smem, s>>>(v, o, q, stats);
    return cudaGetLastError();
}

template <bool ALIGNED, bool MICRO, bool LIGHT, bool STATS>
cudaError_t launch_query_m(const V1View &v, const QueryOut &o, int64_t q,
                           unsigned long long *stats, const DeviceInfo &dev, cudaStream_t s) {
    switch (v.kmode) {
    case kFloatMax: return launch_query_t<ALIGNED, MICRO, LIGHT, kFloatMax, STATS>(v, o, q, stats, dev, s);
    case kIntMin: return launch_query_t<ALIGNED, MICRO, LIGHT, kIntMin, STATS>(v, o, q, stats, dev, s);
    case kIntMax: return launch_query_t<ALIGNED, MICRO, LIGHT, kIntMax, STATS>(v, o, q, stats, dev, s);
    default: return launch_query_t<ALIGNED, MICRO, LIGHT, kFloatMin, STATS>(v, o, q, stats, dev, s);
    }
}

template <bool STATS>
cudaError_t launch_query_s(const BuildPlan &p, const V1View &v, const QueryOut &o, int64_t q,
                           unsigned long long *stats, const DeviceInfo &dev, cudaStream_t s) {
    const bool micro = v.mst != nullptr;
    if (micro && p.light)
        return p.aligned ? launch_query_m<true, true, true, STATS>(v, o, q, stats, dev, s)
                         : launch_query_m<false, true, true, STATS>(v, o, q, stats, dev, s);
    if (p.aligned)
        return micro ? launch_query_m<true, true, false, STATS>(v, o, q, stats, dev, s)
                     : launch_query_m<true, false, false, STATS>(v, o, q, stats, dev, s);
    return micro ? launch_query_m<false, true, false, STATS>(v, o, q, stats, dev, s)
                 : launch_query_m<false, false, false, STATS>(v, o, q, stats, dev, s);
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
    if (a.stats) return launch_query_s<true>(p, v, o, a.q, a.stats, dev, s);
    return launch_query_s<false>(p, v, o, a.q, nullptr, dev, s);
}

cudaError_t launch_probe_random(const unsigned long long *buf, uint64_t words, const QueryArgs &a,
                                const DeviceInfo &dev, cudaStream_t s) {
    if (a.q <= 0) return cudaSuccess;
    QueryOut o;
    o.Q = a.Q;
    o.val = a.val;
    o.idx = a.idx;
    o.invalid = nullptr;
    o.span = a.q;
    int per_sm;
    cudaError_t err = occupancy(random_gather_kernel, &g_random_per_sm, &per_sm);
    if (err != cudaSuccess) return err;
    random_gather_kernel<<<grid_size(a.q, kThreads * kQPT, per_sm, dev), kThreads, 0, s>>>(
        buf, words, o, a.q);
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
