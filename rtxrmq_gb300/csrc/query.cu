// query.cu -- the query kernels.
//
// query_kernel replaces RTX_blocks' ray programs (src/rtx_kernels.cu:85-193
// for values, 350-465 for indices). The reference fires up to three rays per
// query: one through the fully covered blocks lB+1..rB-1, one through the
// left partial block and one through the right partial block, and keeps the
// closest hit. Here the same decomposition is answered from arrays:
//   left partial block   -> suf[l]
//   right partial block  -> pre[r]
//   full blocks between  -> two sparse-table entries (L2-resident)
// and a query inside one block (the reference's single-ray case,
// src/rtx_kernels.cu:116-135) is answered from pre/suf when it touches a
// block edge, otherwise by a warp-cooperative scan of A[l..r] that reduces
// order-preserving keys with __reduce_min_sync.
//
// Differences from the reference kept on purpose: ties between rays are
// resolved leftmost (the reference compares rays with strict `<` in the
// order middle, left, right, src/rtx_kernels.cu:451-465), values are the
// exact bits of A[idx] (the reference returns payload + min, rtx.h:109,
// rtx_kernels.cu:179), and a miss cannot overwrite a minimum
// (src/rtx_kernels.cu:80-83).
//
// scan_kernel is the GPU brute force of alg 2 / 102
// (src/cuda_methods.cuh:3-66): one thread per query, strict `<` from A[l].
#include "engine.h"

namespace rmq {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ void write_result(const QueryArgs &a, int64_t i, Entry e) {
    if (a.val) __stcs(a.val + i, __uint_as_float(e.bits));
    if (a.idx) __stcs(a.idx + i, static_cast<int32_t>(e.idx));
}

__device__ __forceinline__ void write_invalid(const QueryArgs &a, int64_t i) {
    if (a.val) __stcs(a.val + i, __uint_as_float(0x7fc00000u));
    if (a.idx) __stcs(a.idx + i, -1);
    if (a.invalid) atomicAdd(a.invalid, 1ull);
}

__device__ __forceinline__ uint64_t comp_bits(uint32_t bits, uint32_t g) {
    return (static_cast<uint64_t>(fkey(bits)) << 32) | g;
}

// Leftmost minimum of A[l..r] computed by the whole warp. All 32 lanes must
// call it with the same (l, r); every lane gets the result.
template <bool ALIGNED>
__device__ __forceinline__ Entry warp_scan_range(const float *__restrict__ A, uint32_t n,
                                                 uint32_t l, uint32_t r, int lane) {
    uint64_t best = ~0ull;
    if (ALIGNED) {
        const uint32_t p0 = l & ~3u;
        for (uint32_t p = p0 + 4u * lane; p <= r; p += 128u) {
            uint32_t b[4];
            if (p + 3u < n) {
                const float4 f = __ldg(reinterpret_cast<const float4 *>(A + p));
                b[0] = __float_as_uint(f.x);
                b[1] = __float_as_uint(f.y);
                b[2] = __float_as_uint(f.z);
                b[3] = __float_as_uint(f.w);
            } else {
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    b[c] = (p + c < n) ? __float_as_uint(__ldg(A + p + c)) : 0u;
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const uint32_t g = p + c;
                if (g >= l && g <= r) {
                    const uint64_t v = comp_bits(b[c], g);
                    best = v < best ? v : best;
                }
            }
        }
    } else {
        for (uint32_t g = l + lane; g <= r; g += 32u) {
            const uint64_t v = comp_bits(__float_as_uint(__ldg(A + g)), g);
            best = v < best ? v : best;
        }
    }
    const uint32_t k = static_cast<uint32_t>(best >> 32);
    const uint32_t kmin = __reduce_min_sync(0xffffffffu, k);
    const uint32_t cand = (k == kmin) ? static_cast<uint32_t>(best) : 0xffffffffu;
    Entry e;
    e.idx = __reduce_min_sync(0xffffffffu, cand);
    e.bits = __float_as_uint(__ldg(A + e.idx));
    return e;
}

template <bool ALIGNED>
__global__ void __launch_bounds__(kThreads)
query_kernel(BuildPlan p, Div31 dv, QueryArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * kThreads;
    const Entry *__restrict__ pre = p.pre;
    const Entry *__restrict__ suf = p.suf;
    const Entry *__restrict__ st = p.st;

    for (int64_t base = static_cast<int64_t>(blockIdx.x) * kThreads; base < a.q; base += stride) {
        const int64_t i = base + threadIdx.x;
        const bool active = i < a.q;
        int2 qq = make_int2(0, 0);
        if (active) qq = __ldcs(a.Q + i);
        const bool valid = active && qq.x >= 0 && qq.x <= qq.y &&
                           static_cast<uint32_t>(qq.y) < p.n;
        const uint32_t l = static_cast<uint32_t>(qq.x);
        const uint32_t r = static_cast<uint32_t>(qq.y);
        bool scan = false;
        Entry e = entry_max();
        if (valid) {
            const uint32_t lB = div31(l, dv);
            const uint32_t rB = div31(r, dv);
            if (lB != rB) {
                const Entry es = suf[l];
                const Entry ep = pre[r];
                e = better(es, ep);
                if (rB - lB >= 2u) {
                    const uint32_t lo = lB + 1u;
                    const uint32_t hi = rB - 1u;
                    const int k = ilog2(hi - lo + 1u);
                    const Entry *lvl = st + static_cast<size_t>(k) * p.nb;
                    e = better(e, better(lvl[lo], lvl[hi + 1u - (1u << k)]));
                }
            } else {
                const uint32_t bstart = lB * p.bs;
                const uint32_t bend = min(bstart + p.bs, p.n) - 1u;
                if (l == bstart)
                    e = pre[r];
                else if (r == bend)
                    e = suf[l];
                else
                    scan = true;
            }
        }
        if (active && !scan) {
            if (valid)
                write_result(a, i, e);
            else
                write_invalid(a, i);
        }

        unsigned mask = __ballot_sync(0xffffffffu, scan);
        while (mask) {
            const int src = __ffs(mask) - 1;
            mask &= mask - 1u;
            const uint32_t ls = __shfl_sync(0xffffffffu, l, src);
            const uint32_t rs = __shfl_sync(0xffffffffu, r, src);
            const Entry es = warp_scan_range<ALIGNED>(p.A, p.n, ls, rs, lane);
            if (lane == src) write_result(a, i, es);
        }
    }
}

__global__ void __launch_bounds__(kThreads)
scan_kernel(const float *__restrict__ A, uint32_t n, QueryArgs a) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * kThreads;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x; i < a.q;
         i += stride) {
        const int2 qq = a.Q[i];
        if (qq.x < 0 || qq.x > qq.y || static_cast<uint32_t>(qq.y) >= n) {
            write_invalid(a, i);
            continue;
        }
        float m = A[qq.x];
        uint32_t mi = static_cast<uint32_t>(qq.x);
        for (uint32_t j = static_cast<uint32_t>(qq.x); j <= static_cast<uint32_t>(qq.y); ++j) {
            const float v = A[j];
            if (v < m) {
                m = v;
                mi = j;
            }
        }
        Entry e;
        e.bits = __float_as_uint(m);
        e.idx = mi;
        write_result(a, i, e);
    }
}

template <typename K>
cudaError_t grid_for(K kernel, int64_t q, const DeviceInfo &dev, uint32_t *grid) {
    int per_sm = 0;
    cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) per_sm = 1;
    const int64_t need = (q + kThreads - 1) / kThreads;
    const int64_t cap = static_cast<int64_t>(dev.sms) * per_sm;
    *grid = static_cast<uint32_t>(need < cap ? need : cap);
    return cudaSuccess;
}

}  // namespace

cudaError_t launch_query(const BuildPlan &p, const QueryArgs &a, const DeviceInfo &dev,
                         cudaStream_t s) {
    if (a.q <= 0) return cudaSuccess;
    const Div31 dv = make_div31(p.bs);
    uint32_t grid = 0;
    cudaError_t err;
    if (p.aligned) {
        err = grid_for(query_kernel<true>, a.q, dev, &grid);
        if (err != cudaSuccess) return err;
        query_kernel<true><<<grid, kThreads, 0, s>>>(p, dv, a);
    } else {
        err = grid_for(query_kernel<false>, a.q, dev, &grid);
        if (err != cudaSuccess) return err;
        query_kernel<false><<<grid, kThreads, 0, s>>>(p, dv, a);
    }
    return cudaGetLastError();
}

cudaError_t launch_query_scan(const float *A, uint32_t n, const QueryArgs &a,
                              const DeviceInfo &dev, cudaStream_t s) {
    if (a.q <= 0) return cudaSuccess;
    uint32_t grid = 0;
    cudaError_t err = grid_for(scan_kernel, a.q, dev, &grid);
    if (err != cudaSuccess) return err;
    scan_kernel<<<grid, kThreads, 0, s>>>(A, n, a);
    return cudaGetLastError();
}

}  // namespace rmq
