// build.cu -- construction of the block-decomposition index for one array.
//
// The reference builds, for RTX_blocks, one triangle per element plus one
// per block minimum and hands them to the OptiX BVH builder
// (src/device_tools.cuh:139-169, 243-253, src/rtx.h:3-22, 39-99). GB300 has
// no RT cores, so the search structure is rebuilt as arrays a query indexes
// directly: in-block prefix / suffix minima (build_impl.cuh) and a sparse
// table over the block minima:
//   st[k][j] = leftmost minimum of blocks j .. j + 2^k - 1 (k = 0: block minima)
#include "build_impl.cuh"
#include "engine.h"

namespace rmq {
namespace {

template <bool ALIGNED>
__global__ void __launch_bounds__(kBuildThreads)
build_units_kernel(UnitJob J, uint32_t nunits) {
    __shared__ Entry stage[kStageEntries];
    __shared__ uint64_t s_warp[kBuildWarps];
    for (uint32_t u = blockIdx.x; u < nunits; u += gridDim.x)
        build_unit<ALIGNED>(J, u, stage, s_warp);
}

__global__ void st_level_kernel(Entry *st, uint32_t nb, uint32_t k) {
    const Entry *prev = st + static_cast<size_t>(k - 1) * nb;
    Entry *cur = st + static_cast<size_t>(k) * nb;
    const uint32_t half = 1u << (k - 1);
    const uint32_t cnt = nb - (1u << k) + 1;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt;
         j += gridDim.x * blockDim.x)
        cur[j] = better(prev[j], prev[j + half]);
}

// Leftmost minimum of every 32-element micro-block, one thread per block
// reading its 128-byte line with float4 loads.
template <bool ALIGNED>
__global__ void __launch_bounds__(256)
micro_min_kernel(const float *__restrict__ A, uint32_t n, uint32_t nmicro, Entry *mst0) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nmicro;
         j += gridDim.x * blockDim.x) {
        const uint32_t a = j * kMicro;
        const uint32_t b = min(a + kMicro, n);
        uint64_t best = ~0ull;
        uint32_t best_bits = 0u;
        if (ALIGNED && b == a + kMicro) {
            const float4 *src = reinterpret_cast<const float4 *>(A + a);
#pragma unroll
            for (int v = 0; v < 8; ++v) {
                const float4 f = __ldg(src + v);
                const uint32_t w[4] = {__float_as_uint(f.x), __float_as_uint(f.y),
                                       __float_as_uint(f.z), __float_as_uint(f.w)};
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const uint64_t k = (static_cast<uint64_t>(fkey(w[c])) << 32) | (a + 4 * v + c);
                    if (k < best) {
                        best = k;
                        best_bits = w[c];
                    }
                }
            }
        } else {
            for (uint32_t g = a; g < b; ++g) {
                const uint32_t w = __float_as_uint(__ldg(A + g));
                const uint64_t k = (static_cast<uint64_t>(fkey(w)) << 32) | g;
                if (k < best) {
                    best = k;
                    best_bits = w;
                }
            }
        }
        Entry e;
        e.bits = best_bits;
        e.idx = static_cast<uint32_t>(best);
        mst0[j] = e;
    }
}

int g_units_per_sm[2] = {0, 0};

cudaError_t launch_levels(Entry *st, uint32_t nb, uint32_t levels, const DeviceInfo &dev,
                          cudaStream_t s) {
    for (uint32_t k = 1; k < levels; ++k) {
        const uint32_t cnt = nb - (1u << k) + 1;
        uint32_t g = (cnt + 255) / 256;
        const uint32_t cap = static_cast<uint32_t>(dev.sms) * 8u;
        if (g > cap) g = cap;
        st_level_kernel<<<g, 256, 0, s>>>(st, nb, k);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

}  // namespace

uint32_t st_levels(uint32_t nb) { return nb ? static_cast<uint32_t>(ilog2(nb)) + 1u : 0u; }

uint32_t micro_levels(uint32_t bs) {
    if (bs < 2 * kMicro || bs % kMicro) return 0;
    const uint32_t per_block = bs / kMicro;  // a same-block query spans at most per_block - 2 between
    return per_block <= 2 ? 1u : st_levels(per_block - 2);
}

cudaError_t launch_build(const BuildPlan &p, const DeviceInfo &dev, cudaStream_t s) {
    if (p.n == 0) return cudaSuccess;
    UnitJob J;
    J.A = p.A;
    J.off = 0;
    J.limit = p.n;
    J.n = p.n;
    J.bs = p.bs;
    J.U = make_unit_layout(p.bs, p.nb);
    J.dv = make_div31(p.bs);
    J.pre = p.pre;
    J.suf = p.suf;
    J.bmin = p.st;
    const uint32_t nunits = unit_count(p.nb, J.U);

    cudaError_t err;
    int &per_sm = g_units_per_sm[p.aligned ? 1 : 0];
    if (per_sm == 0) {
        err = p.aligned ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &per_sm, build_units_kernel<true>, kBuildThreads, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                              &per_sm, build_units_kernel<false>, kBuildThreads, 0);
        if (err != cudaSuccess) return err;
        if (per_sm < 1) per_sm = 1;
    }
    uint32_t grid = static_cast<uint32_t>(dev.sms) * static_cast<uint32_t>(per_sm);
    if (grid > nunits) grid = nunits;
    if (p.aligned)
        build_units_kernel<true><<<grid, kBuildThreads, 0, s>>>(J, nunits);
    else
        build_units_kernel<false><<<grid, kBuildThreads, 0, s>>>(J, nunits);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    err = launch_levels(p.st, p.nb, p.levels, dev, s);
    if (err != cudaSuccess || !p.micro) return err;

    uint32_t g = (p.nmicro + 255) / 256;
    const uint32_t cap = static_cast<uint32_t>(dev.sms) * 16u;
    if (g > cap) g = cap;
    if (p.aligned)
        micro_min_kernel<true><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, p.mst);
    else
        micro_min_kernel<false><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, p.mst);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    return launch_levels(p.mst, p.nmicro, p.mlevels, dev, s);
}

}  // namespace rmq
