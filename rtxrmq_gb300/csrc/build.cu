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

int g_units_per_sm[2] = {0, 0};

}  // namespace

uint32_t st_levels(uint32_t nb) { return nb ? static_cast<uint32_t>(ilog2(nb)) + 1u : 0u; }

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

    for (uint32_t k = 1; k < p.levels; ++k) {
        const uint32_t cnt = p.nb - (1u << k) + 1;
        uint32_t g = (cnt + 255) / 256;
        const uint32_t cap = static_cast<uint32_t>(dev.sms) * 8u;
        if (g > cap) g = cap;
        st_level_kernel<<<g, 256, 0, s>>>(p.st, p.nb, k);
        err = cudaGetLastError();
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

}  // namespace rmq
