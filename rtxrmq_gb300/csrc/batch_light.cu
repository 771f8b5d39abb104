// batch_light.cu -- the light-index instantiations of the persistent batch
// kernel (batch_impl.cuh): per array only the block table and the
// micro-block table, built from one read of the values, and queries that
// settle what the table probes leave open from lines of values. A separate
// translation unit, so that it compiles in parallel with the full-index
// kernels of batch.cu.
#include "batch_impl.cuh"

namespace rmq {
namespace {

std::atomic<int> g_light_per_sm[8];  // (aligned, key mode)

template <bool ALIGNED, uint32_t MODE>
cudaError_t pick_light(const void **fn, size_t *smem, int *per_sm) {
    auto kern = batch_kernel_light<ALIGNED, MODE>;
    std::atomic<int> &slot = g_light_per_sm[(ALIGNED ? 4 : 0) + MODE];
    if (slot.load(std::memory_order_relaxed) == 0) {
        // above the default 48 KB of dynamic shared memory
        const cudaError_t err = cudaFuncSetAttribute(
            kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kLightSmemBytes));
        if (err != cudaSuccess) return err;
    }
    *fn = reinterpret_cast<const void *>(kern);
    *smem = kLightSmemBytes;
    return occupancy_cached(kern, kBatchThreads, slot, *per_sm, kLightSmemBytes);
}

template <bool ALIGNED>
cudaError_t light_kernel_t(uint32_t mode, const void **fn, size_t *smem, int *per_sm) {
    switch (mode) {
    case kFloatMax: return pick_light<ALIGNED, kFloatMax>(fn, smem, per_sm);
    case kIntMin: return pick_light<ALIGNED, kIntMin>(fn, smem, per_sm);
    case kIntMax: return pick_light<ALIGNED, kIntMax>(fn, smem, per_sm);
    default: return pick_light<ALIGNED, kFloatMin>(fn, smem, per_sm);
    }
}

}  // namespace

cudaError_t batch_light_kernel(bool aligned, uint32_t mode, const void **fn, size_t *smem,
                               int *per_sm) {
    return aligned ? light_kernel_t<true>(mode, fn, smem, per_sm)
                   : light_kernel_t<false>(mode, fn, smem, per_sm);
}

RMQ_VIOLATIONS_READER(violations_batch_light)

}  // namespace rmq
