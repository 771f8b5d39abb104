// build.cu -- construction of the block-decomposition index.
//
// The reference builds, for RTX_blocks, one triangle per element plus one
// per block minimum and hands them to the OptiX BVH builder
// (src/device_tools.cuh:139-169, 243-253, src/rtx.h:3-22, 39-99). GB300 has
// no RT cores, so the search structure is rebuilt as arrays a query can index
// directly:
//   pre[i]  = leftmost minimum of A[blockstart(i) .. i]
//   suf[i]  = leftmost minimum of A[i .. blockend(i)]
//   st[k][j]= leftmost minimum of blocks j .. j + 2^k - 1 (k = 0: block minima)
// One CTA owns a "unit": one block when blocks are large, or G whole blocks
// (G * bs <= 4096 elements) when they are small. A unit is streamed in
// 4096-element tiles (16 consecutive floats per thread, float4 loads):
// suffix pass right-to-left, then prefix pass left-to-right, each tile a
// thread-local scan plus a CTA-wide scan, carried across tiles. Results are
// staged in shared memory and written with coalesced stores.
//
// Segmented scans without flags: every element is turned into one 64-bit
// composite  [segment rank | fkey(value) | local index | -0.0 bit]  whose
// unsigned minimum is the leftmost minimum. In the prefix direction earlier
// blocks of the unit get a larger rank, in the suffix direction later blocks
// do, so a plain min-scan over the unit restarts at every block boundary.
#include "engine.h"

namespace rmq {
namespace {

constexpr int kThreads = 256;
constexpr int kEPT = 16;                      // elements per thread per tile
constexpr int kTile = kThreads * kEPT;        // 4096
constexpr int kWarps = kThreads / 32;
constexpr uint32_t kUnitTarget = 4096;        // elements per multi-block unit

struct UnitLayout {
    uint32_t G;           // blocks per unit
    uint32_t key_shift;   // 32 when G == 1, else 17
    uint32_t seg_shift;   // 49 when G > 1 (unused otherwise)
    uint32_t local_mask;  // 0x7fffffff when G == 1, else 0xffff
};

__device__ __forceinline__ uint64_t make_comp(uint32_t bits, uint32_t local, uint32_t segf,
                                              const UnitLayout &U) {
    const uint64_t nz = (bits == 0x80000000u) ? 1ull : 0ull;
    return (static_cast<uint64_t>(segf) << U.seg_shift) |
           (static_cast<uint64_t>(fkey(bits)) << U.key_shift) |
           (static_cast<uint64_t>(local) << 1) | nz;
}

__device__ __forceinline__ Entry decode(uint64_t c, uint32_t ustart, const UnitLayout &U) {
    Entry e;
    const uint32_t key = static_cast<uint32_t>(c >> U.key_shift);
    e.bits = funkey(key, static_cast<uint32_t>(c & 1ull));
    e.idx = ustart + (static_cast<uint32_t>(c >> 1) & U.local_mask);
    return e;
}

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return b < a ? b : a; }

// Exclusive min-scan of one value per thread across the CTA, in thread order
// (REV = false) or reverse thread order (REV = true). `total` receives the
// CTA-wide minimum.
template <bool REV>
__device__ __forceinline__ uint64_t cta_exclusive_min(uint64_t v, uint64_t *s_warp,
                                                      uint64_t &total) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    uint64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t t = REV ? __shfl_down_sync(0xffffffffu, inc, o)
                               : __shfl_up_sync(0xffffffffu, inc, o);
        const bool ok = REV ? (lane + o < 32) : (lane >= o);
        if (ok) inc = umin64(inc, t);
    }
    uint64_t ex = REV ? __shfl_down_sync(0xffffffffu, inc, 1)
                      : __shfl_up_sync(0xffffffffu, inc, 1);
    if (REV ? (lane == 31) : (lane == 0)) ex = ~0ull;
    if (REV ? (lane == 0) : (lane == 31)) s_warp[warp] = inc;
    __syncthreads();
    uint64_t wex = ~0ull, tot = ~0ull;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        const uint64_t s = s_warp[w];
        tot = umin64(tot, s);
        if (REV ? (w > warp) : (w < warp)) wex = umin64(wex, s);
    }
    total = tot;
    __syncthreads();
    return umin64(ex, wex);
}

template <bool ALIGNED>
__global__ void __launch_bounds__(kThreads)
build_units_kernel(BuildPlan p, UnitLayout U, Div31 dv, uint32_t nunits) {
    __shared__ Entry stage[kTile + kTile / 16];
    __shared__ uint64_t s_warp[kWarps];

    for (uint32_t u = blockIdx.x; u < nunits; u += gridDim.x) {
        const uint32_t ustart = u * U.G * p.bs;
        const uint32_t uend = min(ustart + U.G * p.bs, p.n);
        const uint32_t t_first = ALIGNED ? (ustart & ~3u) : ustart;
        const uint32_t ntiles = (uend - t_first + kTile - 1) / kTile;

#pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
            const bool suffix = (pass == 0);
            uint64_t carry = ~0ull;
#pragma unroll 1
            for (uint32_t tt = 0; tt < ntiles; ++tt) {
                const uint32_t t = suffix ? (ntiles - 1 - tt) : tt;
                const uint32_t t0 = t_first + t * kTile;
                const uint32_t base = t0 + threadIdx.x * kEPT;

                uint32_t bits[kEPT];
                if (ALIGNED && base + kEPT <= p.n) {
                    const float4 *src = reinterpret_cast<const float4 *>(p.A + base);
#pragma unroll
                    for (int v = 0; v < kEPT / 4; ++v) {
                        const float4 f = __ldg(src + v);
                        bits[4 * v + 0] = __float_as_uint(f.x);
                        bits[4 * v + 1] = __float_as_uint(f.y);
                        bits[4 * v + 2] = __float_as_uint(f.z);
                        bits[4 * v + 3] = __float_as_uint(f.w);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < kEPT; ++j) {
                        const uint32_t g = base + j;
                        bits[j] = (g < p.n) ? __float_as_uint(__ldg(p.A + g)) : 0u;
                    }
                }

                uint64_t c[kEPT];
#pragma unroll
                for (int j = 0; j < kEPT; ++j) {
                    const uint32_t g = base + j;
                    if (g >= ustart && g < uend) {
                        const uint32_t local = g - ustart;
                        uint32_t segf = 0;
                        if (U.G > 1) {
                            const uint32_t seg = div31(local, dv);
                            segf = suffix ? seg : (U.G - 1 - seg);
                        }
                        c[j] = make_comp(bits[j], local, segf, U);
                    } else {
                        c[j] = ~0ull;
                    }
                }
                uint64_t agg;
                if (suffix) {
#pragma unroll
                    for (int j = kEPT - 2; j >= 0; --j) c[j] = umin64(c[j], c[j + 1]);
                    agg = c[0];
                } else {
#pragma unroll
                    for (int j = 1; j < kEPT; ++j) c[j] = umin64(c[j], c[j - 1]);
                    agg = c[kEPT - 1];
                }
                uint64_t total;
                uint64_t ex = suffix ? cta_exclusive_min<true>(agg, s_warp, total)
                                     : cta_exclusive_min<false>(agg, s_warp, total);
                ex = umin64(ex, carry);
                carry = umin64(carry, total);

#pragma unroll
                for (int j = 0; j < kEPT; ++j)
                    stage[threadIdx.x * (kEPT + 1) + j] = decode(umin64(c[j], ex), ustart, U);
                __syncthreads();

                Entry *out = suffix ? p.suf : p.pre;
#pragma unroll 4
                for (int k = 0; k < kEPT; ++k) {
                    const uint32_t e = threadIdx.x + k * kThreads;
                    const uint32_t g = t0 + e;
                    if (g >= ustart && g < uend) {
                        const Entry en = stage[e + (e >> 4)];
                        __stcs(reinterpret_cast<uint2 *>(out + g), make_uint2(en.bits, en.idx));
                        if (!suffix) {
                            // block minimum = prefix minimum at the block's last element
                            const uint32_t local = g - ustart;
                            bool last = (g + 1 == uend);
                            uint32_t seg = 0;
                            if (U.G > 1) {
                                seg = div31(local, dv);
                                last = last || (local + 1 == (seg + 1) * p.bs);
                            }
                            if (last) p.st[u * U.G + seg] = en;
                        }
                    }
                }
                __syncthreads();
            }
        }
    }
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

}  // namespace

uint32_t st_levels(uint32_t nb) { return nb ? static_cast<uint32_t>(ilog2(nb)) + 1u : 0u; }

cudaError_t launch_build(const BuildPlan &p, const DeviceInfo &dev, cudaStream_t s) {
    if (p.n == 0) return cudaSuccess;
    UnitLayout U;
    U.G = (p.bs >= kUnitTarget) ? 1u : (kUnitTarget / p.bs);
    if (U.G > p.nb) U.G = p.nb;
    if (U.G <= 1) {
        U.G = 1;
        U.key_shift = 32;
        U.seg_shift = 63;
        U.local_mask = 0x7fffffffu;
    } else {
        U.key_shift = 17;
        U.seg_shift = 49;
        U.local_mask = 0xffffu;
    }
    const uint32_t nunits = (p.nb + U.G - 1) / U.G;
    const Div31 dv = make_div31(p.bs);

    int per_sm = 0;
    cudaError_t err;
    if (p.aligned)
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_units_kernel<true>,
                                                            kThreads, 0);
    else
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, build_units_kernel<false>,
                                                            kThreads, 0);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) per_sm = 1;
    uint32_t grid = static_cast<uint32_t>(dev.sms) * static_cast<uint32_t>(per_sm);
    if (grid > nunits) grid = nunits;
    if (p.aligned)
        build_units_kernel<true><<<grid, kThreads, 0, s>>>(p, U, dv, nunits);
    else
        build_units_kernel<false><<<grid, kThreads, 0, s>>>(p, U, dv, nunits);
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
