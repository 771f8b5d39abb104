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

// CTAs per SM the unit kernel is compiled for (a register bound).
#ifndef RMQ_BUILD_MINB
#define RMQ_BUILD_MINB 4
#endif

namespace rmq {
namespace {

template <bool ALIGNED, uint32_t MODE>
__global__ void __launch_bounds__(kBuildThreads, RMQ_BUILD_MINB)
build_units_kernel(UnitJob J, uint32_t nunits) {
    __shared__ Entry stage[kStageEntries];
    __shared__ uint64_t s_warp[kWarpSlots];
    __shared__ uint32_t s_flag[2 * kBuildWarps];
    for (uint32_t u = blockIdx.x; u < nunits; u += gridDim.x)
        build_unit<ALIGNED, MODE>(J, u, stage, s_warp, s_flag);
}

template <bool ALIGNED>
void launch_units(const UnitJob &J, uint32_t nunits, uint32_t grid, cudaStream_t s) {
    switch (J.kmode) {
    case kFloatMax: build_units_kernel<ALIGNED, kFloatMax><<<grid, kBuildThreads, 0, s>>>(J, nunits); break;
    case kIntMin: build_units_kernel<ALIGNED, kIntMin><<<grid, kBuildThreads, 0, s>>>(J, nunits); break;
    case kIntMax: build_units_kernel<ALIGNED, kIntMax><<<grid, kBuildThreads, 0, s>>>(J, nunits); break;
    default: build_units_kernel<ALIGNED, kFloatMin><<<grid, kBuildThreads, 0, s>>>(J, nunits); break;
    }
}

__global__ void st_level_kernel(Entry *st, uint32_t nb, uint32_t k) {
    const Entry *prev = st + static_cast<size_t>(k - 1) * nb;
    Entry *cur = st + static_cast<size_t>(k) * nb;
    const uint32_t half = 1u << (k - 1);
    const uint32_t cnt = nb - (1u << k) + 1;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < cnt;
         j += gridDim.x * blockDim.x)
        if (rmq_chk(j + half < nb)) cur[j] = better(prev[j], prev[j + half]);
}

// Level k >= 1 of the micro table as offsets (micro_level_at).
template <class O>
__global__ void micro_level_kernel(const Entry *__restrict__ mst0, O *off, uint32_t nmicro,
                                   uint32_t k) {
    const uint32_t cnt = nmicro - (1u << k) + 1;
    O *cur = off + static_cast<size_t>(k - 1) * nmicro;
    const O *prev = off + static_cast<size_t>(k >= 2 ? k - 2 : 0) * nmicro;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt;
         i += gridDim.x * blockDim.x)
        micro_level_at(mst0, cur, prev, nmicro, k, i);
}

// Sub-block level: 8 lanes per 32-element micro-block, 4 consecutive
// elements per lane (one 16-byte load), 4 micro-blocks per warp. Each lane
// scans its 4 elements both ways, then the 8 lanes of a micro-block scan
// their totals with width-8 shuffles; results are written as two 16-byte
// stores per lane and array, and the micro-block minimum (suffix minimum at
// its first element) as level 0 of the micro table.
template <uint32_t MODE>
__global__ void __launch_bounds__(256)
micro_scan_kernel(const float *__restrict__ A, uint32_t n, uint32_t nmicro, Entry *mpre,
                  Entry *msuf, Entry *mst0, bool aligned) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t sub = lane & 7u;        // lane within its micro-block
    const uint32_t grp = lane >> 3;        // micro-block within the warp
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w * 4u < nmicro;
         w += warps) {
        const uint32_t j = w * 4u + grp;
        const uint32_t g0 = j * kMicro + sub * 4u;   // may pass n (then nothing is valid)
        uint32_t b[4];
        if (aligned && g0 + 3u < n) {
            const uint4 f = ld_u4(A + g0);
            b[0] = f.x;
            b[1] = f.y;
            b[2] = f.z;
            b[3] = f.w;
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) b[k] = (g0 + k < n) ? ld_u1(A + g0 + k) : 0u;
        }
        Entry p[4], q[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) p[k] = (g0 + k < n) ? make_entry(b[k], g0 + k, MODE) : kEntryNone;
        q[3] = p[3];
#pragma unroll
        for (int k = 2; k >= 0; --k) q[k] = better(p[k], q[k + 1]);
#pragma unroll
        for (int k = 1; k < 4; ++k) p[k] = better(p[k - 1], p[k]);
        // lane totals scanned across the 8 lanes of the micro-block
        Entry ip = p[3], is = q[0];
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const Entry tp = __shfl_up_sync(0xffffffffu, ip, o, 8);
            const Entry ts = __shfl_down_sync(0xffffffffu, is, o, 8);
            if (sub >= static_cast<uint32_t>(o)) ip = better(ip, tp);
            if (sub + o < 8u) is = better(is, ts);
        }
        Entry ep = __shfl_up_sync(0xffffffffu, ip, 1, 8);
        Entry es = __shfl_down_sync(0xffffffffu, is, 1, 8);
        if (sub == 0u) ep = kEntryNone;
        if (sub == 7u) es = kEntryNone;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            p[k] = better(ep, p[k]);
            q[k] = better(es, q[k]);
        }
        if (j < nmicro) {
            if (g0 + 3u < n) {
                __stcs(reinterpret_cast<ulonglong2 *>(mpre + g0), make_ulonglong2(p[0], p[1]));
                __stcs(reinterpret_cast<ulonglong2 *>(mpre + g0 + 2), make_ulonglong2(p[2], p[3]));
                __stcs(reinterpret_cast<ulonglong2 *>(msuf + g0), make_ulonglong2(q[0], q[1]));
                __stcs(reinterpret_cast<ulonglong2 *>(msuf + g0 + 2), make_ulonglong2(q[2], q[3]));
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (g0 + k < n) {
                        st_entry(mpre + g0 + k, p[k]);
                        st_entry(msuf + g0 + k, q[k]);
                    }
            }
            if (sub == 0u) mst0[j] = q[0];
        }
    }
}

// Light index, one pass over the values: the minimum of every 32-element
// micro-block (level 0 of the micro table) and, folded in with a 64-bit
// atomic minimum, of every block (level 0 of the block table, filled with
// all-ones before; bs a multiple of 32, so every micro-block lies in one
// block). A warp takes 16 consecutive micro-blocks per step: four 512-byte
// rows, each lane 4 consecutive elements of every row, all four loads in
// flight before any reduction; 8 lanes reduce one micro-block. When the 16
// micro-blocks lie in one block (bs a multiple of 512, or away from block
// edges) the warp folds them into that block with a single atomic.

template <uint32_t MODE>
__global__ void __launch_bounds__(256)
micro_min_kernel(const float *__restrict__ A, uint32_t n, uint32_t nmicro, uint32_t per_block,
                 Entry *mst0, Entry *bmin, bool aligned) {
    static_assert(kMicroElems == kMicro, "micro-block size");
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t sub = lane & 7u;
    const uint32_t grp = lane >> 3;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    const uint32_t nblocks = (nmicro + per_block - 1) / per_block;
    for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
         w * kMicroPerWarp < nmicro; w += warps) {
        const uint32_t j0 = w * kMicroPerWarp;
        Entry m[4];  // micro-block j0 + 4i + grp, on all 8 lanes of the group
        if (aligned && (j0 + kMicroPerWarp) * kMicro <= n)
            micro_min_warp<MODE, true>(A, n, j0, nmicro, mst0, 0u, m);
        else
            micro_min_warp<MODE, false>(A, n, j0, nmicro, mst0, 0u, m);
        const uint32_t jl = min(j0 + kMicroPerWarp, nmicro) - 1u;
        if (j0 / per_block == jl / per_block) {
            // one block: micro-blocks past nmicro hold kEntryNone, the identity
            Entry v = better(better(m[0], m[1]), better(m[2], m[3]));
            v = better(v, __shfl_xor_sync(0xffffffffu, v, 8));
            v = better(v, __shfl_xor_sync(0xffffffffu, v, 16));
            const uint32_t blk = j0 / per_block;
            if (lane == 0u && rmq_chk(blk < nblocks))
                atomicMin(reinterpret_cast<unsigned long long *>(bmin + blk),
                          static_cast<unsigned long long>(v));
        } else if (sub == 0u) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const uint32_t j = j0 + 4u * i + grp;
                const uint32_t blk = j / per_block;
                if (j < nmicro && rmq_chk(blk < nblocks))
                    atomicMin(reinterpret_cast<unsigned long long *>(bmin + blk),
                              static_cast<unsigned long long>(m[i]));
            }
        }
    }
}

std::atomic<int> g_units_per_sm[2];

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

template <class O>
cudaError_t launch_micro_levels_w(const BuildPlan &p, const DeviceInfo &dev, cudaStream_t s) {
    // bs <= n keeps every window inside the array (2^k <= nmicro); the
    // bound is checked here as well
    for (uint32_t k = 1; k < p.mlevels && (1u << k) <= p.nmicro; ++k) {
        const uint32_t cnt = p.nmicro - (1u << k) + 1;
        uint32_t g = (cnt + 255) / 256;
        const uint32_t cap = static_cast<uint32_t>(dev.sms) * 8u;
        if (g > cap) g = cap;
        micro_level_kernel<O><<<g, 256, 0, s>>>(p.mst, static_cast<O *>(p.moff), p.nmicro, k);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
    }
    return cudaSuccess;
}

cudaError_t launch_micro_levels(const BuildPlan &p, const DeviceInfo &dev, cudaStream_t s) {
    switch (p.moff_bytes) {
    case 1: return launch_micro_levels_w<uint8_t>(p, dev, s);
    case 2: return launch_micro_levels_w<uint16_t>(p, dev, s);
    default: return launch_micro_levels_w<uint32_t>(p, dev, s);
    }
}

}  // namespace

uint32_t st_levels(uint32_t nb) { return nb ? static_cast<uint32_t>(ilog2(nb)) + 1u : 0u; }

namespace {
size_t a256(size_t x) { return (x + 255) / 256 * 256; }
struct Offsets {
    size_t pre, suf, st, mst, moff, mpre, msuf, counter, total;
};
Offsets offsets_of(const BuildPlan &p) {
    Offsets o;
    const size_t nent = p.light ? 0 : a256(sizeof(Entry) * static_cast<size_t>(p.n));
    o.pre = 0;
    o.suf = nent;
    o.st = 2 * nent;
    o.mst = o.st + a256(sizeof(Entry) * static_cast<size_t>(p.nb) * p.levels);
    o.moff = o.mst + (p.micro ? a256(sizeof(Entry) * static_cast<size_t>(p.nmicro)) : 0);
    o.mpre = o.moff + (p.micro ? a256(static_cast<size_t>(p.moff_bytes) * p.nmicro *
                                      (p.mlevels - 1)) : 0);
    o.msuf = o.mpre + (p.micro ? nent : 0);
    o.counter = o.msuf + (p.micro ? nent : 0);
    o.total = o.counter + 256;
    return o;
}
}  // namespace

size_t plan_index(BuildPlan &p, bool no_micro) {
    p.nb = (p.n + p.bs - 1) / p.bs;
    p.levels = st_levels(p.nb);
    p.mlevels = no_micro ? 0u : micro_levels(p.bs);
    p.micro = p.mlevels > 0;
    p.nmicro = p.micro ? (p.n + kMicro - 1) / kMicro : 0u;
    p.moff_bytes = p.micro ? micro_offset_bytes(p.mlevels) : 0u;
    p.aligned = reinterpret_cast<uintptr_t>(p.A) % 16 == 0;
    return offsets_of(p).total;
}

unsigned long long *place_index(BuildPlan &p, void *base_v) {
    char *base = static_cast<char *>(base_v);
    const Offsets o = offsets_of(p);
    p.pre = p.light ? nullptr : reinterpret_cast<Entry *>(base + o.pre);
    p.suf = p.light ? nullptr : reinterpret_cast<Entry *>(base + o.suf);
    p.st = reinterpret_cast<Entry *>(base + o.st);
    p.mst = p.micro ? reinterpret_cast<Entry *>(base + o.mst) : nullptr;
    p.moff = p.micro ? static_cast<void *>(base + o.moff) : nullptr;
    p.mpre = p.micro && !p.light ? reinterpret_cast<Entry *>(base + o.mpre) : nullptr;
    p.msuf = p.micro && !p.light ? reinterpret_cast<Entry *>(base + o.msuf) : nullptr;
    return reinterpret_cast<unsigned long long *>(base + o.counter);
}

// The sub-block level works on 32-element micro-blocks aligned in the
// array, whatever the block size. A query first probes the micro table over
// every micro-block it touches (a superset of [l, r]; two windows of 2^k
// micro-blocks cover up to 2^(k+1) - 1 of them), so the table holds windows
// long enough for any query inside one block: a block touches bs/32
// micro-blocks when blocks start on micro-block boundaries (bs a multiple
// of 32), at most floor((bs + 30) / 32) + 1 otherwise.
uint32_t micro_levels(uint32_t bs) {
    if (bs < 2 * kMicro) return 0;
    const uint32_t touched = (bs % kMicro == 0) ? bs / kMicro : (bs + kMicro - 2) / kMicro + 1;
    return st_levels(touched);
}

cudaError_t launch_build_light(const BuildPlan &p, const DeviceInfo &dev, cudaStream_t s) {
    cudaError_t err = cudaMemsetAsync(p.st, 0xff, sizeof(Entry) * static_cast<size_t>(p.nb), s);
    if (err != cudaSuccess) return err;
    // 8 warps per CTA, kMicroPerWarp micro-blocks per warp step
    uint32_t g = (p.nmicro + 8 * kMicroPerWarp - 1) / (8 * kMicroPerWarp);
    const uint32_t cap = static_cast<uint32_t>(dev.sms) * 8u;
    if (g > cap) g = cap;
    const uint32_t per_block = p.bs / kMicro;
    switch (p.kmode) {
    case kFloatMax:
        micro_min_kernel<kFloatMax><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, per_block, p.mst, p.st,
                                                      p.aligned);
        break;
    case kIntMin:
        micro_min_kernel<kIntMin><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, per_block, p.mst, p.st,
                                                    p.aligned);
        break;
    case kIntMax:
        micro_min_kernel<kIntMax><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, per_block, p.mst, p.st,
                                                    p.aligned);
        break;
    default:
        micro_min_kernel<kFloatMin><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, per_block, p.mst, p.st,
                                                      p.aligned);
        break;
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    err = launch_levels(p.st, p.nb, p.levels, dev, s);
    if (err != cudaSuccess) return err;
    return launch_micro_levels(p, dev, s);
}

cudaError_t launch_build(const BuildPlan &p, const DeviceInfo &dev, cudaStream_t s) {
    if (p.n == 0) return cudaSuccess;
    if (p.light) return launch_build_light(p, dev, s);
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
    J.kmode = p.kmode;
    J.nb = p.nb;
    const uint32_t nunits = unit_count(p.nb, J.U);

    // every key mode compiles to the same resources; the float-min
    // instantiation stands for all four
    int per_sm;
    cudaError_t err =
        p.aligned ? occupancy_cached(build_units_kernel<true, kFloatMin>, kBuildThreads,
                                     g_units_per_sm[1], per_sm)
                  : occupancy_cached(build_units_kernel<false, kFloatMin>, kBuildThreads,
                                     g_units_per_sm[0], per_sm);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) per_sm = 1;
    uint32_t grid = static_cast<uint32_t>(dev.sms) * static_cast<uint32_t>(per_sm);
    if (grid > nunits) grid = nunits;
    if (p.aligned)
        launch_units<true>(J, nunits, grid, s);
    else
        launch_units<false>(J, nunits, grid, s);
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    err = launch_levels(p.st, p.nb, p.levels, dev, s);
    if (err != cudaSuccess || !p.micro) return err;

    uint32_t g = (p.nmicro + 31) / 32;  // 8 warps per CTA, 4 micro-blocks per warp
    const uint32_t cap = static_cast<uint32_t>(dev.sms) * 8u;
    if (g > cap) g = cap;
    switch (p.kmode) {
    case kFloatMax:
        micro_scan_kernel<kFloatMax><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, p.mpre, p.msuf, p.mst,
                                                       p.aligned);
        break;
    case kIntMin:
        micro_scan_kernel<kIntMin><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, p.mpre, p.msuf, p.mst,
                                                     p.aligned);
        break;
    case kIntMax:
        micro_scan_kernel<kIntMax><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, p.mpre, p.msuf, p.mst,
                                                     p.aligned);
        break;
    default:
        micro_scan_kernel<kFloatMin><<<g, 256, 0, s>>>(p.A, p.n, p.nmicro, p.mpre, p.msuf, p.mst,
                                                       p.aligned);
        break;
    }
    err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    return launch_micro_levels(p, dev, s);
}

RMQ_VIOLATIONS_READER(violations_build)

}  // namespace rmq
