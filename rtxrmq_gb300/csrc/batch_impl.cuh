// batch_impl.cuh -- the persistent batch kernels, shared by batch.cu (full
// index: per-element prefix / suffix entries) and batch_light.cu (light
// index: block and micro-block tables only). Each translation unit
// instantiates only its own kernels.
//
// Persistent kernel, three phases separated by grid-wide barriers of a
// cooperative launch (all CTAs are co-resident, guaranteed by the launch):
//   A  build items. Full: (array, unit) prefix/suffix minima + block minima,
//      the plain builder's CTA body (build_impl.cuh). Light: (array, tile)
//      micro-block minima, every micro-table level and the block minima of
//      a tile, from one read of its values (light_tile); for block sizes
//      above 65536, (array, chunk) micro-block minima only;
//   B  table items (array, kind | level, first entry, count), one step per
//      barrier: block-table level k at step k (at step k + 1 when step 1
//      computes the block minima from the micro-block minima), and for
//      untiled light arrays micro-table level k at step k;
//   C  query items (array, first query, count), query_impl.cuh's queued
//      form (light: misses settle from value lines, no entries).
// Work lists are built on the host once per plan, so a run allocates nothing
// and can be captured in a CUDA graph.
#pragma once

#include <cooperative_groups.h>

#include "build_impl.cuh"
#include "engine.h"
#include "query_impl.cuh"

// CTAs per SM the persistent batch kernels are compiled for (a register bound).
#ifndef RMQ_BATCH_MINB
#define RMQ_BATCH_MINB 4
#endif
#ifndef RMQ_BATCH_LIGHT_MINB
#define RMQ_BATCH_LIGHT_MINB 3  // the light-index kernels
#endif

namespace rmq {

constexpr int kBatchThreads = kBuildThreads;  // phase A runs the unit builder
constexpr int kBatchQPT = 2;
// default tile schedule: queries per query item, table entries per level
// item (a plan can set both per size bucket, rmq_batch_create_ex)
constexpr uint32_t kQueryChunk = 2048;
constexpr uint32_t kLevelChunk = 4096;
constexpr int kMaxLevels = 32;
// micro-blocks per light build item: 16 per warp of the CTA
constexpr uint32_t kLightChunk = kMicroPerWarp * (kBatchThreads / 32);

// kinds of table items (bits 16.. of the item's second word; bits 0..15
// hold the level)
enum : uint32_t {
    kItemBlockLevel = 0,   // block-table level k from level k - 1
    kItemBlockMinima = 1,  // block-table level 0 from the micro-block minima
    kItemMicroLevel = 2,   // micro-table level k from level k - 1
};
// Light tiles (phase A items of a light array whose micro table is shallow
// enough): kMicroTile (or kMicroTileSmall) micro-blocks whose minima, every
// micro-table level and the minima of the blocks inside come from one read
// of the tile's values plus a halo of 2^(mlevels - 1) - 1 micro-blocks. The
// levels are built in two shared-memory buffers of kTileEntries minima each,
// so tile + halo <= kTileEntries: tiles of 2048 up to bs 32768, of 1024 at
// bs 65536. Other light arrays take chunks in phase A and one table item
// per level.
constexpr uint32_t kMicroTile = 2048;
constexpr uint32_t kMicroTileSmall = 1024;
// BatchArray::light_flags
constexpr uint32_t kLightTiled = 1;       // phase A items are tiles
constexpr uint32_t kLightTileBmin = 2;    // tiles also write the block minima (bs / 32 divides the tile)
constexpr uint32_t kLightSmallTile = 4;   // tiles of kMicroTileSmall

struct BatchArray {
    int64_t off;    // first value in the buffer
    int64_t qoff;   // first query
    int64_t pre;    // workspace entry offset of pre[]; suf[] follows at pre + n (full)
    int64_t st;     // workspace entry offset of the sparse table
    int64_t mst;    // workspace entry offset of the micro-block minima (light)
    int64_t moff;   // workspace entry offset of the micro-table offsets (light)
    uint32_t n, bs, nb, levels;
    uint32_t nmicro, mlevels, moff_bytes, light_flags;
    UnitLayout U;
    Div31 dv;
};

struct BatchParams {
    const float *A;
    int64_t limit;
    const int2 *Q;
    float *val;
    int32_t *idx;
    unsigned long long *invalid;
    Entry *ws;
    const BatchArray *arrays;
    const uint2 *build;
    int32_t nbuild;
    const uint4 *lvl;
    int32_t maxlev;   // table steps run: 1 .. maxlev - 1
    int32_t lvl_start[kMaxLevels + 1];
    const uint4 *qitems;
    int32_t nqitems;
    int64_t total_q;  // one past the last query any array owns
    uint32_t phases;  // bit 0 build, bit 1 table levels, bit 2 queries
};

// Dynamic shared memory of a light batch CTA: the warps' miss queues, then
// every thread's line slot (kLineChunks 16-byte chunks).
constexpr size_t kLightQueueBytes = sizeof(MissQueue) * (kBatchThreads / 32);
constexpr size_t kLightSmemBytes =
    kLightQueueBytes + sizeof(uint4) * kLineChunks * static_cast<size_t>(kBatchThreads);
static_assert(kLightQueueBytes % 16 == 0, "line slots start 16-byte aligned");
// minima per buffer of a light tile (two buffers)
constexpr uint32_t kTileEntries = static_cast<uint32_t>(kLightSmemBytes / (2 * sizeof(Entry)));
static_assert(kTileEntries >= kMicroTile + 1023 && kTileEntries >= kMicroTileSmall + 2047,
              "tiles of 2048 up to bs 32768 and of 1024 at bs 65536 fit");

// Light kernels (batch_light.cu): the instantiation for (aligned, key mode),
// its dynamic shared memory and CTAs per SM (the dynamic-memory limit set).
cudaError_t batch_light_kernel(bool aligned, uint32_t mode, const void **fn, size_t *smem,
                               int *per_sm);

namespace {

namespace cg = cooperative_groups;

template <bool LIGHT, uint32_t MODE>
__device__ __forceinline__ V1View batch_view(const BatchParams &P, const BatchArray &a) {
    V1View v;
    v.A = P.A;
    v.off = a.off;
    v.limit = P.limit;
    v.n = a.n;
    v.bs = a.bs;
    v.nb = a.nb;
    v.dv = a.dv;
    v.st = P.ws + a.st;
    v.kmode = MODE;
    v.levels = a.levels;
    v.mpre = nullptr;
    v.msuf = nullptr;
    if (LIGHT) {
        v.pre = nullptr;
        v.suf = nullptr;
        v.mst = P.ws + a.mst;
        v.moff = P.ws + a.moff;
        v.moff_bytes = a.moff_bytes;
        v.nmicro = a.nmicro;
        v.mlevels = a.mlevels;
        v.micro_span = (1u << a.mlevels) - 1u;
    } else {
        // full batched arrays answer same-block queries with warp scans
        v.pre = P.ws + a.pre;
        v.suf = P.ws + a.pre + a.n;
        v.mst = nullptr;
        v.moff = nullptr;
        v.moff_bytes = 0u;
        v.nmicro = 0;
        v.mlevels = 0u;
        v.micro_span = 0u;
    }
    return v;
}

template <uint32_t MODE>
__device__ __forceinline__ UnitJob unit_job(const BatchParams &P, uint32_t array) {
    const BatchArray a = P.arrays[array];
    UnitJob J;
    J.A = P.A;
    J.off = a.off;
    J.limit = P.limit;
    J.n = a.n;
    J.bs = a.bs;
    J.U = a.U;
    J.dv = a.dv;
    J.pre = P.ws + a.pre;
    J.suf = P.ws + a.pre + a.n;
    J.bmin = P.ws + a.st;
    J.kmode = MODE;
    J.nb = a.nb;
    return J;
}

// Light phase A: minima of micro-blocks [c * kLightChunk, ...) of one array,
// kMicroPerWarp per warp.
template <bool ALIGNED, uint32_t MODE>
__device__ __forceinline__ void light_chunk(const BatchParams &P, const BatchArray &a,
                                            uint32_t c) {
    const uint32_t j0 = c * kLightChunk + (threadIdx.x >> 5) * kMicroPerWarp;
    if (j0 >= a.nmicro) return;  // whole warp
    const float *A = P.A + a.off;
    Entry m[4];
    // whole rows inside the array, 16-byte aligned
    if (ALIGNED && a.off % 4 == 0 && (j0 + kMicroPerWarp) * kMicroElems <= a.n)
        micro_min_warp<MODE, true>(A, a.n, j0, a.nmicro, P.ws + a.mst, 0u, m);
    else
        micro_min_warp<MODE, false>(A, a.n, j0, a.nmicro, P.ws + a.mst, 0u, m);
}

// Light table step, kind kItemBlockMinima: block minima of blocks [first,
// first + count) from the micro-block minima (bs / 32 per block): a thread
// per block for small blocks, a warp per block otherwise.
__device__ __forceinline__ void light_block_minima(const BatchParams &P, const BatchArray &a,
                                                   uint32_t first, uint32_t count) {
    const Entry *mst = P.ws + a.mst;
    Entry *bmin = P.ws + a.st;
    const uint32_t pb = a.bs / kMicroElems;
    if (pb <= 16u) {
        for (uint32_t b = first + threadIdx.x; b < first + count; b += kBatchThreads) {
            Entry m = kEntryNone;
            const uint32_t j1 = min(b * pb + pb, a.nmicro);
            for (uint32_t j = b * pb; j < j1; ++j) m = better(m, mst[j]);
            if (rmq_chk(b < a.nb)) bmin[b] = m;
        }
        return;
    }
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t b = first + (threadIdx.x >> 5); b < first + count; b += kBatchThreads / 32) {
        Entry m = kEntryNone;
        const uint32_t j1 = min(b * pb + pb, a.nmicro);
        for (uint32_t j = b * pb + lane; j < j1; j += 32u) m = better(m, mst[j]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = better(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0u && rmq_chk(b < a.nb)) bmin[b] = m;
    }
}

template <class O>
__device__ __forceinline__ void light_micro_level_w(const BatchParams &P, const BatchArray &a,
                                                    uint32_t k, uint32_t first, uint32_t count) {
    O *off = reinterpret_cast<O *>(P.ws + a.moff);
    O *__restrict__ cur = off + static_cast<size_t>(k - 1) * a.nmicro;
    const O *__restrict__ prev = off + static_cast<size_t>(k >= 2 ? k - 2 : 0) * a.nmicro;
    for (uint32_t i = first + threadIdx.x; i < first + count; i += kBatchThreads)
        micro_level_at(P.ws + a.mst, cur, prev, a.nmicro, k, i);
}

// Every level 1 .. mlevels - 1 of the micro table at positions [t0, t0 +
// count) from the minima src[0 .. e) of micro-blocks [t0, t0 + e) in shared
// memory. Level k holds the best minimum of every window of 2^k micro-blocks
// whose window lies in the loaded range (the better of the level below's two
// halves), written to the other buffer; the offset stored is that minimum's
// micro-block (its element index / 32) minus the window's first. One barrier
// per level.
template <class O>
__device__ __forceinline__ void micro_tile_levels(const BatchParams &P, const BatchArray &a,
                                                  uint32_t t0, uint32_t count, uint32_t e,
                                                  Entry *src, Entry *dst) {
    O *off = reinterpret_cast<O *>(P.ws + a.moff);
    for (uint32_t k = 1; k < a.mlevels && (1u << k) <= e; ++k) {
        const uint32_t half = 1u << (k - 1);
        const uint32_t valid = e - (1u << k) + 1;  // windows inside the loaded range
        O *__restrict__ row = off + static_cast<size_t>(k - 1) * a.nmicro + t0;
        for (uint32_t i = threadIdx.x; i < valid; i += kBatchThreads) {
            const Entry m = better(src[i], src[i + half]);
            dst[i] = m;
            if (i < count) row[i] = static_cast<O>((entry_idx(m) >> 5) - (t0 + i));
        }
        __syncthreads();
        Entry *t = src;
        src = dst;
        dst = t;
    }
}

// Light phase A, one tile (kLightTiled arrays): the minima of micro-blocks
// [t0, t0 + count + halo) from the values into shared memory (8 rows of 512
// bytes per warp step, all loads in flight), the tile's own minima to the
// micro-block minima table, the minima of the blocks inside the tile
// (kLightTileBmin), and every micro-table level at [t0, t0 + count). The
// halo's minima are computed again by the next tile.
template <bool ALIGNED, uint32_t MODE, class O>
__device__ __forceinline__ void light_tile(const BatchParams &P, const BatchArray &a, uint32_t t,
                                           unsigned char *smem) {
    Entry *key = reinterpret_cast<Entry *>(smem);
    const uint32_t tile = (a.light_flags & kLightSmallTile) ? kMicroTileSmall : kMicroTile;
    const uint32_t t0 = t * tile;
    const uint32_t count = min(tile, a.nmicro - t0);
    const uint32_t halo = (1u << (a.mlevels - 1)) - 1u;
    const uint32_t jend = min(t0 + count + halo, a.nmicro);
    const uint32_t e = jend - t0;  // minima held in shared memory (<= kTileEntries)
    const float *A = P.A + a.off;
    const bool vec = ALIGNED && a.off % 4 == 0;
    // 8 rows (32 micro-blocks, 4 KB) per warp step: 96 KB of loads in flight per SM
    constexpr uint32_t kRows = 8, kPerWarp = 4 * kRows;
    for (uint32_t j0 = t0 + (threadIdx.x >> 5) * kPerWarp; j0 < jend;
         j0 += kPerWarp * (kBatchThreads / 32)) {
        if (vec && (j0 + kPerWarp) * kMicroElems <= a.n)
            micro_min_rows<MODE, true, kRows>(A, a.n, j0, jend, key, t0);
        else
            micro_min_rows<MODE, false, kRows>(A, a.n, j0, jend, key, t0);
    }
    __syncthreads();
    Entry *mst = P.ws + a.mst;
    for (uint32_t i = threadIdx.x; i < count; i += kBatchThreads) mst[t0 + i] = key[i];
    if (a.light_flags & kLightTileBmin) {
        // blocks [t0 / pb, (t0 + count - 1) / pb], all inside the tile
        const uint32_t pb = a.bs / kMicroElems;
        const uint32_t b0 = t0 / pb, nbt = (count + pb - 1) / pb;
        Entry *bmin = P.ws + a.st;
        if (pb <= 16u) {
            for (uint32_t x = threadIdx.x; x < nbt; x += kBatchThreads) {
                Entry mm = kEntryNone;
                const uint32_t j1 = min(x * pb + pb, count);
                for (uint32_t j = x * pb; j < j1; ++j) mm = better(mm, key[j]);
                if (rmq_chk(b0 + x < a.nb)) bmin[b0 + x] = mm;
            }
        } else {
            const uint32_t lane = threadIdx.x & 31u;
            for (uint32_t x = threadIdx.x >> 5; x < nbt; x += kBatchThreads / 32) {
                Entry mm = kEntryNone;
                const uint32_t j1 = min(x * pb + pb, count);
                for (uint32_t j = x * pb + lane; j < j1; j += 32u) mm = better(mm, key[j]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) mm = better(mm, __shfl_xor_sync(0xffffffffu, mm, o));
                if (lane == 0u && rmq_chk(b0 + x < a.nb)) bmin[b0 + x] = mm;
            }
        }
    }
    // the levels write only the second buffer first; the block minima and
    // the table copy above read the first
    micro_tile_levels<O>(P, a, t0, count, e, key, key + kTileEntries);
    __syncthreads();  // the next tile overwrites both buffers
}

// Phase B: table steps 1 .. maxlev - 1, a grid barrier after each.
template <bool LIGHT>
__device__ __forceinline__ void table_steps(const BatchParams &P, cg::grid_group &grid) {
    for (int s = 1; (P.phases & 2u) && s < P.maxlev; ++s) {
        for (int32_t it = P.lvl_start[s] + blockIdx.x; it < P.lvl_start[s + 1]; it += gridDim.x) {
            const uint4 w = P.lvl[it];
            const BatchArray &a = P.arrays[w.x];
            const uint32_t kind = w.y >> 16, k = w.y & 0xffffu;
            if (LIGHT && kind == kItemBlockMinima) {
                light_block_minima(P, a, w.z, w.w);
            } else if (LIGHT && kind == kItemMicroLevel) {
                if (a.moff_bytes == 1u)
                    light_micro_level_w<uint8_t>(P, a, k, w.z, w.w);
                else if (a.moff_bytes == 2u)
                    light_micro_level_w<uint16_t>(P, a, k, w.z, w.w);
                else
                    light_micro_level_w<uint32_t>(P, a, k, w.z, w.w);
            } else {
                const Entry *__restrict__ prev = P.ws + a.st + static_cast<int64_t>(k - 1) * a.nb;
                Entry *__restrict__ cur = P.ws + a.st + static_cast<int64_t>(k) * a.nb;
                const uint32_t half = 1u << (k - 1);
                for (uint32_t j = w.z + threadIdx.x; j < w.z + w.w; j += kBatchThreads)
                    if (rmq_chk(j + half < a.nb)) cur[j] = better(prev[j], prev[j + half]);
            }
        }
        grid.sync();
    }
}

// Phase C: the query items, in the queued form.
template <bool ALIGNED, bool LIGHT, uint32_t MODE>
__device__ __forceinline__ void query_items(const BatchParams &P, MissQueue &mq, uint4 *lines) {
    for (int32_t it = (P.phases & 4u) ? blockIdx.x : P.nqitems; it < P.nqitems; it += gridDim.x) {
        const uint4 w = P.qitems[it];
        const BatchArray a = P.arrays[w.x];
        const V1View v = batch_view<LIGHT, MODE>(P, a);
        QueryOut o;
        o.Q = P.Q + a.qoff;
        o.val = P.val ? P.val + a.qoff : nullptr;
        o.idx = P.idx ? P.idx + a.qoff : nullptr;
        o.invalid = P.invalid;
        o.span = P.total_q - a.qoff;
        answer_range_queued<ALIGNED, LIGHT, LIGHT, MODE, kBatchThreads, kBatchQPT>(
            v, o, w.y, static_cast<int64_t>(w.y) + w.z, mq, lines);
    }
}

// Full index: prefix / suffix entries per element, warp scans for queries
// inside one block.
template <bool ALIGNED, uint32_t MODE>
__global__ void __launch_bounds__(kBatchThreads, RMQ_BATCH_MINB) batch_kernel(BatchParams P) {
    __shared__ Entry stage[kStageEntries];
    __shared__ uint64_t s_warp[kWarpSlots];
    __shared__ uint32_t s_flag[2 * kBuildWarps];
    cg::grid_group grid = cg::this_grid();

    // A: units
    for (int32_t it = (P.phases & 1u) ? blockIdx.x : P.nbuild; it < P.nbuild; it += gridDim.x) {
        const uint2 w = P.build[it];
        build_unit<ALIGNED, MODE>(unit_job<MODE>(P, w.x), w.y, stage, s_warp, s_flag);
    }
    grid.sync();
    table_steps<false>(P, grid);
    // C: the warps' miss queues live in the staging memory of phase A
    static_assert(sizeof(MissQueue) * (kBatchThreads / 32) <= sizeof(Entry) * kStageEntries,
                  "miss queues fit the staging memory");
    MissQueue &mq = reinterpret_cast<MissQueue *>(stage)[threadIdx.x >> 5];
    query_items<ALIGNED, false, MODE>(P, mq, nullptr);
}

// Light index: block and micro-block tables only. Dynamic shared memory
// (kLightSmemBytes): miss queues, then the threads' line slots.
template <bool ALIGNED, uint32_t MODE>
__global__ void __launch_bounds__(kBatchThreads, RMQ_BATCH_LIGHT_MINB)
batch_kernel_light(BatchParams P) {
    extern __shared__ __align__(16) unsigned char s_light[];
    cg::grid_group grid = cg::this_grid();

    // A: tiles (micro-block minima, micro table, block minima) or chunks
    // (micro-block minima only)
    for (int32_t it = (P.phases & 1u) ? blockIdx.x : P.nbuild; it < P.nbuild; it += gridDim.x) {
        const uint2 w = P.build[it];
        const BatchArray &a = P.arrays[w.x];
        if (!(a.light_flags & kLightTiled))
            light_chunk<ALIGNED, MODE>(P, a, w.y);
        else if (a.moff_bytes == 1u)
            light_tile<ALIGNED, MODE, uint8_t>(P, a, w.y, s_light);
        else
            light_tile<ALIGNED, MODE, uint16_t>(P, a, w.y, s_light);
    }
    grid.sync();
    table_steps<true>(P, grid);
    MissQueue &mq = reinterpret_cast<MissQueue *>(s_light)[threadIdx.x >> 5];
    uint4 *lines = reinterpret_cast<uint4 *>(s_light + kLightQueueBytes);
    query_items<ALIGNED, true, MODE>(P, mq, lines);
}

}  // namespace
}  // namespace rmq
