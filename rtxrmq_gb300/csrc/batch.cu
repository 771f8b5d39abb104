// batch.cu -- many independent arrays of uneven length and their query sets
// answered by one persistent, cooperative launch (build + query), the same
// work as one plain build/query launch sequence per array, the gradient
// scatter of the differentiable range-min, and the per-size-bucket
// autotuner. The kernels are in batch_impl.cuh; this unit instantiates the
// full-index kernels, batch_light.cu the light-index ones.
//
// The reference has no batched form: rtx_rmq<T> (src/rtx.h:24-177) builds one
// structure for one array and launches one optixLaunch per batch of queries.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/rmq.h"
#include "batch_impl.cuh"

namespace rmq {
namespace {

constexpr int kThreads = kBatchThreads;

// grad_vals[off(a) + idx[q]] += grad_out[q] for every query q of array a
__global__ void __launch_bounds__(kThreads)
scatter_grad_kernel(const BatchArray *arrays, const uint4 *qitems, int32_t nqitems,
                    const int32_t *idx, const float *gout, float *gvals) {
    for (int32_t it = blockIdx.x; it < nqitems; it += gridDim.x) {
        const uint4 w = qitems[it];
        const int64_t qoff = arrays[w.x].qoff + w.y;
        const int64_t off = arrays[w.x].off;
        const uint32_t n = arrays[w.x].n;
        for (uint32_t j = threadIdx.x; j < w.z; j += kThreads) {
            // argmins outside the array (-1 for invalid queries) add nothing
            const int32_t li = idx[qoff + j];
            if (li >= 0 && static_cast<uint32_t>(li) < n) atomicAdd(gvals + off + li, gout[qoff + j]);
        }
    }
}

std::atomic<int> g_batch_per_sm[8];  // full kernels: (aligned, key mode)

template <bool ALIGNED, uint32_t MODE>
cudaError_t pick_full(const void **fn, int *per_sm) {
    *fn = reinterpret_cast<const void *>(batch_kernel<ALIGNED, MODE>);
    return occupancy_cached(batch_kernel<ALIGNED, MODE>, kThreads,
                            g_batch_per_sm[(ALIGNED ? 4 : 0) + MODE], *per_sm);
}

template <bool ALIGNED>
cudaError_t full_kernel_t(uint32_t mode, const void **fn, int *per_sm) {
    switch (mode) {
    case kFloatMax: return pick_full<ALIGNED, kFloatMax>(fn, per_sm);
    case kIntMin: return pick_full<ALIGNED, kIntMin>(fn, per_sm);
    case kIntMax: return pick_full<ALIGNED, kIntMax>(fn, per_sm);
    default: return pick_full<ALIGNED, kFloatMin>(fn, per_sm);
    }
}

// The kernel a run of this plan launches, its dynamic shared memory and CTAs per SM.
cudaError_t batch_kernel_for(bool light, bool aligned, uint32_t mode, const void **fn,
                             size_t *smem, int *per_sm) {
    if (light) return batch_light_kernel(aligned, mode, fn, smem, per_sm);
    *smem = 0;
    return aligned ? full_kernel_t<true>(mode, fn, per_sm) : full_kernel_t<false>(mode, fn, per_sm);
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace
RMQ_VIOLATIONS_READER(violations_batch)

}  // namespace rmq

using namespace rmq;

struct rmq_batch {
    int32_t narrays;
    int64_t limit;       // one past the last value any array uses
    int64_t total_q;     // one past the last query any array uses
    int device;
    std::vector<BatchArray> h_arrays;
    std::vector<uint4> h_qitems;
    void *mem;           // one device allocation: metadata, work lists, workspace, counter
    size_t mem_bytes;
    size_t ws_bytes;
    BatchParams P;       // device pointers filled, per-run fields left empty
    uint32_t flags;      // RMQ_BUILD_INT32 / RMQ_BUILD_MAX / RMQ_BUILD_LIGHT
    uint32_t kmode;      // KeyMode of every array
    bool light;          // light index (block and micro-block tables only)
    int32_t bucket_bs[RMQ_BATCH_BUCKETS];
    rmq_batch_tile_t tiles[RMQ_BATCH_BUCKETS];  // block size and tile schedule per bucket
    const float *built_vals;  // values of the last build enqueued on this plan
};

namespace {

int bucket_of(int64_t n) { return n <= 1 ? 0 : ilog2(static_cast<uint32_t>(n)); }

int64_t default_bs(int64_t n, bool light) {
    // Without autotuning, full index: small blocks, so that a query inside
    // one block is a short warp scan (the full batched index has no
    // sub-block level) and the sparse table does the rest; 64 below 2^17
    // elements, 256 above (what the autotuner picks for the ragged
    // benchmark, within 5% of it there). Light index: the micro table
    // answers queries inside a block and settles more of them than the
    // block table does for queries across blocks, so blocks of 4096 (the
    // ragged benchmark's queries: 3.1 ms against 8.8 ms at 1024).
    if (light) return 4096;
    return n < (1 << 17) ? 64 : 256;
}

}  // namespace

namespace {

// Milliseconds of `reps` runs (after one warm run) of a plan holding only
// the arrays `m`, with tile `t` for their bucket bk; <0 on failure (rc set).
float time_bucket(const std::vector<int64_t> &s, const std::vector<int64_t> &l,
                  const std::vector<int64_t> &qs, const std::vector<int64_t> &qc, int bk,
                  const rmq_batch_tile_t &t, uint32_t flags, const float *d_vals,
                  const int32_t *d_queries, float *d_val, int32_t *d_idx, int32_t reps,
                  rmq_stream_t stream, cudaEvent_t e0, cudaEvent_t e1, int &rc) {
    rmq_batch_tile_t cfg[RMQ_BATCH_BUCKETS];
    std::memset(cfg, 0, sizeof(cfg));
    cfg[bk] = t;
    rmq_batch_t *sub = nullptr;
    rc = rmq_batch_create_ex(static_cast<int32_t>(s.size()), s.data(), l.data(), qs.data(),
                             qc.data(), cfg, flags, &sub);
    if (rc) return -1.f;
    rc = rmq_batch_run(sub, d_vals, d_queries, d_val, d_idx, stream);  // warm
    float ms = -1.f;
    if (!rc) {
        cudaEventRecord(e0, stream);
        for (int r = 0; r < reps && !rc; ++r)
            rc = rmq_batch_run(sub, d_vals, d_queries, d_val, d_idx, stream);
        cudaEventRecord(e1, stream);
        const cudaError_t err = cudaEventSynchronize(e1);
        if (err != cudaSuccess && !rc) rc = cuda_fail(err, "rmq_batch_autotune: timing");
        if (!rc) cudaEventElapsedTime(&ms, e0, e1);
    }
    rmq_batch_free(sub);
    return rc ? -1.f : ms;
}

// Per size bucket: the block size, then (tiles == true) the query-item and
// level-item sizes, each the fastest candidate on that bucket's arrays and
// queries with the choices made so far.
int autotune_buckets(int32_t narrays, const int64_t *h_starts, const int64_t *h_lengths,
                     const int64_t *h_qstarts, const int64_t *h_qcounts, const float *d_vals,
                     const int32_t *d_queries, float *d_val, int32_t *d_idx, int32_t reps,
                     rmq_stream_t stream, uint32_t flags, rmq_batch_tile_t *out, bool tiles) {
    NvtxRange nvtx_range("rmq_batch_autotune");
    if (narrays <= 0 || !h_starts || !h_lengths || !h_qstarts || !h_qcounts)
        return set_error(RMQ_EINVAL, "rmq_batch_autotune: NULL argument");
    if (reps < 1) reps = 1;
    std::vector<std::vector<int32_t>> members(RMQ_BATCH_BUCKETS);
    for (int32_t i = 0; i < narrays; ++i) {
        if (h_lengths[i] < 0) return set_error(RMQ_EINVAL, "rmq_batch_autotune: array %d length < 0", i);
        if (h_lengths[i] > 0) members[bucket_of(h_lengths[i])].push_back(i);  // empty: no structure
    }
    static const int32_t bs_cands[] = {64, 256, 1024, 4096, 16384, 65536};
    // light plans: small blocks send short queries through the coarser block
    // probe, so only these, starting from the default; another is taken only
    // when it is more than 3% faster (per-bucket timings are short and noisy)
    static const int32_t light_cands[] = {4096, 1024, 16384};
    const bool light = (flags & RMQ_BUILD_LIGHT) != 0;
    static const int32_t q_cands[] = {512, 1024, 2048, 4096, 8192};
    static const int32_t l_cands[] = {1024, 4096, 16384};
    cudaEvent_t e0, e1;
    cudaError_t err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_batch_autotune: events");
    int rc = RMQ_OK;
    for (int bk = 0; bk < RMQ_BATCH_BUCKETS; ++bk) out[bk] = rmq_batch_tile_t{0, 0, 0, 0};
    for (int bk = 0; bk < RMQ_BATCH_BUCKETS && rc == RMQ_OK; ++bk) {
        const std::vector<int32_t> &m = members[bk];
        if (m.empty()) continue;
        std::vector<int64_t> s, l, qs, qc;
        for (int32_t i : m) {
            s.push_back(h_starts[i]);
            l.push_back(h_lengths[i]);
            qs.push_back(h_qstarts[i]);
            qc.push_back(h_qcounts[i]);
        }
        const int64_t maxlen = int64_t(2) << bk;
        rmq_batch_tile_t best{0, static_cast<int32_t>(kQueryChunk), static_cast<int32_t>(kLevelChunk), 0};
        float best_ms = 0.f;
        const int32_t *cands = light ? light_cands : bs_cands;
        const int ncand = light ? 3 : 6;
        for (int ci = 0; ci < ncand; ++ci) {
            const int32_t c = cands[ci];
            if (!light && c > 2 * maxlen && best.bs != 0) break;
            if (light && c > 2 * maxlen && c > cands[0]) continue;
            rmq_batch_tile_t t = best;
            t.bs = c;
            const float ms = time_bucket(s, l, qs, qc, bk, t, flags, d_vals, d_queries, d_val,
                                         d_idx, reps, stream, e0, e1, rc);
            if (rc) break;
            if (best.bs == 0 || ms < (light ? 0.97f : 1.f) * best_ms) {
                best_ms = ms;
                best = t;
            }
        }
        for (int32_t c : q_cands) {
            if (!tiles || rc) break;
            if (c == best.query_chunk) continue;
            rmq_batch_tile_t t = best;
            t.query_chunk = c;
            const float ms = time_bucket(s, l, qs, qc, bk, t, flags, d_vals, d_queries, d_val,
                                         d_idx, reps, stream, e0, e1, rc);
            if (!rc && ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        }
        for (int32_t c : l_cands) {
            if (!tiles || rc) break;
            if (c == best.level_chunk) continue;
            rmq_batch_tile_t t = best;
            t.level_chunk = c;
            const float ms = time_bucket(s, l, qs, qc, bk, t, flags, d_vals, d_queries, d_val,
                                         d_idx, reps, stream, e0, e1, rc);
            if (!rc && ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        }
        out[bk] = best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
}

}  // namespace

extern "C" {

int rmq_batch_create(int32_t narrays, const int64_t *h_starts, const int64_t *h_lengths,
                     const int64_t *h_qstarts, const int64_t *h_qcounts,
                     const int32_t *h_bucket_bs, rmq_batch_t **out) {
    rmq_batch_tile_t tiles[RMQ_BATCH_BUCKETS];
    for (int i = 0; i < RMQ_BATCH_BUCKETS; ++i) {
        tiles[i].bs = h_bucket_bs ? h_bucket_bs[i] : 0;
        tiles[i].query_chunk = 0;
        tiles[i].level_chunk = 0;
        tiles[i].reserved = 0;
    }
    return rmq_batch_create_ex(narrays, h_starts, h_lengths, h_qstarts, h_qcounts, tiles, 0u, out);
}

int rmq_batch_create_ex(int32_t narrays, const int64_t *h_starts, const int64_t *h_lengths,
                        const int64_t *h_qstarts, const int64_t *h_qcounts,
                        const rmq_batch_tile_t *h_bucket_tiles, uint32_t flags,
                        rmq_batch_t **out) {
    NvtxRange nvtx_range("rmq_batch_create");
    if (!out) return set_error(RMQ_EINVAL, "rmq_batch_create: out is NULL");
    *out = nullptr;
    if (narrays <= 0 || !h_starts || !h_lengths || !h_qstarts || !h_qcounts)
        return set_error(RMQ_EINVAL, "rmq_batch_create: narrays must be > 0 and arrays non-NULL");
    if (flags & ~static_cast<uint32_t>(RMQ_BUILD_MAX | RMQ_BUILD_INT32 | RMQ_BUILD_LIGHT))
        return set_error(RMQ_EINVAL, "rmq_batch_create: unsupported flags 0x%x", flags);
    const bool light = (flags & RMQ_BUILD_LIGHT) != 0;
    if (h_bucket_tiles)
        for (int i = 0; i < RMQ_BATCH_BUCKETS; ++i) {
            const rmq_batch_tile_t &t = h_bucket_tiles[i];
            if (t.query_chunk < 0 || t.level_chunk < 0)
                return set_error(RMQ_EINVAL, "rmq_batch_create: bucket %d has a negative chunk", i);
            if (light && t.bs > 0 && (t.bs < 64 || t.bs % 32 != 0))
                return set_error(RMQ_EINVAL,
                                 "rmq_batch_create: bucket %d: a light index needs a block size "
                                 "that is a multiple of 32 and at least 64 (bs=%d)", i, t.bs);
        }
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;

    rmq_batch_t *b = new (std::nothrow) rmq_batch_t;
    if (!b) return set_error(RMQ_ENOMEM, "rmq_batch_create: host allocation failed");
    b->narrays = narrays;
    b->device = dev.device;
    b->built_vals = nullptr;
    b->limit = 0;
    b->total_q = 0;
    b->mem = nullptr;
    b->flags = flags;
    b->light = light;
    b->kmode = ((flags & RMQ_BUILD_INT32) ? kIntMin : kFloatMin) + ((flags & RMQ_BUILD_MAX) ? 1u : 0u);
    for (int i = 0; i < RMQ_BATCH_BUCKETS; ++i) {
        const rmq_batch_tile_t t = h_bucket_tiles ? h_bucket_tiles[i] : rmq_batch_tile_t{0, 0, 0, 0};
        b->bucket_bs[i] = t.bs > 0 ? t.bs : 0;
        b->tiles[i].bs = b->bucket_bs[i];
        b->tiles[i].query_chunk = t.query_chunk > 0 ? t.query_chunk : static_cast<int32_t>(kQueryChunk);
        b->tiles[i].level_chunk = t.level_chunk > 0 ? t.level_chunk : static_cast<int32_t>(kLevelChunk);
        b->tiles[i].reserved = 0;
    }

    std::vector<uint2> build;
    std::vector<std::vector<uint4>> lvl(kMaxLevels);
    int64_t ws_entries = 0;
    int32_t maxlev = 1;
    b->h_arrays.resize(narrays);
    // table item: (array, kind << 16 | level, first, count) at table step `step`
    auto add_items = [&](int step, uint32_t i, uint32_t kind, uint32_t k, uint32_t cnt,
                         uint32_t chunk) {
        for (uint32_t j = 0; j < cnt; j += chunk)
            lvl[step].push_back(make_uint4(i, (kind << 16) | k, j, std::min(chunk, cnt - j)));
        maxlev = std::max<int32_t>(maxlev, step + 1);
    };
    for (int32_t i = 0; i < narrays; ++i) {
        const int64_t n = h_lengths[i], s = h_starts[i];
        const int64_t qs = h_qstarts[i], qc = h_qcounts[i];
        if (n < 0 || n > 0x7fffffffLL || s < 0 || qs < 0 || qc < 0 || qc > 0xffffffffLL) {
            delete b;
            return set_error(RMQ_EINVAL,
                             "rmq_batch_create: array %d has start=%lld length=%lld qstart=%lld "
                             "qcount=%lld (need length in [0, 2^31-1], others >= 0)",
                             i, (long long)s, (long long)n, (long long)qs, (long long)qc);
        }
        // an empty array has no structure; its queries (if any) are invalid
        const int bk = n > 0 ? bucket_of(n) : 0;
        int64_t bs = n > 0 ? b->bucket_bs[bk] : 1;
        if (bs <= 0) bs = default_bs(n, light);
        const uint32_t qchunk = static_cast<uint32_t>(b->tiles[bk].query_chunk);
        const uint32_t lchunk = static_cast<uint32_t>(b->tiles[bk].level_chunk);
        // light: blocks on micro-block boundaries, one block of at least 64
        // for an array shorter than bs
        if (bs > n) bs = n == 0 ? 1 : (light ? std::max<int64_t>(64, (n + 31) / 32 * 32) : n);
        BatchArray &a = b->h_arrays[i];
        std::memset(&a, 0, sizeof(a));
        a.off = s;
        a.qoff = qs;
        a.n = static_cast<uint32_t>(n);
        a.bs = static_cast<uint32_t>(bs);
        a.nb = static_cast<uint32_t>((n + bs - 1) / bs);
        a.levels = a.nb > 0 ? st_levels(a.nb) : 0u;
        a.U = make_unit_layout(a.bs, a.nb);
        a.dv = make_div31(a.bs);
        a.st = ws_entries;
        ws_entries += static_cast<int64_t>(a.nb) * a.levels;
        if (light) {
            a.nmicro = static_cast<uint32_t>((n + kMicro - 1) / kMicro);
            a.mlevels = n > 0 ? micro_levels(a.bs) : 0u;
            a.moff_bytes = a.mlevels ? micro_offset_bytes(a.mlevels) : 0u;
            a.mst = ws_entries;
            ws_entries += a.nmicro;
            a.moff = ws_entries;
            const int64_t moff_bytes = a.mlevels > 1 ? static_cast<int64_t>(a.moff_bytes) * a.nmicro *
                                                           (a.mlevels - 1) : 0;
            ws_entries += (moff_bytes + 7) / 8;
            a.pre = -1;
        } else {
            a.pre = ws_entries;
            ws_entries += 2 * n;
        }
        ws_entries = (ws_entries + 31) & ~int64_t(31);  // 256-byte alignment per array
        b->limit = std::max(b->limit, s + n);
        b->total_q = std::max(b->total_q, qs + qc);
        if (light && a.nmicro > 0) {
            // A: tiles (micro-block minima, every micro-table level and, when
            // the blocks' micro-blocks divide a tile, the block minima, from
            // one read of the values) if the micro table's halo fits a
            // tile, else chunks of micro-block minima followed by one table
            // item per micro level. B: block minima from the micro-block
            // minima unless the tiles wrote them, then block level k.
            const uint32_t pb = a.bs / kMicro;
            const uint32_t halo = (1u << (a.mlevels - 1)) - 1u;
            const uint32_t tile = halo + kMicroTile <= kTileEntries        ? kMicroTile
                                  : halo + kMicroTileSmall <= kTileEntries ? kMicroTileSmall
                                                                           : 0u;
            if (tile) {
                a.light_flags = kLightTiled | (tile % pb == 0 ? kLightTileBmin : 0u) |
                                (tile == kMicroTileSmall ? kLightSmallTile : 0u);
                for (uint32_t t = 0; t * tile < a.nmicro; ++t) build.push_back(make_uint2(i, t));
            } else {
                for (uint32_t c = 0; c * kLightChunk < a.nmicro; ++c) build.push_back(make_uint2(i, c));
                for (uint32_t k = 1; k < a.mlevels && (1u << k) <= a.nmicro; ++k)
                    add_items(k, i, kItemMicroLevel, k, a.nmicro - (1u << k) + 1, lchunk);
            }
            const int bstep = (a.light_flags & kLightTileBmin) ? 0 : 1;  // step of block level 0
            if (bstep == 1)
                add_items(1, i, kItemBlockMinima, 0, a.nb, std::max<uint32_t>(1u, lchunk / pb));
            for (uint32_t k = 1; k < a.levels; ++k)
                add_items(static_cast<int>(k) + bstep, i, kItemBlockLevel, k, a.nb - (1u << k) + 1,
                          lchunk);
        } else if (!light) {
            const uint32_t nunits = unit_count(a.nb, a.U);
            for (uint32_t u = 0; u < nunits; ++u) build.push_back(make_uint2(i, u));
            for (uint32_t k = 1; k < a.levels; ++k)
                add_items(k, i, kItemBlockLevel, k, a.nb - (1u << k) + 1, lchunk);
        }
        for (int64_t j = 0; j < qc; j += qchunk)
            b->h_qitems.push_back(make_uint4(i, static_cast<uint32_t>(j),
                                             static_cast<uint32_t>(std::min<int64_t>(qchunk, qc - j)), 0));
    }
    if (b->limit > 0xffffffffLL * 4) {
        delete b;
        return set_error(RMQ_EINVAL, "rmq_batch_create: value span too large");
    }
    std::vector<uint4> lvl_flat;
    BatchParams &P = b->P;
    std::memset(&P, 0, sizeof(P));
    P.maxlev = maxlev;
    for (int k = 0; k <= kMaxLevels; ++k) P.lvl_start[k] = 0;
    for (int k = 1; k < kMaxLevels; ++k) {
        P.lvl_start[k] = static_cast<int32_t>(lvl_flat.size());
        lvl_flat.insert(lvl_flat.end(), lvl[k].begin(), lvl[k].end());
    }
    P.lvl_start[kMaxLevels] = static_cast<int32_t>(lvl_flat.size());
    for (int k = maxlev; k < kMaxLevels; ++k) P.lvl_start[k] = P.lvl_start[kMaxLevels];
    P.nbuild = static_cast<int32_t>(build.size());
    P.nqitems = static_cast<int32_t>(b->h_qitems.size());
    P.total_q = b->total_q;

    // one allocation: arrays | build | lvl | qitems | counter | workspace
    const size_t o_arr = 0;
    const size_t o_build = align_up(o_arr + sizeof(BatchArray) * narrays, 256);
    const size_t o_lvl = align_up(o_build + sizeof(uint2) * build.size(), 256);
    const size_t o_q = align_up(o_lvl + sizeof(uint4) * lvl_flat.size(), 256);
    const size_t o_cnt = align_up(o_q + sizeof(uint4) * b->h_qitems.size(), 256);
    const size_t o_ws = align_up(o_cnt + 256, 256);
    b->ws_bytes = sizeof(Entry) * static_cast<size_t>(ws_entries);
    b->mem_bytes = o_ws + b->ws_bytes;
    cudaError_t err = dev_malloc(&b->mem, b->mem_bytes);
    if (err != cudaSuccess) {
        cudaGetLastError();
        size_t bytes = b->mem_bytes;
        delete b;
        return set_error(RMQ_ENOMEM, "rmq_batch_create: cudaMalloc(%zu bytes) failed", bytes);
    }
    char *base = static_cast<char *>(b->mem);
    err = cudaMemcpy(base + o_arr, b->h_arrays.data(), sizeof(BatchArray) * narrays,
                     cudaMemcpyHostToDevice);
    if (err == cudaSuccess && !build.empty())
        err = cudaMemcpy(base + o_build, build.data(), sizeof(uint2) * build.size(),
                         cudaMemcpyHostToDevice);
    if (err == cudaSuccess && !lvl_flat.empty())
        err = cudaMemcpy(base + o_lvl, lvl_flat.data(), sizeof(uint4) * lvl_flat.size(),
                         cudaMemcpyHostToDevice);
    if (err == cudaSuccess && !b->h_qitems.empty())
        err = cudaMemcpy(base + o_q, b->h_qitems.data(), sizeof(uint4) * b->h_qitems.size(),
                         cudaMemcpyHostToDevice);
    if (err == cudaSuccess) err = cudaMemset(base + o_cnt, 0, 256);
    if (err != cudaSuccess) {
        rc = cuda_fail(err, "rmq_batch_create: upload");
        cudaFree(b->mem);
        delete b;
        return rc;
    }
    P.arrays = reinterpret_cast<const BatchArray *>(base + o_arr);
    P.build = reinterpret_cast<const uint2 *>(base + o_build);
    P.lvl = reinterpret_cast<const uint4 *>(base + o_lvl);
    P.qitems = reinterpret_cast<const uint4 *>(base + o_q);
    P.invalid = reinterpret_cast<unsigned long long *>(base + o_cnt);
    P.ws = reinterpret_cast<Entry *>(base + o_ws);
    P.limit = b->limit;
    *out = b;
    return RMQ_OK;
}

static int batch_args(const rmq_batch_t *b, const float *d_vals, const int32_t *d_queries,
                      float *d_val, int32_t *d_idx, const char *who, bool with_queries = true) {
    if (!b) return set_error(RMQ_EINVAL, "%s: batch is NULL", who);
    if (!d_vals || reinterpret_cast<uintptr_t>(d_vals) % 4)
        return set_error(RMQ_EINVAL, "%s: d_vals NULL or not 4-byte aligned", who);
    if (with_queries && b->total_q > 0 && (!d_queries || reinterpret_cast<uintptr_t>(d_queries) % 8))
        return set_error(RMQ_EINVAL, "%s: d_queries NULL or not 8-byte aligned", who);
    if (with_queries && b->total_q > 0 && !d_val && !d_idx)
        return set_error(RMQ_EINVAL, "%s: both outputs are NULL", who);
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return cuda_fail(err, who);
    if (dev != b->device)
        return set_error(RMQ_EINVAL, "%s: batch planned on device %d, current is %d", who,
                         b->device, dev);
    return RMQ_OK;
}

// One cooperative launch of batch_kernel running the given phases.
static int launch_batch(rmq_batch_t *b, const float *d_vals, const int32_t *d_queries,
                        float *d_val, int32_t *d_idx, rmq_stream_t stream, uint32_t phases,
                        const char *who) {
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    BatchParams P = b->P;
    P.A = d_vals;
    P.Q = reinterpret_cast<const int2 *>(d_queries);
    P.val = d_val;
    P.idx = d_idx;
    P.phases = phases;
    const bool aligned = reinterpret_cast<uintptr_t>(d_vals) % 16 == 0;
    const void *kern = nullptr;
    size_t smem = 0;
    int per_sm = 0;
    cudaError_t err = batch_kernel_for(b->light, aligned, b->kmode, &kern, &smem, &per_sm);
    if (err != cudaSuccess) return cuda_fail(err, who);
    // a cooperative launch needs every CTA resident
    if (per_sm < 1) return set_error(RMQ_ENOTSUP, "%s: kernel cannot be resident", who);
    const unsigned grid = static_cast<unsigned>(dev.sms * per_sm);
    void *args[] = {&P};
    err = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(kThreads), args, smem, stream);
    if (err != cudaSuccess) return cuda_fail(err, who);
    if (phases & 1u) b->built_vals = d_vals;
    return RMQ_OK;
}

int rmq_batch_run(rmq_batch_t *b, const float *d_vals, const int32_t *d_queries, float *d_val,
                  int32_t *d_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_batch_run");
    const int rc = batch_args(b, d_vals, d_queries, d_val, d_idx, "rmq_batch_run");
    if (rc) return rc;
    return launch_batch(b, d_vals, d_queries, d_val, d_idx, stream, 7u, "rmq_batch_run");
}

int rmq_batch_build(rmq_batch_t *b, const float *d_vals, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_batch_build");
    const int rc = batch_args(b, d_vals, nullptr, nullptr, nullptr, "rmq_batch_build", false);
    if (rc) return rc;
    return launch_batch(b, d_vals, nullptr, nullptr, nullptr, stream, 3u, "rmq_batch_build");
}

int rmq_batch_query(rmq_batch_t *b, const float *d_vals, const int32_t *d_queries, float *d_val,
                    int32_t *d_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_batch_query");
    const int rc = batch_args(b, d_vals, d_queries, d_val, d_idx, "rmq_batch_query");
    if (rc) return rc;
    if (b->built_vals != d_vals)
        return set_error(RMQ_EINVAL, "rmq_batch_query: the plan was not built (rmq_batch_build or "
                                     "rmq_batch_run) on these values");
    return launch_batch(b, d_vals, d_queries, d_val, d_idx, stream, 4u, "rmq_batch_query");
}

int rmq_batch_run_per_array(rmq_batch_t *b, const float *d_vals, const int32_t *d_queries,
                            float *d_val, int32_t *d_idx, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_batch_run_per_array");
    int rc = batch_args(b, d_vals, d_queries, d_val, d_idx, "rmq_batch_run_per_array");
    if (rc) return rc;
    DeviceInfo dev;
    rc = device_info(&dev);
    if (rc) return rc;
    Entry *ws = b->P.ws;
    std::vector<int64_t> qcount(b->narrays, 0);
    for (const uint4 &w : b->h_qitems) qcount[w.x] += w.z;
    for (int32_t i = 0; i < b->narrays; ++i) {
        const BatchArray &a = b->h_arrays[i];
        BuildPlan p;
        std::memset(&p, 0, sizeof(p));
        p.A = d_vals + a.off;
        p.n = a.n;
        p.bs = a.bs;
        p.nb = a.nb;
        p.levels = a.levels;
        p.aligned = reinterpret_cast<uintptr_t>(p.A) % 16 == 0;
        p.st = ws + a.st;
        p.kmode = b->kmode;
        p.light = b->light;
        if (b->light) {
            // the plain light index over the plan's own workspace layout
            p.micro = a.mlevels > 0;
            p.nmicro = a.nmicro;
            p.mlevels = a.mlevels;
            p.mst = ws + a.mst;
            p.moff = ws + a.moff;
            p.moff_bytes = a.moff_bytes;
        } else {
            p.pre = ws + a.pre;
            p.suf = ws + a.pre + a.n;
        }
        cudaError_t err = launch_build(p, dev, stream);
        if (err != cudaSuccess) return cuda_fail(err, "rmq_batch_run_per_array: build");
        if (qcount[i] == 0) continue;
        QueryArgs q;
        q.Q = reinterpret_cast<const int2 *>(d_queries) + a.qoff;
        q.q = qcount[i];
        q.val = d_val ? d_val + a.qoff : nullptr;
        q.idx = d_idx ? d_idx + a.qoff : nullptr;
        q.invalid = b->P.invalid;
        err = launch_query(p, q, dev, stream);
        if (err != cudaSuccess) return cuda_fail(err, "rmq_batch_run_per_array: query");
    }
    return RMQ_OK;
}

int rmq_batch_scatter_grad(const rmq_batch_t *b, const int32_t *d_idx, const float *d_grad_out,
                           float *d_grad_vals, int32_t accumulate, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_batch_scatter_grad");
    if (!b || !d_idx || !d_grad_out || !d_grad_vals)
        return set_error(RMQ_EINVAL, "rmq_batch_scatter_grad: NULL argument");
    if (b->kmode >= kIntMin)
        return set_error(RMQ_EINVAL, "rmq_batch_scatter_grad: the plan holds int32 values");
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) return rc;
    cudaError_t err = cudaSuccess;
    if (!accumulate)
        err = cudaMemsetAsync(d_grad_vals, 0, sizeof(float) * static_cast<size_t>(b->limit), stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_batch_scatter_grad: memset");
    if (b->P.nqitems > 0) {
        unsigned grid = static_cast<unsigned>(std::min<int64_t>(b->P.nqitems, dev.sms * 8));
        scatter_grad_kernel<<<grid, kThreads, 0, stream>>>(b->P.arrays, b->P.qitems, b->P.nqitems,
                                                           d_idx, d_grad_out, d_grad_vals);
        err = cudaGetLastError();
        if (err != cudaSuccess) return cuda_fail(err, "rmq_batch_scatter_grad: launch");
    }
    return RMQ_OK;
}

int rmq_batch_info(const rmq_batch_t *b, rmq_batch_info_t *info) {
    if (!b || !info) return set_error(RMQ_EINVAL, "rmq_batch_info: NULL argument");
    info->narrays = b->narrays;
    info->values_span = b->limit;
    info->queries_span = b->total_q;
    info->workspace_bytes = static_cast<int64_t>(b->ws_bytes);
    info->device_bytes = static_cast<int64_t>(b->mem_bytes);
    info->build_items = b->P.nbuild;
    info->query_items = b->P.nqitems;
    info->max_levels = b->P.maxlev;
    info->flags = static_cast<int32_t>(b->flags);
    for (int i = 0; i < RMQ_BATCH_BUCKETS; ++i) info->bucket_bs[i] = b->bucket_bs[i];
    return RMQ_OK;
}

int rmq_batch_tiles(const rmq_batch_t *b, rmq_batch_tile_t *h_bucket_tiles) {
    if (!b || !h_bucket_tiles) return set_error(RMQ_EINVAL, "rmq_batch_tiles: NULL argument");
    for (int i = 0; i < RMQ_BATCH_BUCKETS; ++i) h_bucket_tiles[i] = b->tiles[i];
    return RMQ_OK;
}

int rmq_batch_invalid_count(const rmq_batch_t *b, rmq_stream_t stream, int64_t *count) {
    if (!b || !count) return set_error(RMQ_EINVAL, "rmq_batch_invalid_count: NULL argument");
    unsigned long long v = 0;
    cudaError_t err = cudaMemcpyAsync(&v, b->P.invalid, sizeof(v), cudaMemcpyDeviceToHost, stream);
    if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
    if (err != cudaSuccess) return cuda_fail(err, "rmq_batch_invalid_count");
    *count = static_cast<int64_t>(v);
    return RMQ_OK;
}

int rmq_batch_free(rmq_batch_t *b) {
    if (!b) return RMQ_OK;
    cudaError_t err = cudaFree(b->mem);
    delete b;
    if (err != cudaSuccess) return cuda_fail(err, "rmq_batch_free");
    return RMQ_OK;
}

int rmq_batch_autotune(int32_t narrays, const int64_t *h_starts, const int64_t *h_lengths,
                       const int64_t *h_qstarts, const int64_t *h_qcounts, const float *d_vals,
                       const int32_t *d_queries, float *d_val, int32_t *d_idx, int32_t reps,
                       rmq_stream_t stream, int32_t *h_bucket_bs) {
    if (!h_bucket_bs) return set_error(RMQ_EINVAL, "rmq_batch_autotune: NULL argument");
    rmq_batch_tile_t tiles[RMQ_BATCH_BUCKETS];
    const int rc = autotune_buckets(narrays, h_starts, h_lengths, h_qstarts, h_qcounts, d_vals,
                                    d_queries, d_val, d_idx, reps, stream, 0u, tiles, false);
    for (int i = 0; i < RMQ_BATCH_BUCKETS; ++i) h_bucket_bs[i] = rc ? 0 : tiles[i].bs;
    return rc;
}

int rmq_batch_autotune_ex(int32_t narrays, const int64_t *h_starts, const int64_t *h_lengths,
                          const int64_t *h_qstarts, const int64_t *h_qcounts, const float *d_vals,
                          const int32_t *d_queries, float *d_val, int32_t *d_idx, int32_t reps,
                          rmq_stream_t stream, uint32_t flags, rmq_batch_tile_t *h_bucket_tiles) {
    if (!h_bucket_tiles) return set_error(RMQ_EINVAL, "rmq_batch_autotune_ex: NULL argument");
    return autotune_buckets(narrays, h_starts, h_lengths, h_qstarts, h_qcounts, d_vals, d_queries,
                            d_val, d_idx, reps, stream, flags, h_bucket_tiles, true);
}

}  // extern "C"
