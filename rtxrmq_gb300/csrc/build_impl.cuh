// build_impl.cuh -- the CTA-level unit builder shared by the plain build
// kernel (build.cu) and the persistent batch kernel (batch.cu).
//
// For one array A[0..n) cut into blocks of bs it produces
//   pre[i]  = leftmost minimum of A[blockstart(i) .. i]
//   suf[i]  = leftmost minimum of A[i .. blockend(i)]
//   bmin[b] = leftmost minimum of block b
// which replace the reference's per-element triangles and per-block minimum
// triangles (src/device_tools.cuh:139-169, kernel_min_blocks 243-253,
// compute_min_blocks src/rtx.h:3-22).
//
// One CTA owns a "unit": one block when blocks are large, or G whole blocks
// (G * bs <= 4096 elements) when they are small. A tile is 4096 elements:
// 16 consecutive elements per thread, 16-byte loads aligned on absolute
// element indices, results staged in shared memory and written with
// coalesced stores. Entries are the comparison composites of common.cuh. A
// unit takes one of four paths (build_unit):
//   build_unit_aligned  one tile, blocks starting at thread boundaries (the
//                       unit on a 16-byte boundary, bs a multiple of 16):
//                       one load, no per-element segmentation, one CTA scan
//                       segmented by per-thread block start / end flags for
//                       both directions;
//   build_unit_tile     any other one-tile unit: one load, one CTA scan for
//                       both directions, segmented by segment ranks in the
//                       composite (below);
//   build_unit_stream   one block of 2 .. kMaxStreamTiles tiles: per-tile
//                       minima first, then every tile as a one-tile unit
//                       with its prefix and suffix carries;
//   build_unit_tiles    larger blocks: suffix pass right-to-left, then prefix
//                       pass left-to-right, carried across tiles.
//
// Segmented scans without flags (build_unit_tile, build_unit_tiles): every
// element becomes one 64-bit composite
//   [segment rank | key(value) | local index | -0.0 bit]
// whose unsigned minimum is the leftmost minimum. In the prefix direction
// earlier blocks of the unit get a larger rank, in the suffix direction later
// blocks do, so one min-scan over the unit restarts at every block boundary.
#pragma once

#include "common.cuh"
#include "lane_min.cuh"

namespace rmq {

// Tile geometry (compile-time tunables): threads per builder CTA and
// consecutive elements per thread (a power of two, multiple of 4).
#ifndef RMQ_BUILD_THREADS
#define RMQ_BUILD_THREADS 256
#endif
#ifndef RMQ_BUILD_EPT
#define RMQ_BUILD_EPT 16
#endif
constexpr int kBuildThreads = RMQ_BUILD_THREADS;
constexpr int kBuildEPT = RMQ_BUILD_EPT;                // elements per thread per tile
constexpr int kBuildTile = kBuildThreads * kBuildEPT;   // 4096 by default
constexpr int kBuildWarps = kBuildThreads / 32;
constexpr uint32_t kUnitTarget = kBuildTile;            // elements per multi-block unit
// staging: one padding entry after every thread's kBuildEPT entries
constexpr int kStageEntries = kBuildTile + kBuildTile / kBuildEPT;
static_assert(kBuildEPT % 4 == 0 && (kBuildEPT & (kBuildEPT - 1)) == 0, "kBuildEPT");
constexpr int kMaxStreamTiles = 64;                     // blocks up to 64 tiles: two-phase build
// shared words: CTA scans (2 x warps), per-tile minima and suffix carries of
// a multi-tile block (2 x kMaxStreamTiles)
constexpr int kWarpSlots = 2 * kBuildWarps + 2 * kMaxStreamTiles;

struct UnitLayout {
    uint32_t G;           // blocks per unit
    uint32_t key_shift;   // 32 when G == 1, else 17
    uint32_t seg_shift;   // 49 when G > 1 (63, unused, otherwise)
    uint32_t local_mask;  // 0x7fffffff when G == 1, else 0xffff
};

inline UnitLayout make_unit_layout(uint32_t bs, uint32_t nb) {
    UnitLayout U;
    U.G = (bs >= kUnitTarget) ? 1u : (kUnitTarget / bs);
    if (U.G > nb) U.G = nb;
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
    return U;
}

inline uint32_t unit_count(uint32_t nb, const UnitLayout &U) { return (nb + U.G - 1) / U.G; }

// One array to build: A is the base of the value buffer, the array occupies
// A[off .. off + n); loads never go past A[limit - 1].
struct UnitJob {
    const float *A;
    int64_t off;
    int64_t limit;
    uint32_t n;
    uint32_t bs;
    UnitLayout U;
    Div31 dv;
    Entry *pre;   // [n], array-relative
    Entry *suf;   // [n]
    Entry *bmin;  // [nb]
    uint32_t kmode;  // KeyMode (common.cuh)
    uint32_t nb;     // blocks of the array
};

__device__ __forceinline__ uint64_t umin64(uint64_t a, uint64_t b) { return b < a ? b : a; }

// Whether unit u lies inside one tile, and the tile's first element t0
// (absolute; a 16-byte boundary when ALIGNED).
template <bool ALIGNED>
__device__ __forceinline__ bool unit_tile(const UnitJob &J, uint32_t u, int64_t &t0) {
    const uint32_t ustart = u * J.U.G * J.bs;
    const uint32_t ulen = min(ustart + J.U.G * J.bs, J.n) - ustart;
    const int64_t a_lo = J.off + ustart;
    t0 = ALIGNED ? (a_lo & ~int64_t(3)) : a_lo;
    return static_cast<uint32_t>(a_lo - t0) + ulen <= static_cast<uint32_t>(kBuildTile);
}

__device__ __forceinline__ uint64_t unit_comp(uint32_t bits, uint32_t local, uint32_t segf,
                                              const UnitLayout &U, uint32_t mode) {
    const uint64_t nz = negzero_of(bits, mode);
    return (static_cast<uint64_t>(segf) << U.seg_shift) |
           (static_cast<uint64_t>(key_of(bits, mode)) << U.key_shift) |
           (static_cast<uint64_t>(local) << 1) | nz;
}

// Unit composite -> index entry (common.cuh) of the array-relative index.
__device__ __forceinline__ Entry unit_decode(uint64_t c, uint32_t ustart, const UnitLayout &U) {
    const uint32_t key = static_cast<uint32_t>(c >> U.key_shift);
    const uint32_t idx = ustart + (static_cast<uint32_t>(c >> 1) & U.local_mask);
    return (static_cast<uint64_t>(key) << 32) | (idx << 1) | (static_cast<uint32_t>(c) & 1u);
}

// Streaming store of one entry (written once, read by later kernels).
__device__ __forceinline__ void st_entry(Entry *p, Entry e) {
    __stcs(reinterpret_cast<uint2 *>(p),
           make_uint2(static_cast<uint32_t>(e), static_cast<uint32_t>(e >> 32)));
}

// Range-checked stores of the builders (rmq_chk, common.cuh): entry i of a
// per-element array of the job (pre / suf), block minimum b.
__device__ __forceinline__ void st_elem(const UnitJob &J, Entry *t, uint32_t i, Entry e) {
    if (rmq_chk(i < J.n)) st_entry(t + i, e);
}
__device__ __forceinline__ void st_bmin(const UnitJob &J, uint32_t b, Entry e) {
    if (rmq_chk(b < J.nb)) J.bmin[b] = e;
}

// Exclusive min-scan of one value per thread across the CTA, in thread order
// (REV = false) or reverse thread order (REV = true); `total` receives the
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
    for (int w = 0; w < kBuildWarps; ++w) {
        const uint64_t s = s_warp[w];
        tot = umin64(tot, s);
        if (REV ? (w > warp) : (w < warp)) wex = umin64(wex, s);
    }
    total = tot;
    __syncthreads();
    return umin64(ex, wex);
}

// Build unit `u` of job J with the whole CTA (kBuildThreads threads), in
// as many tiles as it spans: suffix pass, then prefix pass.
// stage: kStageEntries entries of shared memory; s_warp: kWarpSlots words.
template <bool ALIGNED, uint32_t MODE>
__device__ __forceinline__ void build_unit_tiles(const UnitJob &J, uint32_t u, Entry *stage,
                                                 uint64_t *s_warp) {
    const UnitLayout U = J.U;
    const uint32_t ustart = u * U.G * J.bs;
    const uint32_t uend = min(ustart + U.G * J.bs, J.n);
    const int64_t a_lo = J.off + ustart;        // absolute [a_lo, a_hi)
    const int64_t a_hi = J.off + uend;
    const int64_t t_first = ALIGNED ? (a_lo & ~int64_t(3)) : a_lo;
    const uint32_t ntiles = static_cast<uint32_t>((a_hi - t_first + kBuildTile - 1) / kBuildTile);

#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
        const bool suffix = (pass == 0);
        uint64_t carry = ~0ull;
#pragma unroll 1
        for (uint32_t tt = 0; tt < ntiles; ++tt) {
            const uint32_t t = suffix ? (ntiles - 1 - tt) : tt;
            const int64_t t0 = t_first + static_cast<int64_t>(t) * kBuildTile;
            const int64_t base = t0 + static_cast<int64_t>(threadIdx.x) * kBuildEPT;

            uint32_t bits[kBuildEPT];
            if (ALIGNED && base + kBuildEPT <= J.limit) {
#pragma unroll
                for (int v = 0; v < kBuildEPT / 4; ++v) {
                    const uint4 f = ld_u4(J.A + base + 4 * v);
                    bits[4 * v + 0] = f.x;
                    bits[4 * v + 1] = f.y;
                    bits[4 * v + 2] = f.z;
                    bits[4 * v + 3] = f.w;
                }
            } else {
#pragma unroll
                for (int j = 0; j < kBuildEPT; ++j) {
                    const int64_t g = base + j;
                    bits[j] = (g >= a_lo && g < a_hi) ? ld_u1(J.A + g) : 0u;
                }
            }

            uint64_t c[kBuildEPT];
#pragma unroll
            for (int j = 0; j < kBuildEPT; ++j) {
                const int64_t g = base + j;
                if (g >= a_lo && g < a_hi) {
                    const uint32_t local = static_cast<uint32_t>(g - a_lo);
                    uint32_t segf = 0;
                    if (U.G > 1) {
                        const uint32_t seg = div31(local, J.dv);
                        segf = suffix ? seg : (U.G - 1 - seg);
                    }
                    c[j] = unit_comp(bits[j], local, segf, U, MODE);
                } else {
                    c[j] = ~0ull;
                }
            }
            uint64_t agg;
            if (suffix) {
#pragma unroll
                for (int j = kBuildEPT - 2; j >= 0; --j) c[j] = umin64(c[j], c[j + 1]);
                agg = c[0];
            } else {
#pragma unroll
                for (int j = 1; j < kBuildEPT; ++j) c[j] = umin64(c[j], c[j - 1]);
                agg = c[kBuildEPT - 1];
            }
            uint64_t total;
            uint64_t ex = suffix ? cta_exclusive_min<true>(agg, s_warp, total)
                                 : cta_exclusive_min<false>(agg, s_warp, total);
            ex = umin64(ex, carry);
            carry = umin64(carry, total);

#pragma unroll
            for (int j = 0; j < kBuildEPT; ++j)
                stage[threadIdx.x * (kBuildEPT + 1) + j] =
                    unit_decode(umin64(c[j], ex), ustart, U);
            __syncthreads();

            Entry *out = suffix ? J.suf : J.pre;
#pragma unroll 4
            for (int k = 0; k < kBuildEPT; ++k) {
                const uint32_t e = threadIdx.x + k * kBuildThreads;
                const int64_t g = t0 + e;
                if (g >= a_lo && g < a_hi) {
                    const Entry en = stage[e + e / kBuildEPT];
                    const uint32_t local = static_cast<uint32_t>(g - J.off);
                    st_elem(J, out, local, en);
                    if (!suffix) {
                        // block minimum = prefix minimum at the block's last element
                        const uint32_t ul = local - ustart;
                        bool last = (g + 1 == a_hi);
                        uint32_t seg = 0;
                        if (U.G > 1) {
                            seg = div31(ul, J.dv);
                            last = last || (ul + 1 == (seg + 1) * J.bs);
                        }
                        if (last) st_bmin(J, u * U.G + seg, en);
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Exclusive min-scans of two values per thread across the CTA: `vp` in
// thread order, `vs` in reverse thread order, one barrier for both.
__device__ __forceinline__ void cta_exclusive_min2(uint64_t vp, uint64_t vs, uint64_t *s_warp,
                                                   uint64_t &xp, uint64_t &xs) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    uint64_t ip = vp, is = vs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t tp = __shfl_up_sync(0xffffffffu, ip, o);
        const uint64_t ts = __shfl_down_sync(0xffffffffu, is, o);
        if (lane >= o) ip = umin64(ip, tp);
        if (lane + o < 32) is = umin64(is, ts);
    }
    uint64_t ep = __shfl_up_sync(0xffffffffu, ip, 1);
    uint64_t es = __shfl_down_sync(0xffffffffu, is, 1);
    if (lane == 0) ep = ~0ull;
    if (lane == 31) es = ~0ull;
    if (lane == 31) s_warp[warp] = ip;
    if (lane == 0) s_warp[kBuildWarps + warp] = is;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < kBuildWarps; ++w) {
        if (w < warp) ep = umin64(ep, s_warp[w]);
        if (w > warp) es = umin64(es, s_warp[kBuildWarps + w]);
    }
    xp = ep;
    xs = es;
}

// Build a unit that lies inside one tile (every unit of bs <= 4096 whose
// first element is at most (tile - unit length) past a 16-byte boundary):
// the values are loaded once and both scans run on them, with one CTA scan
// for the two directions. Positions are 32-bit offsets in the unit; the
// composite is [segment rank (MULTI) | key | unit offset | -0.0 bit] with
// constant shifts; block minima are read from the staged prefix results at
// each block's last element.
template <bool ALIGNED, uint32_t MODE, bool MULTI>
__device__ __forceinline__ void build_unit_tile(const UnitJob &J, uint32_t u, Entry *stage,
                                                uint64_t *s_warp) {
    const uint32_t G = MULTI ? J.U.G : 1u;
    const uint32_t ustart = u * G * J.bs;
    const uint32_t ulen = min(ustart + G * J.bs, J.n) - ustart;
    const int64_t a_lo = J.off + ustart;
    const int64_t t0 = ALIGNED ? (a_lo & ~int64_t(3)) : a_lo;
    const int32_t lead = static_cast<int32_t>(a_lo - t0);
    const int64_t base = t0 + static_cast<int64_t>(threadIdx.x) * kBuildEPT;
    const int32_t ul0 = static_cast<int32_t>(threadIdx.x) * kBuildEPT - lead;

    uint32_t bits[kBuildEPT];
    if (ALIGNED && base + kBuildEPT <= J.limit) {
#pragma unroll
        for (int v = 0; v < kBuildEPT / 4; ++v) {
            const uint4 f = ld_u4(J.A + base + 4 * v);
            bits[4 * v + 0] = f.x;
            bits[4 * v + 1] = f.y;
            bits[4 * v + 2] = f.z;
            bits[4 * v + 3] = f.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < kBuildEPT; ++j)
            bits[j] = (static_cast<uint32_t>(ul0 + j) < ulen) ? ld_u1(J.A + base + j) : 0u;
    }

    constexpr bool kFloat = (MODE == kFloatMin || MODE == kFloatMax);
    uint64_t cb[kBuildEPT];
    uint64_t agg_p = ~0ull, agg_s = ~0ull;
#pragma unroll
    for (int j = 0; j < kBuildEPT; ++j) {
        const uint32_t ul = static_cast<uint32_t>(ul0 + j);
        const bool valid = ul < ulen;
        const uint32_t nz = (kFloat && bits[j] == 0x80000000u) ? 1u : 0u;
        const uint32_t key = key_of(bits[j], MODE);
        const uint64_t c = MULTI ? ((static_cast<uint64_t>(key) << 17) | (ul << 1) | nz)
                                 : ((static_cast<uint64_t>(key) << 32) | (ul << 1) | nz);
        cb[j] = valid ? c : ~0ull;
        if (MULTI) {
            const uint32_t seg = div31(valid ? ul : 0u, J.dv);
            agg_p = umin64(agg_p, cb[j] | (static_cast<uint64_t>(G - 1u - seg) << 49));
            agg_s = umin64(agg_s, cb[j] | (static_cast<uint64_t>(seg) << 49));
        } else {
            agg_p = umin64(agg_p, cb[j]);
        }
    }
    if (!MULTI) agg_s = agg_p;
    uint64_t ex_p, ex_s;
    cta_exclusive_min2(agg_p, agg_s, s_warp, ex_p, ex_s);

    // unit composite -> entry: for one block per unit it only moves the
    // offset to the array-relative index
    auto decode = [&](uint64_t c) -> Entry {
        if (!MULTI) return c + (static_cast<uint64_t>(ustart) << 1);
        const uint32_t lo = static_cast<uint32_t>(c);
        const uint32_t idx = ustart + ((lo >> 1) & 0xffffu);
        return (static_cast<uint64_t>(static_cast<uint32_t>(c >> 17)) << 32) | (idx << 1) | (lo & 1u);
    };

    // prefix minima
    uint64_t run = ex_p;
#pragma unroll
    for (int j = 0; j < kBuildEPT; ++j) {
        uint64_t c = cb[j];
        if (MULTI) {
            const uint32_t ul = static_cast<uint32_t>(ul0 + j);
            const uint32_t seg = div31(ul < ulen ? ul : 0u, J.dv);
            c |= static_cast<uint64_t>(G - 1u - seg) << 49;
        }
        run = umin64(run, c);
        stage[threadIdx.x * (kBuildEPT + 1) + j] = decode(run);
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kBuildEPT; ++k) {
        const uint32_t e = threadIdx.x + k * kBuildThreads;
        const uint32_t ul = e - static_cast<uint32_t>(lead);
        if (ul < ulen) {
            st_elem(J, J.pre, ustart + ul, stage[e + e / kBuildEPT]);
        }
    }
    {
        // block minimum = prefix minimum at the block's last element
        const uint32_t nblk = MULTI ? div31(ulen - 1u, J.dv) + 1u : 1u;
        for (uint32_t b = threadIdx.x; b < nblk; b += kBuildThreads) {
            const uint32_t last = min((b + 1u) * J.bs, ulen) - 1u;
            const uint32_t e = last + static_cast<uint32_t>(lead);
            st_bmin(J, u * G + b, stage[e + e / kBuildEPT]);
        }
    }
    __syncthreads();

    // suffix minima
    run = ex_s;
#pragma unroll
    for (int j = kBuildEPT - 1; j >= 0; --j) {
        uint64_t c = cb[j];
        if (MULTI) {
            const uint32_t ul = static_cast<uint32_t>(ul0 + j);
            const uint32_t seg = div31(ul < ulen ? ul : 0u, J.dv);
            c |= static_cast<uint64_t>(seg) << 49;
        }
        run = umin64(run, c);
        stage[threadIdx.x * (kBuildEPT + 1) + j] = decode(run);
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kBuildEPT; ++k) {
        const uint32_t e = threadIdx.x + k * kBuildThreads;
        const uint32_t ul = e - static_cast<uint32_t>(lead);
        if (ul < ulen) {
            st_elem(J, J.suf, ustart + ul, stage[e + e / kBuildEPT]);
        }
    }
    // The next unit's first shared-memory writes (s_warp, stage) come after
    // a barrier every thread reaches only when it has finished these reads.
}

// Block of more than one tile (one block per unit, up to kMaxStreamTiles
// tiles). Phase 1 streams the block once for its per-tile minima; the
// suffix carry of each tile (minimum of the tiles after it) follows from
// them. Phase 2 streams it again (mostly from L2) and builds every tile as a
// one-tile unit, with the running prefix carry and the tile's suffix carry
// folded into the CTA scan's results. Elements are combined directly as
// index entries.
template <bool ALIGNED, uint32_t MODE>
__device__ __forceinline__ void build_unit_stream(const UnitJob &J, uint32_t u, Entry *stage,
                                                  uint64_t *s_warp) {
    const uint32_t ustart = u * J.bs;
    const uint32_t ulen = min(ustart + J.bs, J.n) - ustart;
    const int64_t a_lo = J.off + ustart;
    const int64_t t_first = ALIGNED ? (a_lo & ~int64_t(3)) : a_lo;
    const uint32_t lead = static_cast<uint32_t>(a_lo - t_first);
    const uint32_t ntiles = (lead + ulen + kBuildTile - 1) / kBuildTile;
    uint64_t *s_tmin = s_warp + 2 * kBuildWarps;
    uint64_t *s_sufc = s_tmin + kMaxStreamTiles;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    constexpr bool kFloat = (MODE == kFloatMin || MODE == kFloatMax);

    // this thread's 16 elements of tile t as entries (kEntryNone outside the block)
    auto load_tile = [&](uint32_t t, Entry (&c)[kBuildEPT]) {
        const int64_t base = t_first + static_cast<int64_t>(t) * kBuildTile +
                             static_cast<int64_t>(threadIdx.x) * kBuildEPT;
        const uint32_t ul0 = t * kBuildTile + threadIdx.x * kBuildEPT - lead;  // may wrap
        uint32_t bits[kBuildEPT];
        if (ALIGNED && base + kBuildEPT <= J.limit) {
#pragma unroll
            for (int v = 0; v < kBuildEPT / 4; ++v) {
                const uint4 f = ld_u4(J.A + base + 4 * v);
                bits[4 * v + 0] = f.x;
                bits[4 * v + 1] = f.y;
                bits[4 * v + 2] = f.z;
                bits[4 * v + 3] = f.w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < kBuildEPT; ++j)
                bits[j] = (ul0 + j < ulen) ? ld_u1(J.A + base + j) : 0u;
        }
#pragma unroll
        for (int j = 0; j < kBuildEPT; ++j) {
            const uint32_t ul = ul0 + j;
            const uint32_t nz = (kFloat && bits[j] == 0x80000000u) ? 1u : 0u;
            const Entry e = (static_cast<uint64_t>(key_of(bits[j], MODE)) << 32) |
                            ((ustart + ul) << 1) | nz;
            c[j] = ul < ulen ? e : kEntryNone;
        }
    };

    // phase 1: per-tile minima (warp minima in alternating slots, one barrier a tile)
#pragma unroll 1
    for (uint32_t t = 0; t < ntiles; ++t) {
        Entry c[kBuildEPT];
        load_tile(t, c);
        uint64_t m = c[0];
#pragma unroll
        for (int j = 1; j < kBuildEPT; ++j) m = umin64(m, c[j]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = umin64(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) s_warp[(t & 1u) * kBuildWarps + warp] = m;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t tm = s_warp[(t & 1u) * kBuildWarps];
#pragma unroll
            for (int w = 1; w < kBuildWarps; ++w) tm = umin64(tm, s_warp[(t & 1u) * kBuildWarps + w]);
            s_tmin[t] = tm;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t acc = kEntryNone;
        for (uint32_t t = ntiles; t-- > 0;) {
            s_sufc[t] = acc;
            acc = umin64(acc, s_tmin[t]);
        }
        st_bmin(J, u, acc);  // block minimum
    }
    __syncthreads();

    // phase 2: every tile as a one-tile unit with carries
    uint64_t carry = kEntryNone;  // minimum of the tiles before t
#pragma unroll 1
    for (uint32_t t = 0; t < ntiles; ++t) {
        Entry c[kBuildEPT];
        load_tile(t, c);
        uint64_t agg = c[0];
#pragma unroll
        for (int j = 1; j < kBuildEPT; ++j) agg = umin64(agg, c[j]);
        uint64_t ex_p, ex_s;
        cta_exclusive_min2(agg, agg, s_warp, ex_p, ex_s);
        ex_p = umin64(ex_p, carry);
        ex_s = umin64(ex_s, s_sufc[t]);
        carry = umin64(carry, s_tmin[t]);
        const int64_t tile_ul = static_cast<int64_t>(t) * kBuildTile - lead;  // offset of tile entry 0

        uint64_t run = ex_p;
#pragma unroll
        for (int j = 0; j < kBuildEPT; ++j) {
            run = umin64(run, c[j]);
            stage[threadIdx.x * (kBuildEPT + 1) + j] = run;
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < kBuildEPT; ++k) {
            const uint32_t e = threadIdx.x + k * kBuildThreads;
            const uint32_t ul = static_cast<uint32_t>(tile_ul + e);
            if (ul < ulen) st_elem(J, J.pre, ustart + ul, stage[e + e / kBuildEPT]);
        }
        __syncthreads();
        run = ex_s;
#pragma unroll
        for (int j = kBuildEPT - 1; j >= 0; --j) {
            run = umin64(run, c[j]);
            stage[threadIdx.x * (kBuildEPT + 1) + j] = run;
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < kBuildEPT; ++k) {
            const uint32_t e = threadIdx.x + k * kBuildThreads;
            const uint32_t ul = static_cast<uint32_t>(tile_ul + e);
            if (ul < ulen) st_elem(J, J.suf, ustart + ul, stage[e + e / kBuildEPT]);
        }
        // the next tile's first shared writes (s_warp in its CTA scan, then
        // stage) follow a barrier that every thread reaches after these reads
    }
}

// Segmented exclusive min-scans across the CTA of one value per thread in
// both directions. Thread order (prefix): a thread with fp set starts a
// segment, and its carry covers the threads of its segment before it. Reverse
// order (suffix): a thread with fs set ends a segment. Pairs combine as
// (F1, S1) + (F2, S2) = (F1 | F2, F2 ? S2 : min(S1, S2)), 2 later in scan
// order; one barrier for both directions. A thread that starts (ends) a
// segment ignores its prefix (suffix) carry itself.
__device__ __forceinline__ void cta_segmented_min2(uint32_t fp, uint32_t fs, uint64_t v,
                                                   uint64_t *s_warp, uint32_t *s_flag,
                                                   uint64_t &xp, uint64_t &xs) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    uint64_t sp = v, ss = v;
    uint32_t gp = fp, gs = fs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t tsp = __shfl_up_sync(0xffffffffu, sp, o);
        const uint32_t tgp = __shfl_up_sync(0xffffffffu, gp, o);
        const uint64_t tss = __shfl_down_sync(0xffffffffu, ss, o);
        const uint32_t tgs = __shfl_down_sync(0xffffffffu, gs, o);
        if (lane >= o) {
            sp = gp ? sp : umin64(tsp, sp);
            gp |= tgp;
        }
        if (lane + o < 32) {
            ss = gs ? ss : umin64(tss, ss);
            gs |= tgs;
        }
    }
    uint64_t ep = __shfl_up_sync(0xffffffffu, sp, 1);
    uint32_t egp = __shfl_up_sync(0xffffffffu, gp, 1);
    uint64_t es = __shfl_down_sync(0xffffffffu, ss, 1);
    uint32_t egs = __shfl_down_sync(0xffffffffu, gs, 1);
    if (lane == 0) { ep = ~0ull; egp = 0u; }
    if (lane == 31) { es = ~0ull; egs = 0u; }
    if (lane == 31) { s_warp[warp] = sp; s_flag[warp] = gp; }
    if (lane == 0) { s_warp[kBuildWarps + warp] = ss; s_flag[kBuildWarps + warp] = gs; }
    __syncthreads();
    uint64_t ap = ~0ull, as = ~0ull;
#pragma unroll
    for (int w = 0; w < kBuildWarps; ++w) {
        if (w < warp) ap = s_flag[w] ? s_warp[w] : umin64(ap, s_warp[w]);
        const int wr = kBuildWarps - 1 - w;
        if (wr > warp)
            as = s_flag[kBuildWarps + wr] ? s_warp[kBuildWarps + wr] : umin64(as, s_warp[kBuildWarps + wr]);
    }
    xp = fp ? ~0ull : (egp ? ep : umin64(ap, ep));
    xs = fs ? ~0ull : (egs ? es : umin64(as, es));
}

// One-tile unit whose blocks start at thread boundaries (the unit starts on
// a 16-byte boundary and bs is a multiple of kBuildEPT; every unit of plain
// arrays and of 4-aligned batched arrays): a thread's elements lie in one
// block, so the thread-local scans need no segmentation and the CTA scan is
// segmented by "this thread starts / ends a block" flags. Elements are
// combined directly as index entries (no decode), so a unit of many small
// blocks costs what a unit of one block does.
template <bool ALIGNED, uint32_t MODE>
__device__ __forceinline__ void build_unit_aligned(const UnitJob &J, uint32_t u, Entry *stage,
                                                   uint64_t *s_warp, uint32_t *s_flag) {
    const uint32_t G = J.U.G;
    const uint32_t bs = J.bs;
    const uint32_t ustart = u * G * bs;
    const uint32_t ulen = min(ustart + G * bs, J.n) - ustart;
    const int64_t base = J.off + ustart + static_cast<int64_t>(threadIdx.x) * kBuildEPT;
    const uint32_t ul0 = threadIdx.x * kBuildEPT;

    uint32_t bits[kBuildEPT];
    if (ALIGNED && base + kBuildEPT <= J.limit) {
#pragma unroll
        for (int v = 0; v < kBuildEPT / 4; ++v) {
            const uint4 f = ld_u4(J.A + base + 4 * v);
            bits[4 * v + 0] = f.x;
            bits[4 * v + 1] = f.y;
            bits[4 * v + 2] = f.z;
            bits[4 * v + 3] = f.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < kBuildEPT; ++j) bits[j] = (ul0 + j < ulen) ? ld_u1(J.A + base + j) : 0u;
    }
    constexpr bool kFloat = (MODE == kFloatMin || MODE == kFloatMax);
    Entry c[kBuildEPT];
    uint64_t agg = kEntryNone;
#pragma unroll
    for (int j = 0; j < kBuildEPT; ++j) {
        const uint32_t ul = ul0 + j;
        const uint32_t nz = (kFloat && bits[j] == 0x80000000u) ? 1u : 0u;
        const Entry e = (static_cast<uint64_t>(key_of(bits[j], MODE)) << 32) |
                        ((ustart + ul) << 1) | nz;
        c[j] = ul < ulen ? e : kEntryNone;
        agg = umin64(agg, c[j]);
    }
    // block boundaries fall between threads: this thread starts a block when
    // its first offset is a multiple of bs, ends one when the next is
    const uint32_t r0 = ul0 - div31(ul0, J.dv) * bs;
    const uint32_t fp = r0 == 0u ? 1u : 0u;
    const uint32_t fs = (r0 + kBuildEPT == bs) ? 1u : 0u;
    uint64_t ex_p, ex_s;
    cta_segmented_min2(fp, fs, agg, s_warp, s_flag, ex_p, ex_s);

    uint64_t run = ex_p;
#pragma unroll
    for (int j = 0; j < kBuildEPT; ++j) {
        run = umin64(run, c[j]);
        stage[threadIdx.x * (kBuildEPT + 1) + j] = run;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kBuildEPT; ++k) {
        const uint32_t e = threadIdx.x + k * kBuildThreads;
        if (e < ulen) st_elem(J, J.pre, ustart + e, stage[e + e / kBuildEPT]);
    }
    {
        // block minimum = prefix minimum at the block's last element
        const uint32_t nblk = div31(ulen - 1u, J.dv) + 1u;
        for (uint32_t b = threadIdx.x; b < nblk; b += kBuildThreads) {
            const uint32_t last = min((b + 1u) * bs, ulen) - 1u;
            st_bmin(J, u * G + b, stage[last + last / kBuildEPT]);
        }
    }
    __syncthreads();
    run = ex_s;
#pragma unroll
    for (int j = kBuildEPT - 1; j >= 0; --j) {
        run = umin64(run, c[j]);
        stage[threadIdx.x * (kBuildEPT + 1) + j] = run;
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < kBuildEPT; ++k) {
        const uint32_t e = threadIdx.x + k * kBuildThreads;
        if (e < ulen) st_elem(J, J.suf, ustart + e, stage[e + e / kBuildEPT]);
    }
}

// Build unit `u`: one-tile units with the single-pass builder, others with
// the tile-streaming one. The choice is uniform across the CTA.
template <bool ALIGNED, uint32_t MODE>
__device__ __forceinline__ void build_unit(const UnitJob &J, uint32_t u, Entry *stage,
                                           uint64_t *s_warp, uint32_t *s_flag) {
    int64_t t0;
    if (unit_tile<ALIGNED>(J, u, t0)) {
        if (ALIGNED && t0 == J.off + static_cast<int64_t>(u) * J.U.G * J.bs &&
            J.bs % kBuildEPT == 0)
            build_unit_aligned<ALIGNED, MODE>(J, u, stage, s_warp, s_flag);
        else if (J.U.G > 1)
            build_unit_tile<ALIGNED, MODE, true>(J, u, stage, s_warp);
        else
            build_unit_tile<ALIGNED, MODE, false>(J, u, stage, s_warp);
    } else if (J.U.G == 1 &&
               (static_cast<uint32_t>(J.off + u * J.bs - t0) + min(J.bs, J.n - u * J.bs) +
                kBuildTile - 1) / kBuildTile <= static_cast<uint32_t>(kMaxStreamTiles)) {
        build_unit_stream<ALIGNED, MODE>(J, u, stage, s_warp);
    } else {
        build_unit_tiles<ALIGNED, MODE>(J, u, stage, s_warp);
    }
}

// ---- light index: micro-block minima and the micro table's levels ----

constexpr uint32_t kMicroElems = 32;    // elements per micro-block
constexpr uint32_t kMicroPerWarp = 16;  // micro-blocks a warp reduces per step

// The composite minimum of one micro-block whose 32 elements lie 4 per lane
// on the 8 lanes of group `grp` (this lane's first element at e = base +
// 4 sub). Composites order by (key, index), so the 32-bit keys are reduced
// first: each lane keeps its smallest key and the first position holding
// it (lane_best4), the group takes the minimum key, and the leftmost lane holding that
// key owns the leftmost best element; its position and -0.0 flag come over
// in one shuffle. Elements at or past n take the largest key; they lie to
// the right of every valid element, so a tie never selects one.
template <uint32_t MODE, bool FULL>
__device__ __forceinline__ Entry micro_row_min(const uint32_t (&b)[4], uint32_t e, uint32_t n,
                                               uint32_t grp, uint32_t sub) {
    uint32_t km, info;  // the lane's best key; its position | (-0.0 flag << 2)
    lane_best4<MODE>(b, FULL ? 4u : (e < n ? min(4u, n - e) : 0u), km, info);
    uint32_t gk = km;
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) gk = min(gk, __shfl_xor_sync(0xffffffffu, gk, o, 8));
    const uint32_t owners = (__ballot_sync(0xffffffffu, km == gk) >> (grp * 8u)) & 0xffu;
    const uint32_t w = __ffs(owners) - 1u;
    const uint32_t winfo = __shfl_sync(0xffffffffu, info, grp * 8u + w);
    const uint32_t base = e - 4u * sub;
    if (!FULL && base >= n) return kEntryNone;
    const uint32_t idx = base + 4u * w + (winfo & 3u);
    return (static_cast<uint64_t>(gk) << 32) | (idx << 1) | (winfo >> 2);
}

// One offset of level k >= 1 of the micro table (as offsets): the window of
// 2^k micro-blocks at i is the windows of 2^(k-1) at i and i + 2^(k-1); each
// half's best micro-block comes from the level below (`prev`, level k - 1;
// level 0 = the minima themselves), the better of the two is kept as its
// offset from i in `cur`. Unsigned comparison of composites keeps the
// leftmost of equal minima.
template <class O>
__device__ __forceinline__ void micro_level_at(const Entry *__restrict__ mst0, O *cur,
                                               const O *prev, uint32_t nmicro, uint32_t k,
                                               uint32_t i) {
    const uint32_t half = 1u << (k - 1);
    uint32_t a = i, b = i + half;
    if (k >= 2) {
        a += prev[i];
        b += prev[i + half];
    }
    if (rmq_chk(a < nmicro && b < nmicro && a - i < half && b - i < 2 * half))
        cur[i] = static_cast<O>((mst0[b] < mst0[a] ? b : a) - i);
}

// Micro-block minima of micro-blocks [j0, j0 + 16) of one array (values
// A[0 .. n)) with one whole warp: four 512-byte rows, each lane 4
// consecutive elements of every row, all loads in flight before any
// reduction (micro_row_min). VEC: 16-byte loads (A + j0 * 32 16-byte aligned
// and all 512 elements inside the array). Writes dst[j - base] for j < jend
// (jend <= ceil(n / 32)); returns the four minima of the lane's group
// (micro-blocks j0 + 4i + lane / 8; kEntryNone past the array).
template <uint32_t MODE, bool VEC>
__device__ __forceinline__ void micro_min_warp(const float *__restrict__ A, uint32_t n,
                                               uint32_t j0, uint32_t jend, Entry *dst,
                                               uint32_t base, Entry (&m)[4]) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t sub = lane & 7u;
    const uint32_t grp = lane >> 3;
    const uint32_t e0 = j0 * kMicroElems + lane * 4u;  // row 0 of this lane
    uint32_t b[4][4];
    if (VEC) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint4 f = ld_u4(A + e0 + i * 128u);
            b[i][0] = f.x;
            b[i][1] = f.y;
            b[i][2] = f.z;
            b[i][3] = f.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t g = e0 + i * 128u + k;
                b[i][k] = g < n ? ld_u1(A + g) : 0u;
            }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) m[i] = micro_row_min<MODE, VEC>(b[i], e0 + i * 128u, n, grp, sub);
    if (sub == 0u) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint32_t j = j0 + 4u * i + grp;
            if (j < jend) dst[j - base] = m[i];
        }
    }
}

// micro_min_warp over ROWS rows (4 * ROWS micro-blocks [j0, j0 + 4 ROWS)),
// every row's loads in flight before any reduction, each row's minima
// written (dst[j - base], j < jend) as soon as they are reduced, none kept.
template <uint32_t MODE, bool VEC, int ROWS>
__device__ __forceinline__ void micro_min_rows(const float *__restrict__ A, uint32_t n,
                                               uint32_t j0, uint32_t jend, Entry *dst,
                                               uint32_t base) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t sub = lane & 7u;
    const uint32_t grp = lane >> 3;
    const uint32_t e0 = j0 * kMicroElems + lane * 4u;
    uint32_t b[ROWS][4];
    if (VEC) {
#pragma unroll
        for (int i = 0; i < ROWS; ++i) {
            const uint4 f = ld_u4(A + e0 + i * 128u);
            b[i][0] = f.x;
            b[i][1] = f.y;
            b[i][2] = f.z;
            b[i][3] = f.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < ROWS; ++i)
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t g = e0 + i * 128u + k;
                b[i][k] = g < n ? ld_u1(A + g) : 0u;
            }
    }
#pragma unroll
    for (int i = 0; i < ROWS; ++i) {
        const Entry m = micro_row_min<MODE, VEC>(b[i], e0 + i * 128u, n, grp, sub);
        const uint32_t j = j0 + 4u * i + grp;
        if (sub == 0u && j < jend) dst[j - base] = m;
    }
}

}  // namespace rmq
