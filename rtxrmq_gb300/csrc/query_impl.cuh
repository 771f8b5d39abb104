// query_impl.cuh -- the CTA-level query body shared by the plain query kernel
// (query.cu) and the persistent batch kernel (batch.cu).
//
// It replaces RTX_blocks' ray programs (src/rtx_kernels.cu:85-193 for
// values, 350-465 for indices). The reference fires up to three rays per
// query: one through the fully covered blocks lB+1..rB-1, one through the
// left partial block and one through the right partial block, and keeps the
// closest hit. Here the same decomposition is answered from arrays:
//   left partial block   -> suf[l]   (random HBM lookup)
//   right partial block  -> pre[r]   (random HBM lookup)
//   full blocks between  -> two sparse-table entries (L2-resident)
// and it is needed only for the few queries a cheaper test does not settle:
// every query first probes a small L2-resident table over all the units it
// touches (blocks lB..rB, or with the sub-block level the 32-element
// micro-blocks l/32..r/32), and when the leftmost best of that superset
// lies inside [l, r] it is the answer without any per-element lookup. A
// query inside one micro-block is settled by one thread's scan of that
// 128-byte line; without the sub-block level a query inside one block that
// the probe does not settle reads pre / suf at a block edge, or is scanned
// by the whole warp (__reduce_min_sync over the composites). All
// comparisons are unsigned minima of the composites of common.cuh; only the
// final answer is decoded.
//
// Differences from the reference kept on purpose: ties between rays are
// resolved leftmost (the reference compares rays with strict `<` in the
// order middle, left, right, src/rtx_kernels.cu:451-465), values are the
// exact bits of A[idx] (the reference returns payload + min, rtx.h:109,
// rtx_kernels.cu:179), and a miss cannot overwrite a minimum
// (src/rtx_kernels.cu:80-83).
#pragma once

#include "common.cuh"

namespace rmq {

// One built array: values A[off .. off + n) of the buffer A (loads never go
// past A[limit - 1]); structure arrays are array-relative.
struct V1View {
    const float *A;
    int64_t off;
    int64_t limit;
    uint32_t n;
    uint32_t bs;
    uint32_t nb;
    Div31 dv;
    const Entry *pre;
    const Entry *suf;
    const Entry *st;
    // sub-block level: 32-element micro-blocks (local index / 32), whatever
    // the block size; null when the index has none (same-block queries then
    // use the warp-cooperative scan)
    const Entry *mst;   // micro-block minima (micro-table level 0)
    const void *moff;   // levels 1..: offsets of each window's best micro-block
    uint32_t moff_bytes;
    uint32_t nmicro;
    const Entry *mpre;  // in-micro-block prefix / suffix minima
    const Entry *msuf;
    uint32_t kmode;     // KeyMode: element type and minimum / maximum
    uint32_t levels;    // sparse-table levels (st holds levels * nb entries)
    uint32_t mlevels;   // micro-table levels (moff holds mlevels - 1 rows of nmicro)
    // 2^mlevels - 1: a query whose end micro-blocks ml < mr have
    // mr - ml < micro_span is probed through the micro table (0: no micro level)
    uint32_t micro_span;
};

// Range-checked accesses (rmq_chk, common.cuh): element loads by absolute
// index into A, table entries by index into a table of `size` entries.
__device__ __forceinline__ uint32_t ld_elem(const V1View &v, int64_t g) {
    return rmq_chk(g >= 0 && g < v.limit) ? ld_u1(v.A + g) : 0u;
}
__device__ __forceinline__ uint4 ld_elem4(const V1View &v, int64_t g) {
    return rmq_chk(g >= 0 && g + 3 < v.limit) ? ld_u4(v.A + g) : make_uint4(0u, 0u, 0u, 0u);
}
__device__ __forceinline__ Entry ld_entry(const Entry *t, uint64_t i, uint64_t size) {
    return rmq_chk(i < size) ? t[i] : kEntryNone;
}

// The same, as a streaming load (evict-first in L1 and L2), for the random
// per-element sub-block entries: they are read once, and the micro table
// they would otherwise evict is read by every same-block query.
__device__ __forceinline__ Entry ld_entry_cs(const Entry *t, uint64_t i, uint64_t size) {
    return rmq_chk(i < size) ? __ldcs(reinterpret_cast<const unsigned long long *>(t) + i)
                             : kEntryNone;
}

// The small tables every query probes (the sparse table over block minima,
// the micro table) are read with an L2 evict-last policy (PTX createpolicy +
// ld.L2::cache_hint), so that the per-element lines and the query stream
// passing through L2 evict them last. No L2 carve-out is set aside, unlike a
// persisting access-policy window. The policy is made once per step.
__device__ __forceinline__ uint64_t l2_keep_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ Entry ld_entry_keep(const Entry *t, uint64_t i, uint64_t size,
                                               uint64_t pol) {
    if (!rmq_chk(i < size)) return kEntryNone;
    unsigned long long v;
    asm volatile("ld.global.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(t + i), "l"(pol));
    return v;
}

// Offset i of the micro table's levels 1.. (moff_bytes wide, the same for
// every query of an index, so the branch does not diverge).
__device__ __forceinline__ uint32_t ld_moff(const V1View &v, uint64_t i, uint64_t pol) {
    if (!rmq_chk(i < static_cast<uint64_t>(v.mlevels - 1u) * v.nmicro)) return 0u;
    uint32_t r;
    if (v.moff_bytes == 1u)
        asm volatile("ld.global.L2::cache_hint.u8 %0, [%1], %2;"
                     : "=r"(r) : "l"(static_cast<const uint8_t *>(v.moff) + i), "l"(pol));
    else if (v.moff_bytes == 2u)
        asm volatile("ld.global.L2::cache_hint.u16 %0, [%1], %2;"
                     : "=r"(r) : "l"(static_cast<const uint16_t *>(v.moff) + i), "l"(pol));
    else
        asm volatile("ld.global.L2::cache_hint.u32 %0, [%1], %2;"
                     : "=r"(r) : "l"(static_cast<const uint32_t *>(v.moff) + i), "l"(pol));
    return r;
}

// The aligned 8-byte word of the 1-byte micro-table offsets that holds
// offset i (the table starts 256-byte aligned; its tail is padded to 256
// bytes, so the word never passes the allocation).
__device__ __forceinline__ uint64_t ld_moff_word(const V1View &v, uint64_t i, uint64_t pol) {
    const uint64_t w = i >> 3;
    if (!rmq_chk(w < (static_cast<uint64_t>(v.mlevels - 1u) * v.nmicro + 7) / 8)) return 0u;
    uint64_t r;
    asm volatile("ld.global.L2::cache_hint.u64 %0, [%1], %2;"
                 : "=l"(r) : "l"(static_cast<const uint64_t *>(v.moff) + w), "l"(pol));
    return r;
}

// Leftmost minimum of local A[a..b] (b - a < 32) computed by one thread.
// ALIGNED: 16-byte loads of the chunks covering [a, b] (at most 9), two per
// round, so that few registers are live.
template <bool ALIGNED>
__device__ __forceinline__ Entry thread_range_min(const V1View &v, uint32_t a, uint32_t b,
                                                  uint32_t mode) {
    const int64_t aa = v.off + a, ab = v.off + b;
    Entry best = kEntryNone;
    if (ALIGNED) {
#pragma unroll 2
        for (int64_t p = aa & ~int64_t(3); p <= ab; p += 4) {
            uint32_t w[4];
            if (p + 3 < v.limit) {
                const uint4 f = ld_elem4(v, p);
                w[0] = f.x;
                w[1] = f.y;
                w[2] = f.z;
                w[3] = f.w;
            } else {
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    w[c] = (p + c <= ab) ? ld_elem(v, p + c) : 0u;
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int64_t g = p + c;
                if (g >= aa && g <= ab)
                    best = better(best, make_entry(w[c], static_cast<uint32_t>(g - v.off), mode));
            }
        }
    } else {
        for (int64_t g = aa; g <= ab; ++g)
            best = better(best, make_entry(ld_elem(v, g), static_cast<uint32_t>(g - v.off), mode));
    }
    return best;
}

struct QueryOut {
    const int2 *Q;        // queries of this array (local l, r)
    float *val;           // outputs aligned with Q, may be null
    int32_t *idx;         // may be null
    unsigned long long *invalid;
    int64_t span;         // entries of Q / val / idx from these pointers on
};

__device__ __forceinline__ void put_bits_idx(const QueryOut &o, int64_t i, uint32_t bits,
                                             uint32_t idx) {
    if (!rmq_chk(i >= 0 && i < o.span)) return;
    if (o.val) __stcs(reinterpret_cast<unsigned int *>(o.val) + i, bits);
    if (o.idx) __stcs(o.idx + i, static_cast<int32_t>(idx));
}

__device__ __forceinline__ void put_result(const QueryOut &o, int64_t i, Entry e, uint32_t mode) {
    put_bits_idx(o, i, o.val ? entry_bits(e, mode) : 0u, entry_idx(e));
}

__device__ __forceinline__ void put_invalid(const QueryOut &o, int64_t i) {
    if (!rmq_chk(i >= 0 && i < o.span)) return;
    if (o.val) __stcs(reinterpret_cast<unsigned int *>(o.val) + i, 0x7fc00000u);
    if (o.idx) __stcs(o.idx + i, -1);
    if (o.invalid) atomicAdd(o.invalid, 1ull);
}

// Leftmost minimum of local A[l..r] computed by the whole warp. All 32 lanes
// call it with the same (l, r); every lane gets the result. ALIGNED: the
// buffer base is 16-byte aligned, so 16-byte loads on absolute indices are.
template <bool ALIGNED>
__device__ __forceinline__ Entry warp_scan_range(const V1View &v, uint32_t l, uint32_t r,
                                                 int lane, uint32_t mode) {
    Entry best = kEntryNone;
    const int64_t al = v.off + l, ar = v.off + r;
    if (ALIGNED) {
        for (int64_t p = (al & ~int64_t(3)) + 4 * lane; p <= ar; p += 128) {
            uint32_t b[4];
            if (p + 3 < v.limit) {
                const uint4 f = ld_elem4(v, p);
                b[0] = f.x;
                b[1] = f.y;
                b[2] = f.z;
                b[3] = f.w;
            } else {
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    b[c] = (p + c <= ar) ? ld_elem(v, p + c) : 0u;
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int64_t g = p + c;
                if (g >= al && g <= ar)
                    best = better(best, make_entry(b[c], static_cast<uint32_t>(g - v.off), mode));
            }
        }
    } else {
        for (int64_t g = al + lane; g <= ar; g += 32)
            best = better(best, make_entry(ld_elem(v, g), static_cast<uint32_t>(g - v.off), mode));
    }
    // 64-bit minimum across the warp: the key word first, then the low word
    // among the lanes that hold that key
    const uint32_t key = static_cast<uint32_t>(best >> 32);
    const uint32_t kmin = __reduce_min_sync(0xffffffffu, key);
    const uint32_t cand = (key == kmin) ? static_cast<uint32_t>(best) : 0xffffffffu;
    const uint32_t lo = __reduce_min_sync(0xffffffffu, cand);
    return (static_cast<uint64_t>(kmin) << 32) | lo;
}

// Answer queries [q0, q1) of one array with the whole CTA. The loop is
// uniform across the CTA (warp-cooperative scans need full warps).
// QPT queries per thread per iteration keep several independent lookups in
// flight per thread.
// Queries base + threadIdx.x + k * blockDim.x (k < QPT) of [.., q1), loaded
// ahead of use (the query stream may come from host memory over the host
// link, so a caller can issue the next step's loads before answering the
// current step).
template <int QPT>
__device__ __forceinline__ void load_queries(const QueryOut &o, int64_t base, int64_t q1,
                                             int2 (&qq)[QPT]) {
#pragma unroll
    for (int k = 0; k < QPT; ++k) {
        const int64_t i = base + threadIdx.x + static_cast<int64_t>(k) * blockDim.x;
        qq[k] = make_int2(0, 0);
        if (i < q1 && rmq_chk(i < o.span)) qq[k] = __ldcs(o.Q + i);
    }
}

// ---- per-query work --------------------------------------------------------
//
// Every probe of a small table returns the leftmost best element of a set of
// whole units (blocks of the sparse table, micro-blocks of the micro table)
// that contains [l, r]. If that element's index lies in [l, r], it is the
// answer: it beats every element of the superset, and an equal element
// further left inside [l, r] would have been chosen instead. Otherwise the
// best lies outside on one side, say left of l in unit a; then the answer is
// better(S[l], best of units a+1..b) when the latter falls at or before r
// (S[l] covers [l, end of a]), and the three-part decomposition of the
// reference (left partial, units between, right partial) only when it does
// not. The per-element entries S / P, the random HBM lookups, are read only
// on those two fallbacks.

// Query counters of a measurement launch (rmq_query_stats); the normal
// kernels compile them out.
enum QStat : int {
    kStatFirst = 0,   // settled by the superset probe
    kStatSecond,      // settled by the second probe and one per-element entry
    kStatFull,        // three-part decomposition: two entries and a middle probe
    kStatMicroScan,   // inside one micro-block: one thread scans its line
    kStatBlockEdge,   // one block, no sub-block level: pre / suf at a block edge
    kStatWarpScan,    // one block, no sub-block level: warp-cooperative scan
    kStatEntries,     // per-element entries read (pre, suf, mpre, msuf)
    kStatTable,       // small-table words read (sparse table, micro offsets and minima)
    kStatSectors,     // 32-byte sectors of A read by scans
    kStatInvalid,     // invalid queries
    kStatCount
};
struct QStats {
    uint32_t c[kStatCount];
};

// Leftmost best of blocks a..b (a <= b < nb) from the sparse table: two
// entries of level floor(log2(b - a + 1)), one when the window is exact.
template <bool STATS>
__device__ __forceinline__ Entry st_probe(const V1View &v, uint32_t a, uint32_t b, uint64_t pol,
                                          QStats &s) {
    const int lev = ilog2(b - a + 1u);
    const uint64_t row = static_cast<uint64_t>(lev) * v.nb;
    const uint64_t size = static_cast<uint64_t>(v.levels) * v.nb;
    const uint32_t c = b + 1u - (1u << lev);
    const Entry x = ld_entry_keep(v.st, row + a, size, pol);
    Entry y = x;
    if (c != a) y = ld_entry_keep(v.st, row + c, size, pol);
    if constexpr (STATS) s.c[kStatTable] += (c != a) ? 2u : 1u;
    return better(x, y);
}

// Leftmost best of micro-blocks a..b (a <= b, b - a + 1 < 2^mlevels): the
// offsets of the two windows' best micro-blocks, then their minima.
template <bool STATS>
__device__ __forceinline__ Entry micro_probe(const V1View &v, uint32_t a, uint32_t b, uint64_t pol,
                                             QStats &s) {
    const int lev = ilog2(b - a + 1u);
    uint32_t x = a, y = b + 1u - (1u << lev);
    if (lev > 0) {
        const uint64_t row = static_cast<uint64_t>(lev - 1) * v.nmicro;
        const bool two = y != x;
        const uint32_t ox = ld_moff(v, row + x, pol);
        const uint32_t oy = two ? ld_moff(v, row + y, pol) : ox;
        if constexpr (STATS) s.c[kStatTable] += two ? 2u : 1u;
        x += ox;
        y += oy;
    }
    const Entry ex = ld_entry_keep(v.mst, x, v.nmicro, pol);
    Entry ey = ex;
    if (y != x) ey = ld_entry_keep(v.mst, y, v.nmicro, pol);
    if constexpr (STATS) s.c[kStatTable] += (y != x) ? 2u : 1u;
    return better(ex, ey);
}

template <bool STATS>
__device__ __forceinline__ Entry unit_probe(const V1View &v, bool micro, uint32_t a, uint32_t b,
                                            uint64_t pol, QStats &s) {
    return micro ? micro_probe<STATS>(v, a, b, pol, s) : st_probe<STATS>(v, a, b, pol, s);
}

// S[l]: best of A[l .. end of l's unit]; P[r]: best of A[start of r's unit .. r].
// The micro-level entries are read with streaming loads (they are read once,
// and would otherwise push the micro table out of L2).
template <bool STATS>
__device__ __forceinline__ Entry left_entry(const V1View &v, bool micro, uint32_t l, QStats &s) {
    if constexpr (STATS) s.c[kStatEntries] += 1u;
    return micro ? ld_entry_cs(v.msuf, l, v.n) : ld_entry(v.suf, l, v.n);
}
template <bool STATS>
__device__ __forceinline__ Entry right_entry(const V1View &v, bool micro, uint32_t r, QStats &s) {
    if constexpr (STATS) s.c[kStatEntries] += 1u;
    return micro ? ld_entry_cs(v.mpre, r, v.n) : ld_entry(v.pre, r, v.n);
}

// 32-byte sectors of the local range A[a..b]
__device__ __forceinline__ uint32_t range_sectors(const V1View &v, uint32_t a, uint32_t b) {
    return static_cast<uint32_t>(((v.off + b) >> 3) - ((v.off + a) >> 3) + 1);
}

// the probe that served a queued query (its code's low bits)
enum : uint32_t {
    kPathTable = 1,       // superset probe over blocks lB..rB
    kPathMicroTable = 2,  // superset probe over micro-blocks ml..mr
    kPathBlock = 4,       // one block, no sub-block level (an edge entry settles it)
};

// ---- the queued form (query_kernel, batch_kernel's query phase) -------------
//
// Settling a query that its probe leaves open inside the same step would
// make a warp wait for the slowest lane's chain of dependent loads (entry,
// narrower probe, then maybe the rest). The queued form is specialised at
// compile time on the key mode and on whether the index has the sub-block
// level, and its main pass does only the superset probe: a query the probe
// settles is stored at once; one it leaves open goes into a per-warp queue
// in shared memory, and whenever 32 are waiting the warp settles them
// together, one per lane (finish_miss).

// code of a queued query: its path, and kMissLeft when the probe's best
// lay left of l (else right of r)
constexpr uint32_t kMissLeft = 8u;

// Shared-memory slot of one thread for a line of values: up to 9 16-byte
// chunks (a 32-element micro-block not starting on a chunk boundary).
constexpr int kLineChunks = 10;

// Leftmost best of local A[lo..hi] (inside one micro-block) through an
// asynchronous copy of the 16-byte chunks that cover it into the calling
// thread's slot (cp.async.cg, bypassing L1), then a scan of the slot: one
// memory round trip, few registers. The values base must be 16-byte
// aligned; chunks past the end of the buffer are not read.
template <uint32_t MODE>
__device__ __forceinline__ Entry line_min_async(const V1View &v, uint32_t lo, uint32_t hi,
                                                uint4 *slot) {
    const int64_t glo = v.off + lo, ghi = v.off + hi;
    const int64_t p0 = glo & ~int64_t(3);
    const int nc = static_cast<int>(((ghi & ~int64_t(3)) - p0) / 4) + 1;
    const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(slot));
    const float *base = v.A + p0;  // 16-byte aligned
    const int64_t room = v.limit - p0;  // elements from base to the end of the buffer
    if (room >= 4 * nc) {
#pragma unroll 1
        for (int c = 0; c < nc; ++c)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;"
                         :: "r"(sbase + 16u * c), "l"(base + 4 * c) : "memory");
    } else {
        // the buffer ends inside the line: copy what lies inside it
#pragma unroll 1
        for (int c = 0; c < nc; ++c) {
            const int64_t avail = room - 4 * c;  // elements of the chunk inside the buffer
            const uint32_t bytes = avail >= 4 ? 16u : static_cast<uint32_t>(avail > 0 ? avail * 4 : 0);
            if (rmq_chk(p0 >= 0 && bytes > 0u))
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;"
                             :: "r"(sbase + 16u * c), "l"(base + 4 * c), "r"(bytes) : "memory");
        }
    }
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
    // 32-bit keys first, one composite at the end: the smallest key and the
    // first local index holding it (strict <, in index order) is the
    // leftmost best; if every key is the largest, that is element lo.
    const int32_t l0 = static_cast<int32_t>(p0 - v.off);  // local index of slot[0].x
    uint32_t km = 0xffffffffu, pos = lo, nz = 0u;
#pragma unroll 1
    for (int c = 0; c < nc; ++c) {
        const uint4 f = slot[c];
        const uint32_t w[4] = {f.x, f.y, f.z, f.w};
        const int32_t c0 = l0 + 4 * c;  // local index of w[0]
        if constexpr (MODE == kFloatMin || MODE == kFloatMax) {
            // the chunk's IEEE minimum (maximum) over its values in [lo, hi]
            // (others as NaN, which it skips), the first value equal to it,
            // and one key from that value's bits
            float x[4];
#pragma unroll
            for (int k = 0; k < 4; ++k)
                x[k] = __uint_as_float(
                    static_cast<uint32_t>(c0 + k - static_cast<int32_t>(lo)) <= hi - lo
                        ? w[k] : 0x7fc00000u);
            const float m = MODE == kFloatMin ? fminf(fminf(x[0], x[1]), fminf(x[2], x[3]))
                                              : fmaxf(fmaxf(x[0], x[1]), fmaxf(x[2], x[3]));
            const uint32_t p = x[0] == m ? 0u : x[1] == m ? 1u : x[2] == m ? 2u : x[3] == m ? 3u : 0u;
            const uint32_t wb = __float_as_uint(p == 0u ? x[0] : p == 1u ? x[1] : p == 2u ? x[2] : x[3]);
            const uint32_t kk = key_of(wb, MODE);
            if (kk < km) {
                km = kk;
                pos = static_cast<uint32_t>(c0) + p;
                nz = negzero_of(wb, MODE);
            }
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int32_t li = c0 + k;
                const uint32_t kk = key_of(w[k], MODE);
                if (static_cast<uint32_t>(li - static_cast<int32_t>(lo)) <= hi - lo && kk < km) {
                    km = kk;
                    pos = static_cast<uint32_t>(li);
                    nz = negzero_of(w[k], MODE);
                }
            }
        }
    }
    return (static_cast<uint64_t>(km) << 32) | (pos << 1) | nz;
}

// Leftmost best of local A[lo..hi] inside one micro-block for a miss: the
// asynchronous line copy when the thread has a slot and the values are
// aligned, else the thread's own scan.
template <bool ALIGNED, uint32_t MODE>
__device__ __forceinline__ Entry line_min(const V1View &v, uint32_t lo, uint32_t hi, uint4 *slot) {
    if (ALIGNED && slot) return line_min_async<MODE>(v, lo, hi, slot);
    return thread_range_min<ALIGNED>(v, lo, hi, MODE);
}

// With per-element entries, the part of a query in its end unit on the
// left, [l, end of l's unit] (micro-block, or block), and on the right,
// [start of r's unit, r]: one entry each.
template <bool STATS>
__device__ __forceinline__ Entry left_part(const V1View &v, bool micro, uint32_t l, QStats &s) {
    return left_entry<STATS>(v, micro, l, s);
}
template <bool STATS>
__device__ __forceinline__ Entry right_part(const V1View &v, bool micro, uint32_t r, QStats &s) {
    return right_entry<STATS>(v, micro, r, s);
}

// Light index: the query's part in its end unit on one side, [l, end of
// l's unit] (left) or [start of r's unit, r] (right): one line of values
// inside the end micro-block, plus for a block unit the micro table over
// the block's whole micro-blocks on that side. The side is a value, not a
// branch, so lanes settling left and right parts run the same code.
template <bool ALIGNED, uint32_t MODE, bool STATS>
__device__ __forceinline__ Entry light_part(const V1View &v, bool micro, bool left, uint32_t a,
                                            uint32_t b, uint32_t l, uint32_t r, uint64_t pol,
                                            QStats &s, uint4 *slot) {
    const uint32_t lo = left ? l : (r & ~31u);
    const uint32_t hi = left ? min(l | 31u, v.n - 1u) : r;
    const Entry line = line_min<ALIGNED, MODE>(v, lo, hi, slot);
    if constexpr (STATS) s.c[kStatSectors] += range_sectors(v, lo, hi);
    if (micro) return line;
    // block a is full when a < b: its last micro-block ends inside the array
    const uint32_t ml = l >> 5, me = (((a + 1u) * v.bs) >> 5) - 1u;
    const uint32_t mr = r >> 5, ms = (b * v.bs) >> 5;
    const bool has = left ? ml < me : ms < mr;
    if (!has) return line;
    return better(line, micro_probe<STATS>(v, left ? ml + 1u : ms, left ? me : mr - 1u, pol, s));
}

// Settles one query whose superset best lay outside [l, r] (or, without
// the sub-block level, inside one block at an edge): the query's part in
// the end unit on that side and a narrower probe, loaded together, then
// only if needed the other end's part and the middle units.
template <bool ALIGNED, bool MICRO, bool LIGHT, uint32_t MODE, bool STATS>
__device__ __forceinline__ Entry finish_miss(const V1View &v, uint32_t l, uint32_t r,
                                             uint32_t code, uint64_t pol, QStats &s,
                                             uint4 *slot) {
    const uint32_t path = code & 7u;
    if constexpr (LIGHT) {
        // one copy of the part's code: the second pass (the other end, after
        // the middle units) runs only for the rare query the narrower probe
        // does not settle
        const bool micro = path == kPathMicroTable;
        const uint32_t a = micro ? (l >> 5) : div31(l, v.dv);
        const uint32_t b = micro ? (r >> 5) : div31(r, v.dv);
        bool left = (code & kMissLeft) != 0u;
        const Entry e2 = unit_probe<STATS>(v, micro, left ? a + 1u : a, left ? b : b - 1u, pol, s);
        Entry res = kEntryNone;
#pragma unroll 1
        for (int pass = 0; pass < 2; ++pass) {
            res = better(res, light_part<ALIGNED, MODE, STATS>(v, micro, left, a, b, l, r, pol, s,
                                                               slot));
            if (pass == 1) break;
            const uint32_t m2 = entry_idx(e2);
            if (left ? m2 <= r : m2 >= l) {
                if constexpr (STATS) s.c[kStatSecond] += 1u;
                return better(res, e2);
            }
            if constexpr (STATS) s.c[kStatFull] += 1u;
            if (b - a >= 2u) res = better(res, unit_probe<STATS>(v, micro, a + 1u, b - 1u, pol, s));
            left = !left;
        }
        return res;
    } else {
        if (path == kPathBlock) {
            if constexpr (STATS) s.c[kStatBlockEdge] += 1u;
            const uint32_t bstart = div31(l, v.dv) * v.bs;
            const uint32_t bend = min(bstart + v.bs, v.n) - 1u;
            return r == bend ? left_entry<STATS>(v, false, l, s) : right_entry<STATS>(v, false, r, s);
        }
        const bool micro = path == kPathMicroTable;
        const uint32_t a = micro ? (l >> 5) : div31(l, v.dv);
        const uint32_t b = micro ? (r >> 5) : div31(r, v.dv);
        const bool left = (code & kMissLeft) != 0u;
        // the narrower probe first: its loads are in flight while the part's
        // entry is loaded
        const Entry e2 = left ? unit_probe<STATS>(v, micro, a + 1u, b, pol, s)
                              : unit_probe<STATS>(v, micro, a, b - 1u, pol, s);
        const Entry e1 = left ? left_part<STATS>(v, micro, l, s) : right_part<STATS>(v, micro, r, s);
        const uint32_t m2 = entry_idx(e2);
        if (left ? m2 <= r : m2 >= l) {
            if constexpr (STATS) s.c[kStatSecond] += 1u;
            return better(e1, e2);
        }
        if constexpr (STATS) s.c[kStatFull] += 1u;
        const Entry mid = (b - a >= 2u) ? unit_probe<STATS>(v, micro, a + 1u, b - 1u, pol, s)
                                        : kEntryNone;
        const Entry other = left ? right_part<STATS>(v, micro, r, s) : left_part<STATS>(v, micro, l, s);
        return better(better(e1, other), mid);
    }
}

// One warp's queue: up to 31 waiting queries plus the 32 that one query
// slot of a step can add.
struct MissQueue {
    static constexpr int kCap = 64;
    int64_t qi[kCap];
    uint32_t l[kCap];
    uint32_t r[kCap];
    uint8_t code[kCap];
};

// Settles the last min(count, 32) queued queries, one per lane; the whole
// warp calls it (count is warp-uniform).
// `lines`: kLineChunks chunks of shared memory per thread of the CTA for
// the light index's line copies, or null.
template <bool ALIGNED, bool MICRO, bool LIGHT, uint32_t MODE, bool STATS>
__device__ __forceinline__ void drain_misses(const V1View &v, const QueryOut &o, MissQueue &mq,
                                             uint32_t &count, uint64_t pol, QStats &s,
                                             uint4 *lines) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t take = count < 32u ? count : 32u;
    __syncwarp();
    if (lane < take) {
        const uint32_t e = count - take + lane;
        const Entry r = finish_miss<ALIGNED, MICRO, LIGHT, MODE, STATS>(
            v, mq.l[e], mq.r[e], mq.code[e], pol, s,
            lines ? lines + threadIdx.x * kLineChunks : nullptr);
        put_result(o, mq.qi[e], r, MODE);
    }
    __syncwarp();
    count -= take;
}

// The bits of an entry's element for key mode MODE, without branches
// (unkey for a mode known at compile time).
template <uint32_t MODE>
__device__ __forceinline__ uint32_t decode_bits(Entry e) {
    const uint32_t k = static_cast<uint32_t>(e >> 32);
    if constexpr (MODE == kIntMin) {
        return k ^ 0x80000000u;
    } else if constexpr (MODE == kIntMax) {
        return k ^ 0x7fffffffu;
    } else {
        const uint32_t nz = static_cast<uint32_t>(e) & 1u;
        // f = fkey(bits): bits | 2^31 for a positive value (2^31 for +-0,
        // negzero telling them apart), ~bits for a negative one
        const uint32_t f = (MODE == kFloatMax) ? ~k : k;
        const uint32_t b = (f & 0x80000000u) ? ((f & 0x7fffffffu) | (nz << 31)) : ~f;
        return k == 0xffffffffu ? 0x7fc00000u : b;  // NaN: the canonical quiet NaN
    }
}

// The superset probe of the queued form for a valid query not inside one
// micro-block: through the micro table when the query's micro-blocks fit
// it (`mic`), else through the block table (two entries, one straight
// sequence).
template <bool MICRO, bool STATS>
__device__ __forceinline__ Entry superset_probe(const V1View &v, uint32_t l, uint32_t r,
                                                uint64_t pol, QStats &s, bool &mic) {
    const uint32_t ml = l >> 5, mr = r >> 5;
    mic = MICRO && mr - ml < v.micro_span;
    const uint32_t a = mic ? ml : div31(l, v.dv);
    const uint32_t b = mic ? mr : div31(r, v.dv);
    const int lev = ilog2(b - a + 1u);
    uint32_t x = a, y = b + 1u - (1u << lev);
    if (MICRO && mic) {
        // lev >= 1: the query spans at least two micro-blocks. The two
        // windows overlap, so 1-byte offsets often share an aligned 8-byte
        // word (one load), and both windows often point at the same best
        // micro-block (one minimum load).
        const uint64_t row = static_cast<uint64_t>(lev - 1) * v.nmicro;
        if (v.moff_bytes == 1u && ((row + x) >> 3) == ((row + y) >> 3)) {
            const uint64_t w = ld_moff_word(v, row + x, pol);
            x += static_cast<uint32_t>(w >> (8 * ((row + x) & 7))) & 0xffu;
            y += static_cast<uint32_t>(w >> (8 * ((row + y) & 7))) & 0xffu;
            if constexpr (STATS) s.c[kStatTable] += 1u;
        } else {
            x += ld_moff(v, row + x, pol);
            y += ld_moff(v, row + y, pol);
            if constexpr (STATS) s.c[kStatTable] += 2u;
        }
        const Entry e1 = ld_entry_keep(v.mst, x, v.nmicro, pol);
        Entry e2 = e1;
        if (x != y) e2 = ld_entry_keep(v.mst, y, v.nmicro, pol);
        if constexpr (STATS) s.c[kStatTable] += x != y ? 2u : 1u;
        return better(e1, e2);
    }
    const Entry *t = v.st + static_cast<uint64_t>(lev) * v.nb;
    const uint64_t size = static_cast<uint64_t>(v.levels - lev) * v.nb;
    const Entry e1 = ld_entry_keep(t, x, size, pol);
    const Entry e2 = ld_entry_keep(t, y, size, pol);
    if constexpr (STATS) s.c[kStatTable] += 2u;
    return better(e1, e2);
}

// One step of the queued form over queries [base, base + cnt) (cnt <=
// THREADS * QPT): thread t handles base + t + k * THREADS, already loaded
// into qq. FULL: cnt == THREADS * QPT, so no query needs a bounds check.
// MICRO: the index has the sub-block level (then every query inside one
// block spans few enough micro-blocks for the micro table, and only the
// block table serves longer ones). LIGHT: a light index (no per-element
// entries; `lines` holds the threads' line slots). `count` carries the warp's queue length
// from step to step; the caller drains the rest.
template <bool ALIGNED, bool MICRO, bool LIGHT, uint32_t MODE, int THREADS, int QPT, bool STATS,
          bool FULL>
__device__ __forceinline__ void answer_step_queued(const V1View &v, const QueryOut &o,
                                                   int64_t base, uint32_t cnt,
                                                   const int2 (&qq)[QPT], QStats &s,
                                                   MissQueue &mq, uint32_t &count,
                                                   uint4 *lines = nullptr) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint64_t pol = l2_keep_policy();
    float *const vs = o.val ? o.val + base : nullptr;
    int32_t *const is = o.idx ? o.idx + base : nullptr;
    Entry res[QPT];
    bool ok[QPT], scan[QPT], mic[QPT];
#pragma unroll
    for (int k = 0; k < QPT; ++k) {
        const uint32_t j = threadIdx.x + k * THREADS;
        const uint32_t l = static_cast<uint32_t>(qq[k].x), r = static_cast<uint32_t>(qq[k].y);
        ok[k] = (FULL || j < cnt) && qq[k].x >= 0 && l <= r && r < v.n;
        scan[k] = MICRO && (l >> 5) == (r >> 5);
        mic[k] = false;
        res[k] = kEntryNone;
        if (ok[k] && !scan[k]) res[k] = superset_probe<MICRO, STATS>(v, l, r, pol, s, mic[k]);
    }
    bool miss[QPT];
    bool any_miss = false;
#pragma unroll
    for (int k = 0; k < QPT; ++k) {
        const uint32_t j = threadIdx.x + k * THREADS;
        const uint32_t l = static_cast<uint32_t>(qq[k].x), r = static_cast<uint32_t>(qq[k].y);
        miss[k] = false;
        if (!ok[k]) {
            if (FULL || j < cnt) {
                put_invalid(o, base + j);
                if constexpr (STATS) s.c[kStatInvalid] += 1u;
            }
            continue;
        }
        if (MICRO && scan[k]) {
            res[k] = thread_range_min<ALIGNED>(v, l, r, MODE);
            if constexpr (STATS) {
                s.c[kStatMicroScan] += 1u;
                s.c[kStatSectors] += range_sectors(v, l, r);
            }
        } else {
            miss[k] = entry_idx(res[k]) - l > r - l;
            if constexpr (STATS) s.c[kStatFirst] += miss[k] ? 0u : 1u;
        }
        any_miss |= miss[k];
        // the probe's answer is stored even for a query it leaves open: the
        // drain (same warp, after __syncwarp) or the warp scan (same thread)
        // overwrites it, and whole-warp stores keep the output lines whole
        if (vs) __stcs(reinterpret_cast<unsigned int *>(vs) + j, decode_bits<MODE>(res[k]));
        if (is) __stcs(is + j, static_cast<int32_t>(entry_idx(res[k])));
    }
    if (!__any_sync(0xffffffffu, any_miss)) return;
    bool wscan[QPT];
#pragma unroll
    for (int k = 0; k < QPT; ++k) {
        const uint32_t l = static_cast<uint32_t>(qq[k].x), r = static_cast<uint32_t>(qq[k].y);
        uint32_t code = mic[k] ? kPathMicroTable : kPathTable;
        wscan[k] = false;
        if (!MICRO && miss[k]) {
            const uint32_t lB = div31(l, v.dv);
            if (lB == div31(r, v.dv)) {
                // one block without the sub-block level: an edge entry when the
                // query touches the block's edge, else the warp scans it
                const uint32_t bstart = lB * v.bs;
                const uint32_t bend = min(bstart + v.bs, v.n) - 1u;
                code = kPathBlock;
                if (r != bend && l != bstart) {
                    miss[k] = false;
                    wscan[k] = true;
                }
            }
        }
        const unsigned mask = __ballot_sync(0xffffffffu, miss[k]);
        if (miss[k]) {
            const uint32_t e = count + __popc(mask & ((1u << lane) - 1u));
            if (code != kPathBlock && entry_idx(res[k]) < l) code |= kMissLeft;
            mq.qi[e] = base + threadIdx.x + k * THREADS;
            mq.l[e] = l;
            mq.r[e] = r;
            mq.code[e] = static_cast<uint8_t>(code);
        }
        count += __popc(mask);
        if (count >= 32u) drain_misses<ALIGNED, MICRO, LIGHT, MODE, STATS>(v, o, mq, count, pol, s, lines);
    }
    if constexpr (!MICRO) {
#pragma unroll
        for (int k = 0; k < QPT; ++k) {
            unsigned mask = __ballot_sync(0xffffffffu, wscan[k]);
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1u;
                const uint32_t ls = __shfl_sync(0xffffffffu, static_cast<uint32_t>(qq[k].x), src);
                const uint32_t rs = __shfl_sync(0xffffffffu, static_cast<uint32_t>(qq[k].y), src);
                const Entry e = warp_scan_range<ALIGNED>(v, ls, rs, static_cast<int>(lane), MODE);
                if (static_cast<int>(lane) == src) {
                    put_result(o, base + threadIdx.x + k * THREADS, e, MODE);
                    if constexpr (STATS) {
                        s.c[kStatWarpScan] += 1u;
                        s.c[kStatSectors] += range_sectors(v, ls, rs);
                    }
                }
            }
        }
    }
}

// Adds a thread's counters to the launch's device counters (one atomic per
// warp and counter).
__device__ __forceinline__ void flush_stats(const QStats &s, unsigned long long *out) {
#pragma unroll
    for (int c = 0; c < kStatCount; ++c) {
        unsigned long long x = s.c[c];
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) x += __shfl_down_sync(0xffffffffu, x, d);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(out + c, x);
    }
}

// Answer queries [q0, q1) of one array with the whole CTA (THREADS
// threads) in the queued form, QPT queries per thread per step; `mq` is the
// calling warp's queue, empty on entry and on return. LIGHT: a light index,
// `lines` the CTA's line slots (kLineChunks chunks per thread).
template <bool ALIGNED, bool MICRO, bool LIGHT, uint32_t MODE, int THREADS, int QPT>
__device__ __forceinline__ void answer_range_queued(const V1View &v, const QueryOut &o,
                                                    int64_t q0, int64_t q1, MissQueue &mq,
                                                    uint4 *lines) {
    constexpr int64_t step = static_cast<int64_t>(THREADS) * QPT;
    QStats s;
    uint32_t waiting = 0;
    for (int64_t base = q0; base < q1; base += step) {
        int2 qq[QPT];
        load_queries<QPT>(o, base, q1, qq);
        if (base + step <= q1)
            answer_step_queued<ALIGNED, MICRO, LIGHT, MODE, THREADS, QPT, false, true>(
                v, o, base, static_cast<uint32_t>(step), qq, s, mq, waiting, lines);
        else
            answer_step_queued<ALIGNED, MICRO, LIGHT, MODE, THREADS, QPT, false, false>(
                v, o, base, static_cast<uint32_t>(q1 - base), qq, s, mq, waiting, lines);
    }
    if (waiting)
        drain_misses<ALIGNED, MICRO, LIGHT, MODE, false>(v, o, mq, waiting, l2_keep_policy(), s,
                                                         lines);
}

}  // namespace rmq
