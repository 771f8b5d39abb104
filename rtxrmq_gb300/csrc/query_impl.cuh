// query_impl.cuh -- the CTA-level query body shared by the plain query kernel
// (query.cu) and the persistent batch kernel (batch.cu).
//
// It replaces RTX_blocks' ray programs (src/rtx_kernels.cu:85-193 for
// values, 350-465 for indices). The reference fires up to three rays per
// query: one through the fully covered blocks lB+1..rB-1, one through the
// left partial block and one through the right partial block, and keeps the
// closest hit. Here the same decomposition is answered from arrays:
//   left partial block   -> suf[l]
//   right partial block  -> pre[r]
//   full blocks between  -> two sparse-table entries (L2-resident)
// A query inside one block (the reference's single-ray case,
// src/rtx_kernels.cu:116-135) is answered from pre/suf when it touches a
// block edge; otherwise through the sub-block level when the index has one
// (32-element micro-blocks: msuf[l], mpre[r] and two micro-table entries, or
// one thread's scan of a single 128-byte line), and by a warp-cooperative
// scan of A[l..r] reducing the composites with __reduce_min_sync when it
// does not. All comparisons are unsigned minima of the composites of
// common.cuh; only the final answer is decoded.
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

// The tables a query reads beside its two random per-element lookups (the
// sparse table over block minima, the micro table) are small; their loads
// carry an L2 evict-last policy (PTX createpolicy + ld.L2::cache_hint) so
// that the per-element lines streaming through L2 evict them last. No L2
// carve-out is set aside, unlike a persisting access-policy window. The
// policy is made at each load: holding it across the step costs registers
// (and resident CTAs) for nothing measurable.
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

// Leftmost minimum of local A[a..b] (b - a < 32, at most 9 16-byte loads)
// computed by one thread.
template <bool ALIGNED>
__device__ __forceinline__ Entry thread_range_min(const V1View &v, uint32_t a, uint32_t b) {
    const int64_t aa = v.off + a, ab = v.off + b;
    Entry best = kEntryNone;
    if (ALIGNED) {
        const int64_t p0 = aa & ~int64_t(3);
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const int64_t p = p0 + 4 * k;
            if (p <= ab) {
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
                        best = better(best, make_entry(w[c], static_cast<uint32_t>(g - v.off), v.kmode));
                }
            }
        }
    } else {
        for (int64_t g = aa; g <= ab; ++g)
            best = better(best, make_entry(ld_elem(v, g), static_cast<uint32_t>(g - v.off), v.kmode));
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
                                                 int lane) {
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
                    best = better(best, make_entry(b[c], static_cast<uint32_t>(g - v.off), v.kmode));
            }
        }
    } else {
        for (int64_t g = al + lane; g <= ar; g += 32)
            best = better(best, make_entry(ld_elem(v, g), static_cast<uint32_t>(g - v.off), v.kmode));
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

// One step of the CTA: the QPT * blockDim.x queries starting at `base`,
// already loaded into qq. Uniform across the CTA (warp-cooperative scans
// need full warps).
template <bool ALIGNED, int QPT>
__device__ __forceinline__ void answer_step(const V1View &v, const QueryOut &o, int64_t base,
                                            int64_t q1, const int2 (&qq)[QPT]) {
    const int lane = threadIdx.x & 31;
    {
        uint32_t l[QPT], r[QPT];
        bool act[QPT], ok[QPT], scan[QPT];
        Entry es[QPT], ep[QPT], ea[QPT], eb[QPT];
#pragma unroll
        for (int k = 0; k < QPT; ++k) {
            const int64_t i = base + threadIdx.x + static_cast<int64_t>(k) * blockDim.x;
            act[k] = i < q1;
            ok[k] = act[k] && qq[k].x >= 0 && qq[k].x <= qq[k].y &&
                    static_cast<uint32_t>(qq[k].y) < v.n;
            l[k] = ok[k] ? static_cast<uint32_t>(qq[k].x) : 0u;
            r[k] = ok[k] ? static_cast<uint32_t>(qq[k].y) : 0u;
        }
#pragma unroll
        for (int k = 0; k < QPT; ++k) {
            const uint32_t lB = div31(l[k], v.dv);
            const uint32_t rB = div31(r[k], v.dv);
            const bool cross = ok[k] && lB != rB;
            const uint32_t bstart = lB * v.bs;
            const uint32_t bend = min(bstart + v.bs, v.n) - 1u;
            const bool same = ok[k] && lB == rB;
            const bool use_suf = cross || (same && r[k] == bend);
            const bool use_pre = cross || (same && l[k] == bstart);
            scan[k] = same && !use_suf && !use_pre;
            es[k] = use_suf ? ld_entry(v.suf, l[k], v.n) : kEntryNone;
            ep[k] = use_pre ? ld_entry(v.pre, r[k], v.n) : kEntryNone;
            ea[k] = kEntryNone;
            eb[k] = kEntryNone;
            if (cross && rB - lB >= 2u) {
                const uint32_t lo = lB + 1u, hi = rB - 1u;
                const int lev = ilog2(hi - lo + 1u);
                const uint64_t row = static_cast<uint64_t>(lev) * v.nb;
                const uint64_t size = static_cast<uint64_t>(v.levels) * v.nb;
                ea[k] = ld_entry_keep(v.st, row + lo, size, l2_keep_policy());
                eb[k] = ld_entry_keep(v.st, row + hi + 1u - (1u << lev), size, l2_keep_policy());
            }
            if (v.mst && scan[k] && (l[k] >> 5) != (r[k] >> 5)) {
                // same block through the sub-block level, issued here beside the
                // other queries' lookups so that all of them are in flight at
                // once: the partial micro-blocks at both ends from the
                // in-micro-block suffix / prefix minima, the micro-blocks between
                // from the micro table (two offsets, then the two minima they
                // point at; L2-resident). Only a query inside one micro-block
                // is left to scan.
                const uint32_t ml = l[k] >> 5, mr = r[k] >> 5;
                es[k] = ld_entry_cs(v.msuf, l[k], v.n);
                ep[k] = ld_entry_cs(v.mpre, r[k], v.n);
                if (mr - ml >= 2u) {
                    const uint32_t lo = ml + 1u, hi = mr - 1u;
                    const int lev = ilog2(hi - lo + 1u);
                    uint32_t a = lo, b = hi + 1u - (1u << lev);
                    if (lev > 0) {
                        const uint64_t row = static_cast<uint64_t>(lev - 1) * v.nmicro;
                        a += ld_moff(v, row + a, l2_keep_policy());
                        b += ld_moff(v, row + b, l2_keep_policy());
                    }
                    ea[k] = ld_entry_keep(v.mst, a, v.nmicro, l2_keep_policy());
                    eb[k] = ld_entry_keep(v.mst, b, v.nmicro, l2_keep_policy());
                }
                scan[k] = false;
            }
        }
        if (v.mst) {
            // sub-block level: every query of the step is answered by its own
            // thread (a query inside one micro-block scans that micro-block's
            // line), so each result is stored once and a warp's 128-byte
            // output line is written by one instruction (partial-line writes
            // cost extra transactions, most of all to host memory)
#pragma unroll
            for (int k = 0; k < QPT; ++k) {
                if (!act[k]) continue;
                const int64_t i = base + threadIdx.x + static_cast<int64_t>(k) * blockDim.x;
                if (!ok[k]) {
                    put_invalid(o, i);
                    continue;
                }
                const Entry e = scan[k] ? thread_range_min<ALIGNED>(v, l[k], r[k])
                                        : better(better(es[k], ep[k]), better(ea[k], eb[k]));
                put_result(o, i, e, v.kmode);
            }
            return;
        }
#pragma unroll
        for (int k = 0; k < QPT; ++k) {
            if (act[k] && !scan[k]) {
                const int64_t i = base + threadIdx.x + static_cast<int64_t>(k) * blockDim.x;
                if (ok[k])
                    put_result(o, i, better(better(es[k], ep[k]), better(ea[k], eb[k])), v.kmode);
                else
                    put_invalid(o, i);
            }
        }
#pragma unroll
        for (int k = 0; k < QPT; ++k) {
            unsigned mask = __ballot_sync(0xffffffffu, scan[k]);
            while (mask) {
                const int src = __ffs(mask) - 1;
                mask &= mask - 1u;
                const uint32_t ls = __shfl_sync(0xffffffffu, l[k], src);
                const uint32_t rs = __shfl_sync(0xffffffffu, r[k], src);
                const Entry e = warp_scan_range<ALIGNED>(v, ls, rs, lane);
                if (lane == src)
                    put_result(o, base + threadIdx.x + static_cast<int64_t>(k) * blockDim.x, e,
                               v.kmode);
            }
        }
    }
}

// Answer queries [q0, q1) of one array with the whole CTA, QPT queries per
// thread per step.
template <bool ALIGNED, int QPT>
__device__ __forceinline__ void answer_range(const V1View &v, const QueryOut &o, int64_t q0,
                                             int64_t q1) {
    const int64_t step = static_cast<int64_t>(blockDim.x) * QPT;
    for (int64_t base = q0; base < q1; base += step) {
        int2 qq[QPT];
        load_queries<QPT>(o, base, q1, qq);
        answer_step<ALIGNED, QPT>(v, o, base, q1, qq);
    }
}

}  // namespace rmq
