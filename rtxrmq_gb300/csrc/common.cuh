// common.cuh -- types and helpers shared by the build, query, batch and
// gradient kernels and by the host code of the C ABI.
//
// Ordering. Every comparison in the engine is made on a 64-bit composite
//     (fkey(value) << 32) | index
// so that a plain unsigned min returns the smallest value and, among equal
// values, the smallest index. fkey() is order preserving for the float `<`
// used by the reference's oracles (src/cpu_methods.h:42-53,
// src/cuda_methods.cuh:23-42): -0.0 and +0.0 map to one key, NaN maps above
// +inf. Stored entries keep the raw float bits, so results are bit-exact.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define RMQ_HD __host__ __device__ __forceinline__

namespace rmq {

// One structure entry: raw float bits of a minimum and its global index.
struct __align__(8) Entry {
    uint32_t bits;
    uint32_t idx;
};

// Order-preserving map float bits -> uint32 (see file comment).
RMQ_HD uint32_t fkey(uint32_t b) {
    const uint32_t a = b & 0x7fffffffu;
    if (a > 0x7f800000u) return 0xffffffffu;   // NaN: after +inf
    if (a == 0u) return 0x80000000u;           // -0.0 == +0.0
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

// Inverse of fkey for every key it produces; `negzero` restores -0.0.
RMQ_HD uint32_t funkey(uint32_t k, uint32_t negzero) {
    if (k == 0xffffffffu) return 0x7fc00000u;  // canonical quiet NaN
    if (k == 0x80000000u) return negzero ? 0x80000000u : 0u;
    return (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
}

RMQ_HD uint64_t entry_comp(Entry e) {
    return (static_cast<uint64_t>(fkey(e.bits)) << 32) | e.idx;
}

// Leftmost minimum of two entries.
RMQ_HD Entry better(Entry a, Entry b) {
    return entry_comp(b) < entry_comp(a) ? b : a;
}

RMQ_HD Entry entry_max() {
    Entry e;
    e.bits = 0x7fc00000u;
    e.idx = 0xffffffffu;
    return e;
}

// Exact unsigned division of x < 2^31 by a runtime divisor d >= 1:
//   q = floor(x * m / 2^(31 + s)),  s = ceil(log2 d),  m = ceil(2^(31+s) / d).
// With e = m*d - 2^(31+s) < d <= 2^s and x < 2^31 the error term
// x*e / (d * 2^(31+s)) stays below 1/d, so the floor is exact
// (Granlund & Montgomery, PLDI 1994, round-up variant).
struct Div31 {
    uint32_t d;
    uint32_t m;      // multiplier (unused for powers of two)
    uint32_t shift;  // s - 1 after the high multiply, or log2 d for pow2
    uint32_t pow2;
};

inline Div31 make_div31(uint32_t d) {
    Div31 r;
    r.d = d;
    uint32_t s = 0;
    while ((1ull << s) < d) ++s;
    if ((1u << s) == d) {
        r.pow2 = 1;
        r.m = 0;
        r.shift = s;
    } else {
        r.pow2 = 0;
        const uint64_t num = 1ull << (31 + s);
        r.m = static_cast<uint32_t>((num + d - 1) / d);
        r.shift = s - 1;
    }
    return r;
}

RMQ_HD uint32_t div31(uint32_t x, const Div31 &D) {
    if (D.pow2) return x >> D.shift;
#ifdef __CUDA_ARCH__
    return __umulhi(x, D.m) >> D.shift;
#else
    return static_cast<uint32_t>((static_cast<uint64_t>(x) * D.m) >> 32) >> D.shift;
#endif
}

// floor(log2 x) for x >= 1
RMQ_HD int ilog2(uint32_t x) {
#ifdef __CUDA_ARCH__
    return 31 - __clz(x);
#else
    return 31 - __builtin_clz(x);
#endif
}

}  // namespace rmq
