// common.cuh -- types and helpers shared by the build, query, batch and
// gradient kernels and by the host code of the C ABI.
//
// Ordering. Every element is compared through a 64-bit composite
//     (key(value) << 32) | (index << 1) | negzero
// so that a plain unsigned min returns the smallest value and, among equal
// values, the smallest index. For floats key() = fkey(), order preserving
// for the float `<` used by the reference's oracles (src/cpu_methods.h:42-53,
// src/cuda_methods.cuh:23-42): -0.0 and +0.0 map to one key, NaN maps above
// +inf; `negzero` marks -0.0 so its bits come back exactly. The index tables
// store these composites, so every comparison is one unsigned min.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define RMQ_HD __host__ __device__ __forceinline__

namespace rmq {

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

// Key modes: what "best" means for an index. Every mode maps the 32-bit
// element to an unsigned key whose minimum is the best element, so one
// unsigned min over (key << 32 | index) returns the leftmost best.
enum KeyMode : uint32_t {
    kFloatMin = 0,  // float32, range minimum (the reference's semantics)
    kFloatMax = 1,  // float32, range maximum
    kIntMin = 2,    // int32, range minimum
    kIntMax = 3,    // int32, range maximum
};

RMQ_HD uint32_t key_of(uint32_t b, uint32_t mode) {
    switch (mode) {
    case kFloatMax: {
        const uint32_t k = fkey(b);
        return k == 0xffffffffu ? k : ~k;  // NaN stays last
    }
    case kIntMin: return b ^ 0x80000000u;
    case kIntMax: return b ^ 0x7fffffffu;
    default: return fkey(b);
    }
}

// Inverse of key_of; `negzero` restores -0.0 in the float modes.
RMQ_HD uint32_t unkey(uint32_t k, uint32_t negzero, uint32_t mode) {
    switch (mode) {
    case kFloatMax: return k == 0xffffffffu ? 0x7fc00000u : funkey(~k, negzero);
    case kIntMin: return k ^ 0x80000000u;
    case kIntMax: return k ^ 0x7fffffffu;
    default: return funkey(k, negzero);
    }
}

// One structure entry: the composite of its element (file comment). Indices
// are below 2^31, so `index << 1` fits the low word.
using Entry = uint64_t;

// An entry that loses against every real entry.
constexpr Entry kEntryNone = ~0ull;

RMQ_HD uint32_t negzero_of(uint32_t b, uint32_t mode) {
    return ((mode == kFloatMin || mode == kFloatMax) && b == 0x80000000u) ? 1u : 0u;
}

RMQ_HD Entry make_entry(uint32_t b, uint32_t idx, uint32_t mode) {
    return (static_cast<uint64_t>(key_of(b, mode)) << 32) | (idx << 1) | negzero_of(b, mode);
}

RMQ_HD uint32_t entry_idx(Entry e) { return static_cast<uint32_t>(e) >> 1; }

// The element's bits (a NaN comes back as the canonical quiet NaN).
RMQ_HD uint32_t entry_bits(Entry e, uint32_t mode) {
    return unkey(static_cast<uint32_t>(e >> 32), static_cast<uint32_t>(e) & 1u, mode);
}

// Leftmost best of two entries.
RMQ_HD Entry better(Entry a, Entry b) { return b < a ? b : a; }

// Element loads as raw 32-bit words. Elements are never moved through float
// registers: bit operations on a value that came from one (say an XOR of the
// sign bit) may be lowered to float instructions that do not keep NaN
// payloads, and the int32 key modes treat every bit pattern as a value.
#ifdef __CUDACC__
__device__ __forceinline__ uint4 ld_u4(const float *p) {
    return __ldg(reinterpret_cast<const uint4 *>(p));
}
__device__ __forceinline__ uint32_t ld_u1(const float *p) {
    return __ldg(reinterpret_cast<const unsigned int *>(p));
}
#endif

// Checked builds (-DRMQ_CHECKED=1), the engine's stand-in for a memory
// sanitizer: every global index a kernel uses is range-checked first with
// rmq_chk(in_range); a failed check is counted in this translation unit's
// device counter and the access is skipped (no trap, no fault). Normal
// builds compile rmq_chk to `true`.
#ifndef RMQ_CHECKED
#define RMQ_CHECKED 0
#endif
#ifdef __CUDACC__
#if RMQ_CHECKED
static __device__ unsigned long long g_rmq_violations = 0;
__device__ __forceinline__ bool rmq_chk(bool in_range) {
    if (!in_range) atomicAdd(&g_rmq_violations, 1ull);
    return in_range;
}
// host reader of this translation unit's counter
#define RMQ_VIOLATIONS_READER(name)                                                     \
    unsigned long long name() {                                                         \
        unsigned long long v = 0;                                                       \
        if (cudaMemcpyFromSymbol(&v, g_rmq_violations, sizeof(v)) != cudaSuccess) v = ~0ull; \
        return v;                                                                       \
    }
#else
__device__ __forceinline__ bool rmq_chk(bool) { return true; }
#define RMQ_VIOLATIONS_READER(name) \
    unsigned long long name() { return 0; }
#endif
#endif

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
