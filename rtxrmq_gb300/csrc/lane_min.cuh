// lane_min.cuh -- the best of one lane's four consecutive values, as a key
// (common.cuh) and a position, for the micro-block minima of the light
// index. Host and device code, so that the host tests run it against the
// definition (the smallest key, leftmost among equal keys).
#pragma once

#include <cmath>
#include <cstring>

#include "common.cuh"

namespace rmq {

RMQ_HD float float_of_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, sizeof(f));
    return f;
#endif
}

RMQ_HD uint32_t bits_of_float(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t b;
    std::memcpy(&b, &f, sizeof(b));
    return b;
#endif
}

// The IEEE minimum / maximum that skips any NaN operand: CUDA's fminf /
// fmaxf on the device (a NaN operand, quiet or signaling, gives the other
// operand). On the host the C library's fminf returns NaN for a signaling
// NaN operand, so the host spells the device semantics out.
RMQ_HD float min_num(float a, float b) {
#ifdef __CUDA_ARCH__
    return fminf(a, b);
#else
    return a != a ? b : b != b ? a : (b < a ? b : a);
#endif
}
RMQ_HD float max_num(float a, float b) {
#ifdef __CUDA_ARCH__
    return fmaxf(a, b);
#else
    return a != a ? b : b != b ? a : (b > a ? b : a);
#endif
}

// The lane's best of b[0 .. nvalid) (the rest lie past the array's end) in
// key mode MODE: its key, and its position | (-0.0 flag << 2). With no
// valid value: the largest key, position 0.
//
// Float modes: the IEEE minimum (maximum) skips NaN, quiet or signaling,
// which is last in the key order, unless every value is NaN; the first value
// equal to it (+0 == -0, so the leftmost zero) is the leftmost best, and its
// bits give the key and the -0.0 flag; values past the end enter as NaN and
// lie to the right of every valid one. With every value NaN, element 0.
// Integer modes: the keys themselves, strict < in index order.
template <uint32_t MODE>
RMQ_HD void lane_best4(const uint32_t (&b)[4], uint32_t nvalid, uint32_t &key, uint32_t &info) {
    if constexpr (MODE == kFloatMin || MODE == kFloatMax) {
        float f[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            f[k] = float_of_bits(static_cast<uint32_t>(k) < nvalid ? b[k] : 0x7fc00000u);
        const float m = MODE == kFloatMin ? min_num(min_num(f[0], f[1]), min_num(f[2], f[3]))
                                          : max_num(max_num(f[0], f[1]), max_num(f[2], f[3]));
        const uint32_t pos = f[0] == m ? 0u : f[1] == m ? 1u : f[2] == m ? 2u : f[3] == m ? 3u : 0u;
        const uint32_t wb = bits_of_float(pos == 0u ? f[0] : pos == 1u ? f[1] : pos == 2u ? f[2] : f[3]);
        key = key_of(wb, MODE);
        info = pos | (negzero_of(wb, MODE) << 2);
    } else {
        key = 0u < nvalid ? key_of(b[0], MODE) : 0xffffffffu;
        info = negzero_of(b[0], MODE) << 2;
#pragma unroll
        for (int k = 1; k < 4; ++k) {
            const uint32_t kk = static_cast<uint32_t>(k) < nvalid ? key_of(b[k], MODE) : 0xffffffffu;
            if (kk < key) {
                key = kk;
                info = static_cast<uint32_t>(k) | (negzero_of(b[k], MODE) << 2);
            }
        }
    }
}

}  // namespace rmq
