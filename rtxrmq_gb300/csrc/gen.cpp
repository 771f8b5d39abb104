// gen.cpp -- synthetic inputs on the host (values and (l, r) queries).
//
// Plays the role of the reference's generators (src/rand.cuh): uniform
// values (create_random_array_dev, rand.cuh:23-43) and queries with the
// length modes of random_queries_par_cpu (rand.cuh:179-201). Unlike the
// reference, each element / query draws from its own counter-based stream
// (splitmix64 of seed and position), so the output is the same for any
// OpenMP thread count; the reference seeds thread t with mt19937(seed*t)
// (rand.cuh:120, 140, 160), so its output changes with --nt.
// Lognormal lengths are rounded to nearest and clamped to [1, n]; the
// reference truncates and redraws outside [1, n] (rand.cuh:161-169).
#include <cmath>
#include <cstdint>
#include <omp.h>

#include "../../include/rmq.h"

namespace {

inline uint64_t splitmix_next(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline uint64_t stream_for(uint64_t seed, uint64_t i) {
    uint64_t s = seed * 0xD1B54A32D192ED03ull + i * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    splitmix_next(s);
    return s;
}

// uniform in (0, 1] with 53-bit resolution
inline double u01_open0(uint64_t &s) {
    return (static_cast<double>(splitmix_next(s) >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

// uniform integer in [0, m), m <= 2^32 (multiply-shift; bias <= m / 2^32)
inline uint64_t uniform_below(uint64_t &s, uint64_t m) {
    return ((splitmix_next(s) >> 32) * m) >> 32;
}

inline double std_normal(uint64_t &s) {
    const double u1 = u01_open0(s);
    const double u2 = u01_open0(s);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

void fill_queries(int32_t *out, int64_t q, int64_t n, int fixed_len, double mu, double sigma,
                  bool uniform_len, uint64_t seed) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < q; ++i) {
        uint64_t s = stream_for(seed, static_cast<uint64_t>(i));
        int64_t len;
        if (fixed_len > 0) {
            len = fixed_len;
        } else if (uniform_len) {
            len = 1 + static_cast<int64_t>(uniform_below(s, static_cast<uint64_t>(n)));
        } else {
            const double x = std::exp(mu + sigma * std_normal(s));
            len = (x >= 9.0e18) ? n : std::llround(x);
            if (len < 1) len = 1;
            if (len > n) len = n;
        }
        const int64_t l = static_cast<int64_t>(uniform_below(s, static_cast<uint64_t>(n - len + 1)));
        out[2 * i] = static_cast<int32_t>(l);
        out[2 * i + 1] = static_cast<int32_t>(l + len - 1);
    }
}

}  // namespace

namespace rmq {
int set_error(int code, const char *fmt, ...);  // api.cu: status + message for rmq_last_error_string
}
using rmq::set_error;

extern "C" {

int rmq_gen_values_uniform(float *h_out, int64_t n, uint64_t seed) {
    if (!h_out || n < 0) return set_error(RMQ_EINVAL, "rmq_gen_values_uniform: NULL output or n < 0");
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t s = stream_for(seed, static_cast<uint64_t>(i));
        h_out[i] = static_cast<float>(splitmix_next(s) >> 40) * (1.0f / 16777216.0f);
    }
    return RMQ_OK;
}

int rmq_gen_values_normal(float *h_out, int64_t n, double mean, double stddev, uint64_t seed) {
    if (!h_out || n < 0) return set_error(RMQ_EINVAL, "rmq_gen_values_normal: NULL output or n < 0");
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t s = stream_for(seed, static_cast<uint64_t>(i));
        h_out[i] = static_cast<float>(mean + stddev * std_normal(s));
    }
    return RMQ_OK;
}

int rmq_gen_values_int(float *h_out, int64_t n, int32_t range, uint64_t seed) {
    if (!h_out || n < 0 || range <= 0)
        return set_error(RMQ_EINVAL, "rmq_gen_values_int: NULL output, n < 0 or range <= 0");
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        uint64_t s = stream_for(seed, static_cast<uint64_t>(i));
        h_out[i] = static_cast<float>(uniform_below(s, static_cast<uint64_t>(range)));
    }
    return RMQ_OK;
}

int rmq_gen_queries(int32_t *h_out, int64_t q, int64_t n, int32_t lr, uint64_t seed) {
    if (!h_out || q < 0 || n <= 0 || n > 0x7fffffffLL)
        return set_error(RMQ_EINVAL, "rmq_gen_queries: NULL output, q < 0 or n outside [1, 2^31-1]");
    if (lr > 0) {
        if (lr > n)
            return set_error(RMQ_EINVAL, "rmq_gen_queries: fixed length lr=%d exceeds n=%lld", lr,
                             static_cast<long long>(n));
        fill_queries(h_out, q, n, lr, 0.0, 0.0, false, seed);
        return RMQ_OK;
    }
    const double dn = static_cast<double>(n);
    switch (lr) {
    case -1: fill_queries(h_out, q, n, 0, 0.0, 0.0, true, seed); return RMQ_OK;
    case -2: fill_queries(h_out, q, n, 0, 0.6 * std::log(dn), 0.3, false, seed); return RMQ_OK;
    case -3: fill_queries(h_out, q, n, 0, 0.3 * std::log(dn), 0.3, false, seed); return RMQ_OK;
    case -4: {
        const double sc = dn / 256.0 < 1.0 ? 1.0 : std::floor(dn / 256.0);
        fill_queries(h_out, q, n, 0, std::log(sc), 0.3, false, seed);
        return RMQ_OK;
    }
    case -5: {
        const double sc = dn / 32768.0 < 1.0 ? 1.0 : std::floor(dn / 32768.0);
        fill_queries(h_out, q, n, 0, std::log(sc), 0.3, false, seed);
        return RMQ_OK;
    }
    default: return set_error(RMQ_EINVAL, "rmq_gen_queries: lr=%d is not a length mode (> 0, -1 .. -5)", lr);
    }
}

int rmq_gen_queries_lognormal(int32_t *h_out, int64_t q, int64_t n, double mu, double sigma,
                              uint64_t seed) {
    if (!h_out || q < 0 || n <= 0 || n > 0x7fffffffLL || !(sigma >= 0.0))
        return set_error(RMQ_EINVAL, "rmq_gen_queries_lognormal: bad arguments (q, n or sigma)");
    fill_queries(h_out, q, n, 0, mu, sigma, false, seed);
    return RMQ_OK;
}

}  // extern "C"
