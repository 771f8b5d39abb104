// cli.cpp -- `rtxrmq <n> <q> <lr> <alg> [options]`, the reference's command
// line (README.md:17-49, src/main.cu:51-171, src/tools.h:76-189) over the C
// ABI of include/rmq.h.
//
// Algorithms served here: 5 / 105 (the block-decomposition engine; values /
// indices) and 2 / 102 (GPU brute force). The CPU algorithms 0/1/100/101 and
// the other ray-tracing variants 3,4,6,8,9,10,103 are not part of this
// engine; asking for them prints a message and exits with status 2.
//
// Timing follows src/rtx.h:150-162: a host stopwatch around `reps` launches,
// each followed by a stream synchronize; construction is timed on its own.
// --save-time appends the reference's CSV row
//   dev,alg,reps,n,bs,q,lr,t,q/s,ns/q,construction,outbuffer,tempbuffer
// (src/tools.h:268-336; header line of scripts/perf-benchmark.sh:30).
#include <getopt.h>
#include <unistd.h>

#include <chrono>
#include <cctype>
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include <cuda_runtime.h>
#include <omp.h>

#include "../../include/rmq.h"

namespace {

const char *kAlgStr[11] = {"[CPU] BASE",      "[CPU] HRMQ",        "[GPU] BASE",
                           "[GPU] RTX_cast",  "[GPU] RTX_trans",   "[GPU] RTX_blocks",
                           "[GPU] RTX_lup",   "[GPU] LCA (TODO)",  "[GPU] RTX_ias",
                           "[GPU] RTX_ias_trans", "[GPU] RTX_ser"};

struct Args {
    long long n = 0, q = 0;
    int lr = 0, alg = 0;
    long long bs = 1 << 15, nb = 0;
    int reps = 10, dev = 0, nt = 1, check = 0, save_time = 0, save_power = 0;
    long long seed = 0;
    std::string time_file, power_file;
};

void usage() {
    std::fprintf(stderr,
                 "usage: rtxrmq <n> <q> <lr> <alg> [options]\n"
                 "\n"
                 "Builds a range-minimum index over n random float32 values and answers q\n"
                 "random inclusive queries (l, r) on the GPU, timing the query launches.\n"
                 "\n"
                 "positional arguments\n"
                 "  n     array length (1 .. 2^31-1)\n"
                 "  q     number of queries\n"
                 "  lr    query length: a positive value fixes every length (at most n);\n"
                 "        -1 draws lengths uniformly from [1, n], -2 / -3 from lognormal\n"
                 "        distributions centred near n^0.6 / n^0.3, -4 / -5 near n/2^8 and\n"
                 "        n/2^15\n"
                 "  alg   5 = block decomposition (%s), returning minimum values\n"
                 "        2 = brute force on the GPU (%s), returning minimum values\n"
                 "        105, 102 = the same two, returning leftmost argmin indices\n"
                 "        (every other id of the original tool exits with status 2 here)\n"
                 "\n"
                 "options\n"
                 "  --bs <k>            elements per block for alg 5 (default 32768)\n"
                 "  --nb <k>            number of blocks instead; block size = n / k\n"
                 "  --reps <k>          timed repetitions of the query launch (default 10)\n"
                 "  --dev <id>          CUDA device (default 0)\n"
                 "  --nt <k>            host threads for generating the queries\n"
                 "  --seed <s>          generator seed (default: the current time)\n"
                 "  --check             compare every answer with the brute force\n"
                 "  --save-time=<file>  append one CSV row of timings\n"
                 "  --save-power=<file> record board power (NVML) over the timed loop\n",
                 kAlgStr[5], kAlgStr[2]);
}

const char *alg_name(int alg) { return kAlgStr[alg % 100 <= 10 ? alg % 100 : 0]; }

enum { ARG_BS = 1, ARG_NB, ARG_REPS, ARG_DEV, ARG_NT, ARG_SEED, ARG_CHECK, ARG_TIME, ARG_POWER };

// src/tools.h:76-189 semantics (including --bs/--nb integer division and
// bs = 0 for algorithms without blocks).
bool parse(int argc, char **argv, Args &a) {
    if (argc < 5) return false;
    a.n = std::atoll(argv[1]);
    a.q = std::atoll(argv[2]);
    a.lr = std::atoi(argv[3]);
    a.alg = std::atoi(argv[4]);
    if (!a.n || !a.q || !a.lr) return false;
    if (a.n < 0 || a.n > 0x7fffffffLL || a.q < 0) {
        std::fprintf(stderr, "Error: n must be in [1, 2^31-1] and q >= 1\n");
        std::exit(EXIT_FAILURE);
    }
    if (a.lr > a.n) {
        std::fprintf(stderr, "Error: lr=%i > n=%lld  (lr must be between '1' and 'n')\n", a.lr, a.n);
        std::exit(EXIT_FAILURE);
    }
    a.bs = 1 << 15;
    if (a.bs > a.n) a.bs = a.n;
    a.nb = a.n / a.bs;
    a.seed = static_cast<long long>(std::time(nullptr));
    static struct option opts[] = {
        {"bs", required_argument, 0, ARG_BS},     {"nb", required_argument, 0, ARG_NB},
        {"reps", required_argument, 0, ARG_REPS}, {"dev", required_argument, 0, ARG_DEV},
        {"nt", required_argument, 0, ARG_NT},     {"seed", required_argument, 0, ARG_SEED},
        {"check", no_argument, 0, ARG_CHECK},     {"save-time", optional_argument, 0, ARG_TIME},
        {"save-power", optional_argument, 0, ARG_POWER}, {0, 0, 0, 0}};
    int opt, idx;
    optind = 5;
    while ((opt = getopt_long(argc, argv, "", opts, &idx)) != -1) {
        switch (opt) {
        case ARG_BS: {
            long long v = std::atoll(optarg);
            if (v < 1) v = 1;
            a.bs = v < a.n ? v : a.n;
            a.nb = a.n / a.bs;
            break;
        }
        case ARG_NB: {
            long long v = std::atoll(optarg);
            if (v < 1) v = 1;
            a.nb = v < a.n ? v : a.n;
            a.bs = a.n / a.nb;
            break;
        }
        case ARG_REPS: a.reps = std::atoi(optarg); break;
        case ARG_DEV: a.dev = std::atoi(optarg); break;
        case ARG_NT: a.nt = std::atoi(optarg); break;
        case ARG_SEED: a.seed = std::atoll(optarg); break;
        case ARG_CHECK: a.check = 1; break;
        case ARG_TIME:
            a.save_time = 1;
            if (optarg) a.time_file = optarg;
            break;
        case ARG_POWER:
            a.save_power = 1;
            if (optarg) a.power_file = optarg;
            break;
        default: return false;
        }
    }
    if (a.reps < 1) a.reps = 1;
    if (a.alg % 100 != 5) {
        a.bs = 0;
        a.nb = 0;
    }
    return true;
}

#define CK(call)                                                                        \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            std::fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_),    \
                         __FILE__, __LINE__);                                           \
            std::exit(EXIT_FAILURE);                                                    \
        }                                                                               \
    } while (0)

#define RK(call)                                                                        \
    do {                                                                                \
        int r_ = (call);                                                                \
        if (r_ != RMQ_OK) {                                                             \
            std::fprintf(stderr, "rmq error %d: %s\n", r_, rmq_last_error_string());    \
            std::exit(EXIT_FAILURE);                                                    \
        }                                                                               \
    } while (0)

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void csv_prefix(const Args &a, const char *device) {
    if (!a.save_time) return;
    const std::string f = a.time_file.empty() ? "../results/data.csv" : a.time_file;
    FILE *fp = std::fopen(f.c_str(), "a");
    if (!fp) return;
    std::fprintf(fp, "%s,%s,%i,%lld,%lld,%lld,%i", device, alg_name(a.alg), a.reps, a.n, a.bs, a.q,
                 a.lr);
    std::fclose(fp);
}

void csv_suffix(const Args &a, double time_ms, double construction_ms, double out_mb, double tmp_mb) {
    if (!a.save_time) return;
    const std::string f = a.time_file.empty() ? "../results/data.csv" : a.time_file;
    FILE *fp = std::fopen(f.c_str(), "a");
    if (!fp) return;
    const double it = time_ms / a.reps;
    std::fprintf(fp, ",%f,%f,%f,%f,%f,%f\n", time_ms / 1000.0,
                 static_cast<double>(a.q) / (it / 1000.0), it * 1e6 / static_cast<double>(a.q),
                 construction_ms, out_mb, tmp_mb);
    std::fclose(fp);
}

}  // namespace

int main(int argc, char **argv) {
    std::printf("----------------------------------\n");
    std::printf("   RTX-RMQ (GB300 CUDA engine)    \n");
    std::printf("----------------------------------\n");
    Args a;
    if (!parse(argc, argv, a)) {
        usage();
        return EXIT_FAILURE;
    }
    const int base_alg = a.alg % 100;
    const bool idx_mode = a.alg >= 100;
    if (!((base_alg == 2 || base_alg == 5) && (a.alg < 100 || a.alg == 102 || a.alg == 105))) {
        std::fprintf(stderr,
                     "alg %d is not available in this engine (served: 2, 5, 102, 105; CPU "
                     "algorithms and the other ray-tracing variants are out of scope)\n",
                     a.alg);
        return 2;
    }

    CK(cudaSetDevice(a.dev));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, a.dev));
    std::printf("Params:\n   reps = %i\n   seed = %lld\n   dev  = %i (%s, %d SMs)\n"
                "   n    = %lld (~%f GB, float)\n   bs   = %lld\n   q    = %lld (~%f GB, int2)\n"
                "   lr   = %i\n   nt   = %i CPU threads\n   alg  = %i (%s)\n\n",
                a.reps, a.seed, a.dev, prop.name, prop.multiProcessorCount, a.n,
                sizeof(float) * a.n / 1e9, a.bs, a.q, sizeof(int) * 2 * a.q / 1e9, a.lr, a.nt,
                a.alg, alg_name(a.alg));
    if (a.nt > 0) omp_set_num_threads(a.nt);  // generators in librmq.so share this runtime

    // 1) data and queries
    auto t0 = std::chrono::steady_clock::now();
    std::vector<float> hA(static_cast<size_t>(a.n));
    RK(rmq_gen_values_uniform(hA.data(), a.n, static_cast<uint64_t>(a.seed)));
    float *dA = nullptr;
    CK(cudaMalloc(&dA, sizeof(float) * a.n));
    CK(cudaMemcpy(dA, hA.data(), sizeof(float) * a.n, cudaMemcpyHostToDevice));
    std::printf("Generating n=%-10lld values............done: %f secs\n", a.n, ms_since(t0) / 1e3);
    t0 = std::chrono::steady_clock::now();
    std::vector<int32_t> hQ(static_cast<size_t>(2 * a.q));
    RK(rmq_gen_queries(hQ.data(), a.q, a.n, a.lr, static_cast<uint64_t>(a.seed) + 7));
    int32_t *dQ = nullptr;
    CK(cudaMalloc(&dQ, sizeof(int32_t) * 2 * a.q));
    CK(cudaMemcpy(dQ, hQ.data(), sizeof(int32_t) * 2 * a.q, cudaMemcpyHostToDevice));
    std::printf("Generating q=%-10lld queries...........done: %f secs\n", a.q, ms_since(t0) / 1e3);

    csv_prefix(a, prop.name);

    float *dV = nullptr;
    int32_t *dI = nullptr;
    if (idx_mode)
        CK(cudaMalloc(&dI, sizeof(int32_t) * a.q));
    else
        CK(cudaMalloc(&dV, sizeof(float) * a.q));

    // 2) computation
    double construction = 0.0, out_mb = 0.0;
    rmq_handle_t *h = nullptr;
    if (base_alg == 5) {
        t0 = std::chrono::steady_clock::now();
        RK(rmq_build(dA, a.n, a.bs, nullptr, &h));
        CK(cudaDeviceSynchronize());
        construction = ms_since(t0);
        rmq_info_t info;
        RK(rmq_info(h, &info));
        out_mb = info.struct_bytes / 1e6;
        std::printf("Building index (bs=%lld, nb=%lld)........done: %f ms [structure %f MB]\n",
                    static_cast<long long>(info.bs), static_cast<long long>(info.nb), construction,
                    out_mb);
    }
    std::printf("Computing RMQs%s (%-16s,r=%-3i)...", idx_mode ? " index" : "", alg_name(a.alg),
                a.reps);
    std::fflush(stdout);
    bool sampling = false;
    if (a.save_power) {
        // src/rtx.h:148-158: 100 ms samples around the timed loop, the
        // reference's file name when none is given
        const std::string f = a.power_file.empty()
                                  ? std::string("../results/power-") + alg_name(a.alg) + ".dat"
                                  : a.power_file;
        const int prc = rmq_power_begin(a.dev, 100, 1000, f.c_str());
        if (prc == RMQ_OK)
            sampling = true;
        else
            std::fprintf(stderr, "warning: power sampling unavailable (status %d); continuing\n", prc);
    }
    t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < a.reps; ++i) {
        if (base_alg == 5)
            RK(rmq_query(h, dQ, a.q, dV, dI, nullptr));
        else
            RK(rmq_query_scan(dA, a.n, dQ, a.q, dV, dI, nullptr));
        CK(cudaDeviceSynchronize());
    }
    const double timems = ms_since(t0);
    if (sampling) {
        double watts = 0, joules = 0, secs = 0;
        if (rmq_power_end(1000, &watts, &joules, &secs) == RMQ_OK)
            std::printf("power: %.2f W average, %.2f J over %.2f s sampled [%.3e RMQs/J]\n", watts,
                        joules, secs,
                        joules > 0 ? static_cast<double>(a.q) * a.reps / joules : 0.0);
    }
    const double avg = timems / (1000.0 * a.reps);
    std::printf("done: %f secs (avg %f secs): [%.2f RMQs/sec, %f nsec/RMQ]\n", timems / 1000.0, avg,
                static_cast<double>(a.q) / avg, avg * 1e9 / static_cast<double>(a.q));
    csv_suffix(a, timems, construction, out_mb, 0.0);

    int rc = 0;
    if (a.check) {
        // src/main.cu:140-167: compare against GPU BASE on the same inputs
        std::printf("\nCHECKING RESULT:\n");
        float *eV = nullptr;
        int32_t *eI = nullptr;
        if (idx_mode)
            CK(cudaMalloc(&eI, sizeof(int32_t) * a.q));
        else
            CK(cudaMalloc(&eV, sizeof(float) * a.q));
        RK(rmq_query_scan(dA, a.n, dQ, a.q, eV, eI, nullptr));
        CK(cudaDeviceSynchronize());
        std::vector<uint32_t> got(static_cast<size_t>(a.q)), exp(static_cast<size_t>(a.q));
        CK(cudaMemcpy(got.data(), idx_mode ? static_cast<void *>(dI) : static_cast<void *>(dV),
                      4 * a.q, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(exp.data(), idx_mode ? static_cast<void *>(eI) : static_cast<void *>(eV),
                      4 * a.q, cudaMemcpyDeviceToHost));
        long long bad = 0;
        for (long long i = 0; i < a.q; ++i) {
            if (got[i] != exp[i]) {
                if (bad < 10) {
                    if (idx_mode)
                        std::printf("Error on %lld-th query: got %d, expected %d  [%d,%d]\n", i,
                                    static_cast<int>(got[i]), static_cast<int>(exp[i]), hQ[2 * i],
                                    hQ[2 * i + 1]);
                    else {
                        float g, e;
                        std::memcpy(&g, &got[i], 4);
                        std::memcpy(&e, &exp[i], 4);
                        std::printf("Error on %lld-th query: got %.9g, expected %.9g  [%d,%d]\n", i,
                                    g, e, hQ[2 * i], hQ[2 * i + 1]);
                    }
                }
                ++bad;
            }
        }
        std::printf("Checking result (bit-exact)...............%s (%lld mismatches)\n",
                    bad ? "failed" : "pass", bad);
        rc = bad ? 1 : 0;
        cudaFree(eV);
        cudaFree(eI);
    }
    rmq_free(h);
    cudaFree(dA);
    cudaFree(dQ);
    cudaFree(dV);
    cudaFree(dI);
    std::printf("Benchmark Finished\n");
    return rc;
}
