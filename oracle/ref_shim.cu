// ref_shim.cu -- TEST INFRASTRUCTURE. Compiles the reference's own CPU RMQ
// code (src/cpu_methods.h: cpu_rmq, cpu_rmq_idx, rmq_rmm_par,
// rmq_rmm_par_idx; src/rand.cuh: random_queries_par_cpu) unmodified, from
// the reference tree, into oracle/_ref/libref.so, and exposes it through a
// C ABI for the golden-vector generator and the oracle pin tests.
//
// The reference headers expect definitions that live in files this shim
// must not include (src/main.cu, common/common.h pulls in optix.h,
// common/nvmlPower.cpp needs NVML): they are supplied here. CUDA 13 removed
// cudaDeviceProp::memoryClockRate, which src/tools.h:263-265 prints; it is
// mapped onto another int field so the header compiles (never called).
#include <cstdio>
#include <cstring>
#include <string>

#define BSIZE 1024
#define WARPSIZE 32
#define ALG_CPU_BASE 0
#define ALG_CPU_HRMQ 1
#define ALG_GPU_BASE 2
#define ALG_GPU_RTX_CAST 3
#define ALG_GPU_RTX_TRANS 4
#define ALG_GPU_RTX_BLOCKS 5
#define ALG_GPU_RTX_LUP 6
#define ALG_GPU_RTX_IAS 8
#define ALG_GPU_RTX_IAS_TRANS 9
#define ALG_GPU_RTX_SER 10
#define ALG_CPU_BASE_IDX 100
#define ALG_CPU_HRMQ_IDX 101
#define ALG_GPU_BASE_IDX 102
#define ALG_GPU_RTX_CAST_IDX 103
#define ALG_GPU_RTX_BLOCKS_IDX 105

#define AC_RESET ""
#define AC_GREEN ""
#define AC_BOLDGREEN ""
#define AC_BOLDCYAN ""
#define AC_YELLOW ""

static const char *algStr[11] = {"[CPU] BASE", "[CPU] HRMQ", "[GPU] BASE", "", "", "", "", "", "", "", ""};

static void GPUPowerBegin(const char *, int, int, std::string) {}
static void GPUPowerEnd() {}
static void CPUPowerBegin(const char *, int, std::string) {}
static void CPUPowerEnd() {}

#define memoryClockRate memoryBusWidth

#include "common/Timer.h"
#include "src/rand.cuh"
#include "src/tools.h"
#include "src/cpu_methods.h"

static CmdArgs quiet_args(int alg, int nt) {
    CmdArgs a;
    a.n = a.q = a.lr = 0;
    a.alg = alg;
    a.bs = a.nb = 0;
    a.reps = 1;
    a.dev = 0;
    a.nt = nt;
    a.seed = 0;
    a.check = 0;
    a.save_time = 0;
    a.save_power = 0;
    return a;
}

extern "C" {

// random_queries_par_cpu (src/rand.cuh:179-201) into out[2*q]
int ref_random_queries(int q, int lr, int n, int nt, int seed, int *out) {
    int2 *Q = random_queries_par_cpu(q, lr, n, nt, seed);
    for (int i = 0; i < q; ++i) {
        out[2 * i] = Q[i].x;
        out[2 * i + 1] = Q[i].y;
    }
    delete[] Q;
    return 0;
}

// cpu_rmq<float> (src/cpu_methods.h:18-40)
int ref_cpu_rmq(int n, int q, const float *A, const int *Qflat, int nt, float *out) {
    float *Ac = const_cast<float *>(A);
    int2 *Q = reinterpret_cast<int2 *>(const_cast<int *>(Qflat));
    float *r = cpu_rmq<float>(n, q, Ac, Q, nt, quiet_args(ALG_CPU_BASE, nt));
    std::memcpy(out, r, sizeof(float) * q);
    delete[] r;
    return 0;
}

// cpu_rmq_idx<float> (src/cpu_methods.h:56-77)
int ref_cpu_rmq_idx(int n, int q, const float *A, const int *Qflat, int nt, int *out) {
    float *Ac = const_cast<float *>(A);
    int2 *Q = reinterpret_cast<int2 *>(const_cast<int *>(Qflat));
    int *r = cpu_rmq_idx<float>(n, q, Ac, Q, nt, quiet_args(ALG_CPU_BASE_IDX, nt));
    std::memcpy(out, r, sizeof(int) * q);
    delete[] r;
    return 0;
}

// rmq_rmm_par (src/cpu_methods.h:80-119): HRMQ, values; A reinterpreted as
// int exactly as src/main.cu:118 does.
int ref_rmq_rmm_par(int n, int q, const float *A, const int *Qflat, int nt, float *out) {
    int *Ai = reinterpret_cast<int *>(const_cast<float *>(A));
    int2 *Q = reinterpret_cast<int2 *>(const_cast<int *>(Qflat));
    int *r = rmq_rmm_par(n, q, Ai, Q, nt, quiet_args(ALG_CPU_HRMQ, nt));
    std::memcpy(out, r, sizeof(int) * q);
    delete[] r;
    return 0;
}

// rmq_rmm_par_idx (src/cpu_methods.h:121-159): HRMQ, indices (rightmost on
// ties, from the >= pop of hrmq/RMQRMM64.cpp:211).
int ref_rmq_rmm_par_idx(int n, int q, const float *A, const int *Qflat, int nt, int *out) {
    int *Ai = reinterpret_cast<int *>(const_cast<float *>(A));
    int2 *Q = reinterpret_cast<int2 *>(const_cast<int *>(Qflat));
    int *r = rmq_rmm_par_idx(n, q, Ai, Q, nt, quiet_args(ALG_CPU_HRMQ_IDX, nt));
    std::memcpy(out, r, sizeof(int) * q);
    delete[] r;
    return 0;
}

}  // extern "C"
