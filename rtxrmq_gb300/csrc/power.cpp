// power.cpp -- GPU power sampling around a timed region (the CLI's
// --save-power and bench.py's energy figure).
//
// Plays the role of the reference's GPUPowerBegin / GPUPowerEnd
// (common/nvmlPower.cpp:37-84, 91-167): a thread polls
// nvmlDeviceGetPowerUsage every `sample_ms` and writes the same whitespace
// table (#timestep power acc-energy avg-power dt acc-time; W, J, s). NVML is
// loaded at run time (libnvidia-ml.so.1, or the library named by
// RTXRMQ_NVML_LIBRARY), only read from, and shut down at the end; the CUDA
// device is matched to its NVML handle by PCI bus id. Errors are status
// codes; nothing exits (the reference calls exit(0) on NVML errors).
#include <dlfcn.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>
#include <thread>

#include <cuda_runtime.h>

#include "../../include/rmq.h"

namespace {

typedef int (*nvml_init_t)(void);
typedef int (*nvml_shutdown_t)(void);
typedef int (*nvml_by_index_t)(unsigned, void **);
typedef int (*nvml_by_pci_t)(const char *, void **);
typedef int (*nvml_power_t)(void *, unsigned *);

struct Sampler {
    std::mutex mu;
    bool running = false;
    void *lib = nullptr;
    nvml_shutdown_t shutdown = nullptr;
    nvml_power_t power = nullptr;
    void *dev = nullptr;
    std::thread th;
    std::atomic<bool> stop{false};
    FILE *fp = nullptr;
    int sample_ms = 100;
    double energy = 0.0, seconds = 0.0, last_w = 0.0;
};

Sampler g_s;

void poll() {
    using clk = std::chrono::steady_clock;
    auto t1 = clk::now();
    long step = 0;
    while (!g_s.stop.load()) {
        std::this_thread::sleep_for(std::chrono::milliseconds(g_s.sample_ms));
        const auto t2 = clk::now();
        const double dt = std::chrono::duration<double>(t2 - t1).count();
        t1 = t2;
        unsigned mw = 0;
        if (g_s.power(g_s.dev, &mw) != 0) continue;
        const double w = mw / 1000.0;
        ++step;
        g_s.seconds += dt;
        g_s.energy += w * dt;
        g_s.last_w = w;
        if (g_s.fp)
            std::fprintf(g_s.fp, "%-15ld %-15f %-15f %-15f %-15f %-15f\n", step, w, g_s.energy,
                         g_s.energy / g_s.seconds, dt, g_s.seconds);
    }
}

}  // namespace

namespace rmq {
int set_error(int code, const char *fmt, ...);  // api.cu: status + message for rmq_last_error_string
}
using rmq::set_error;

extern "C" {

int rmq_power_begin(int32_t device, int32_t sample_ms, int32_t cooldown_ms, const char *path) {
    std::lock_guard<std::mutex> lock(g_s.mu);
    if (g_s.running) return set_error(RMQ_EINVAL, "rmq_power_begin: a sampling is already running");
    if (sample_ms <= 0 || cooldown_ms < 0)
        return set_error(RMQ_EINVAL, "rmq_power_begin: sample_ms must be > 0 and cooldown_ms >= 0");
    const char *name = std::getenv("RTXRMQ_NVML_LIBRARY");
    void *lib = dlopen(name && *name ? name : "libnvidia-ml.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!lib) return set_error(RMQ_ENOTSUP, "rmq_power_begin: NVML library not found");
    auto init = reinterpret_cast<nvml_init_t>(dlsym(lib, "nvmlInit_v2"));
    auto shut = reinterpret_cast<nvml_shutdown_t>(dlsym(lib, "nvmlShutdown"));
    auto by_idx = reinterpret_cast<nvml_by_index_t>(dlsym(lib, "nvmlDeviceGetHandleByIndex_v2"));
    auto by_pci = reinterpret_cast<nvml_by_pci_t>(dlsym(lib, "nvmlDeviceGetHandleByPciBusId_v2"));
    auto pw = reinterpret_cast<nvml_power_t>(dlsym(lib, "nvmlDeviceGetPowerUsage"));
    if (!init || !shut || !by_idx || !pw || init() != 0) {
        dlclose(lib);
        return set_error(RMQ_ENOTSUP, "rmq_power_begin: NVML symbols missing or initialisation failed");
    }
    void *dev = nullptr;
    char bus[64];
    bool found = false;
    if (by_pci && cudaDeviceGetPCIBusId(bus, sizeof(bus), device) == cudaSuccess)
        found = by_pci(bus, &dev) == 0;
    else
        cudaGetLastError();
    if (!found && by_idx(static_cast<unsigned>(device), &dev) != 0) {
        shut();
        dlclose(lib);
        return set_error(RMQ_ENOTSUP, "rmq_power_begin: no NVML device for CUDA device %d", device);
    }
    FILE *fp = nullptr;
    if (path && *path) {
        fp = std::fopen(path, "w+");
        if (!fp) {
            shut();
            dlclose(lib);
            return set_error(RMQ_EINVAL, "rmq_power_begin: cannot open %s", path);
        }
        std::fprintf(fp, "%-15s %-15s %-15s %-15s %-15s %-15s\n", "#timestep", "power",
                     "acc-energy", "avg-power", "dt", "acc-time");
    }
    g_s.lib = lib;
    g_s.shutdown = shut;
    g_s.power = pw;
    g_s.dev = dev;
    g_s.fp = fp;
    g_s.sample_ms = sample_ms;
    g_s.energy = g_s.seconds = g_s.last_w = 0.0;
    g_s.stop.store(false);
    g_s.th = std::thread(poll);
    g_s.running = true;
    if (cooldown_ms) std::this_thread::sleep_for(std::chrono::milliseconds(cooldown_ms));
    return RMQ_OK;
}

int rmq_power_end(int32_t cooldown_ms, double *avg_watts, double *energy_joules,
                  double *seconds) {
    {
        std::lock_guard<std::mutex> lock(g_s.mu);
        if (!g_s.running) return set_error(RMQ_EINVAL, "rmq_power_end: no sampling is running");
    }
    if (cooldown_ms > 0) std::this_thread::sleep_for(std::chrono::milliseconds(cooldown_ms));
    std::lock_guard<std::mutex> lock(g_s.mu);
    // another caller may have ended the sampling during the cool-down
    if (!g_s.running) return set_error(RMQ_EINVAL, "rmq_power_end: no sampling is running");
    g_s.stop.store(true);
    g_s.th.join();
    if (g_s.fp) std::fclose(g_s.fp);
    g_s.fp = nullptr;
    g_s.shutdown();
    dlclose(g_s.lib);
    g_s.lib = nullptr;
    g_s.running = false;
    if (avg_watts) *avg_watts = g_s.seconds > 0 ? g_s.energy / g_s.seconds : 0.0;
    if (energy_joules) *energy_joules = g_s.energy;
    if (seconds) *seconds = g_s.seconds;
    return RMQ_OK;
}

}  // extern "C"
