// persist.cu -- saving a built index to a file and loading it back.
//
// The role of HRMQ's saveDS / loadDS (hrmq/RMQRMM64.cpp:1471-1659), which
// write the structure's scalars and tables so it can be reused without a
// rebuild. Here the file is a fixed header followed by the handle's single
// device allocation (prefix/suffix minima, sparse tables, sub-block level).
// The values are not stored (the index refers to the caller's array); the
// header holds a 64-bit fingerprint of all values, computed on the GPU, and
// rmq_load refuses an array whose fingerprint, length or layout differs.
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/rmq.h"
#include "engine.h"

namespace rmq {
namespace {

constexpr char kMagic[16] = "RTXRMQ-GB300-IX";
// 2: entries are comparison composites; 3: sub-block level for every
// bs >= 64; 4: micro-table levels 1.. stored as offsets; 5: micro table
// deep enough for every micro-block a block touches, light indexes
constexpr uint32_t kVersion = 5;
constexpr size_t kIoChunk = size_t(64) << 20;

struct FileHeader {
    char magic[16];
    uint32_t version;
    uint32_t flags;          // rmq_build_ex flags the index was built with
    uint64_t n, bs, nb, levels, nmicro, mlevels;
    uint64_t bytes;          // size of the device allocation that follows
    uint64_t values_print;   // fingerprint of A[0..n)
    uint64_t header_check;   // hash of the fields above
};

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// XOR over i of mix64((i << 32) | bits(A[i])): order independent, changes
// with any value or position. Groups of 4 elements per 16-byte load when A
// is 16-byte aligned, several groups in flight per thread.
__global__ void fingerprint_kernel(const float *__restrict__ A, uint32_t n,
                                   unsigned long long *out) {
    uint64_t acc = 0;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t done = 0;  // elements covered by 16-byte groups
    if (reinterpret_cast<uintptr_t>(A) % 16 == 0) {
        const uint32_t groups = n / 4;
#pragma unroll 4
        for (uint32_t gi = tid; gi < groups; gi += nthreads) {
            const uint4 f = ld_u4(A + 4 * gi);
            const uint64_t i = 4ull * gi;
            acc ^= mix64((i << 32) | f.x) ^ mix64(((i + 1) << 32) | f.y) ^
                   mix64(((i + 2) << 32) | f.z) ^ mix64(((i + 3) << 32) | f.w);
        }
        done = groups * 4;
    }
    for (uint32_t i = done + tid; i < n; i += nthreads)
        acc ^= mix64((static_cast<uint64_t>(i) << 32) | ld_u1(A + i));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc ^= __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicXor(out, static_cast<unsigned long long>(acc));
}

int fingerprint(const float *A, uint32_t n, cudaStream_t s, uint64_t *out) {
    unsigned long long *d = nullptr;
    cudaError_t err = dev_malloc(reinterpret_cast<void **>(&d), sizeof(*d));
    if (err != cudaSuccess) return cuda_fail(err, "fingerprint: cudaMalloc");
    DeviceInfo dev;
    int rc = device_info(&dev);
    if (rc) {
        cudaFree(d);
        return rc;
    }
    err = cudaMemsetAsync(d, 0, sizeof(*d), s);
    if (err == cudaSuccess) {
        fingerprint_kernel<<<dev.sms * 4, 256, 0, s>>>(A, n, d);
        err = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (err == cudaSuccess) err = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    cudaFree(d);
    if (err != cudaSuccess) return cuda_fail(err, "fingerprint");
    *out = h;
    return RMQ_OK;
}

uint64_t header_hash(const FileHeader &h) {
    const unsigned char *p = reinterpret_cast<const unsigned char *>(&h);
    uint64_t x = 0;
    for (size_t i = 0; i < offsetof(FileHeader, header_check); ++i) x = mix64(x ^ p[i]);
    return x;
}

}  // namespace
RMQ_VIOLATIONS_READER(violations_persist)

}  // namespace rmq

using namespace rmq;

extern "C" {

int rmq_save(const rmq_handle_t *h, const char *path, rmq_stream_t stream) {
    NvtxRange nvtx_range("rmq_save");
    if (!h || !path) return set_error(RMQ_EINVAL, "rmq_save: NULL argument");
    BuildPlan p;
    void *mem = nullptr;
    size_t bytes = 0;
    int rc = handle_view(h, &p, &mem, &bytes);
    if (rc) return rc;
    FileHeader hd;
    std::memset(&hd, 0, sizeof(hd));
    std::memcpy(hd.magic, kMagic, sizeof(kMagic));
    hd.version = kVersion;
    hd.flags = (p.micro ? 0u : RMQ_BUILD_NO_MICRO) | ((p.kmode & 1u) ? RMQ_BUILD_MAX : 0u) |
               (p.kmode >= kIntMin ? RMQ_BUILD_INT32 : 0u) | (p.light ? RMQ_BUILD_LIGHT : 0u);
    hd.n = p.n;
    hd.bs = p.bs;
    hd.nb = p.nb;
    hd.levels = p.levels;
    hd.nmicro = p.nmicro;
    hd.mlevels = p.mlevels;
    hd.bytes = bytes;
    rc = fingerprint(p.A, p.n, stream, &hd.values_print);
    if (rc) return rc;
    hd.header_check = header_hash(hd);
    FILE *fp = std::fopen(path, "wb");
    if (!fp) return set_error(RMQ_EINVAL, "rmq_save: cannot open %s for writing", path);
    std::vector<char> buf;
    try {
        buf.resize(bytes < kIoChunk ? bytes : kIoChunk);
    } catch (...) {
        std::fclose(fp);
        return set_error(RMQ_ENOMEM, "rmq_save: host buffer");
    }
    bool ok = std::fwrite(&hd, sizeof(hd), 1, fp) == 1;
    for (size_t off = 0; ok && off < bytes; off += buf.size()) {
        const size_t m = bytes - off < buf.size() ? bytes - off : buf.size();
        cudaError_t err = cudaMemcpyAsync(buf.data(), static_cast<char *>(mem) + off, m,
                                          cudaMemcpyDeviceToHost, stream);
        if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
        if (err != cudaSuccess) {
            std::fclose(fp);
            return cuda_fail(err, "rmq_save: copy");
        }
        ok = std::fwrite(buf.data(), 1, m, fp) == m;
    }
    ok = (std::fclose(fp) == 0) && ok;
    if (!ok) return set_error(RMQ_EINVAL, "rmq_save: write to %s failed", path);
    return RMQ_OK;
}

int rmq_load(const float *d_vals, int64_t n, const char *path, rmq_stream_t stream,
             rmq_handle_t **out) {
    NvtxRange nvtx_range("rmq_load");
    if (!out || !path || !d_vals) return set_error(RMQ_EINVAL, "rmq_load: NULL argument");
    *out = nullptr;
    if (n <= 0 || n > 0x7fffffffLL) return set_error(RMQ_EINVAL, "rmq_load: bad n=%lld", (long long)n);
    if (reinterpret_cast<uintptr_t>(d_vals) % 4)
        return set_error(RMQ_EINVAL, "rmq_load: d_vals not 4-byte aligned");
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return set_error(RMQ_EINVAL, "rmq_load: cannot open %s", path);
    FileHeader hd;
    if (std::fread(&hd, sizeof(hd), 1, fp) != 1 || std::memcmp(hd.magic, kMagic, sizeof(kMagic)) ||
        hd.version != kVersion || hd.header_check != header_hash(hd)) {
        std::fclose(fp);
        return set_error(RMQ_EINVAL, "rmq_load: %s is not an index file of this version", path);
    }
    if (hd.n != static_cast<uint64_t>(n)) {
        std::fclose(fp);
        return set_error(RMQ_EINVAL, "rmq_load: index is for n=%llu, values have n=%lld",
                         (unsigned long long)hd.n, (long long)n);
    }
    BuildPlan p;
    std::memset(&p, 0, sizeof(p));
    p.A = d_vals;
    p.n = static_cast<uint32_t>(n);
    p.bs = static_cast<uint32_t>(hd.bs);
    p.kmode = ((hd.flags & RMQ_BUILD_INT32) ? kIntMin : kFloatMin) + ((hd.flags & RMQ_BUILD_MAX) ? 1u : 0u);
    p.light = (hd.flags & RMQ_BUILD_LIGHT) != 0;
    // a light index may round a block size above n up to a multiple of 32
    const uint64_t bs_max = p.light ? (hd.n + 31) / 32 * 32 : hd.n;
    const size_t bytes = (hd.bs >= 1 && hd.bs <= bs_max)
                             ? plan_index(p, (hd.flags & RMQ_BUILD_NO_MICRO) != 0) : 0;
    if (!bytes || bytes != hd.bytes || p.nb != hd.nb || p.levels != hd.levels ||
        p.nmicro != hd.nmicro || p.mlevels != hd.mlevels) {
        std::fclose(fp);
        return set_error(RMQ_EINVAL, "rmq_load: %s has an inconsistent layout", path);
    }
    uint64_t print = 0;
    int rc = fingerprint(d_vals, p.n, stream, &print);
    if (rc) {
        std::fclose(fp);
        return rc;
    }
    if (print != hd.values_print) {
        std::fclose(fp);
        return set_error(RMQ_EINVAL,
                         "rmq_load: the values differ from those the index was built from");
    }
    void *mem = nullptr;
    cudaError_t err = dev_malloc(&mem, bytes);
    if (err != cudaSuccess) {
        std::fclose(fp);
        cudaGetLastError();
        return set_error(RMQ_ENOMEM, "rmq_load: cudaMalloc(%zu) failed", bytes);
    }
    std::vector<char> buf;
    try {
        buf.resize(bytes < kIoChunk ? bytes : kIoChunk);
    } catch (...) {
        std::fclose(fp);
        cudaFree(mem);
        return set_error(RMQ_ENOMEM, "rmq_load: host buffer");
    }
    for (size_t off = 0; off < bytes; off += buf.size()) {
        const size_t m = bytes - off < buf.size() ? bytes - off : buf.size();
        if (std::fread(buf.data(), 1, m, fp) != m) {
            std::fclose(fp);
            cudaFree(mem);
            return set_error(RMQ_EINVAL, "rmq_load: %s is truncated", path);
        }
        err = cudaMemcpyAsync(static_cast<char *>(mem) + off, buf.data(), m,
                              cudaMemcpyHostToDevice, stream);
        if (err == cudaSuccess) err = cudaStreamSynchronize(stream);
        if (err != cudaSuccess) {
            std::fclose(fp);
            cudaFree(mem);
            return cuda_fail(err, "rmq_load: copy");
        }
    }
    std::fclose(fp);
    rc = handle_adopt(p, mem, bytes, stream, out);
    if (rc) cudaFree(mem);
    return rc;
}

}  // extern "C"
