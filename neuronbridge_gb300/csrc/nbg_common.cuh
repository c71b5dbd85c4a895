// nbg_common.cuh -- internals shared by the translation units of libnbg:
// thread-local error text (read through nbg_last_error), the CUDA status
// check, and a minimal owning device buffer.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "nbg.h"

#define NBG_HIDDEN __attribute__((visibility("hidden")))

// Record `fmt` as the calling thread's last error and return `code`.
NBG_HIDDEN nbg_status nbg_fail(nbg_status code, const char *fmt, ...);

#define NBG_CUDA(call)                                                                                   \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess)                                                                           \
            return nbg_fail(e_ == cudaErrorMemoryAllocation ? NBG_ERR_OOM : NBG_ERR_CUDA,                \
                            "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count) {
        release();
        n = count;
        if (count == 0) return cudaSuccess;
        return cudaMalloc(&p, count * sizeof(T));
    }
    cudaError_t upload(const std::vector<T> &h) {
        cudaError_t e = alloc(h.size());
        if (e != cudaSuccess || h.empty()) return e;
        return cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    }
    cudaError_t zero() { return n ? cudaMemset(p, 0, n * sizeof(T)) : cudaSuccess; }
};

// PoissonRate hash (reference PoissonRate.cpp:12-22)
__device__ __forceinline__ float nbg_hash_uniform01(int neuron_index, int time_step) {
    unsigned int x = (unsigned int)neuron_index * 747796405u + (unsigned int)(time_step + 1) * 2891336453u +
                     0x9e3779b9u;
    x ^= x >> 16;
    x *= 2246822519u;
    x ^= x >> 13;
    x *= 3266489917u;
    x ^= x >> 16;
    return (float)(x & 0x00FFFFFFu) / (float)0x01000000u;
}
