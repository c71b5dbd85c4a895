// nbg_decay.cu -- STDP decay factors of the dense-runtime profile, computed
// on the device with CUDA's expf exactly as the reference's dense GPU
// learning kernels do (src/native/gpu/include/dense_subnetwork/learning/
// DenseLearningDeviceRuntime.cuh:65-77: expf(-(float)(t - last) * dt_ms *
// inv_tau)), so the table holds the same bits those kernels would use.  This
// translation unit keeps nvcc's default floating-point contraction, as the
// reference's kernels are built; the engine's other kernels are built
// without it.

#include <cuda_runtime.h>

#include "nbg_common.cuh"

namespace {

// Factor w (0: LTP trace, 1: LTD trace) of rule r at gap k, the two traces of
// one gap side by side (the engine reads both with one 8-byte load):
// tab[(r * len + k) * 2 + w] = expf(-((float)k * dt) * inv[r * 2 + w])
__global__ void k_decay_table(float *__restrict__ tab, const float *__restrict__ inv, int len, float dt,
                              long long total) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int row = (int)(i / len), k = (int)(i % len);
    const float delta_time = (float)k * dt;
    tab[((size_t)(row >> 1) * len + k) * 2 + (row & 1)] = expf(-delta_time * inv[row]);
}

} // namespace

// Fill `tab` (device, rows x len floats, rows = 2 per rule, laid out as above)
// from the per-row inverse time constants `inv_host`; synchronous.
NBG_HIDDEN cudaError_t nbg_device_decay_table(float *tab, const float *inv_host, int rows, int len, float dt) {
    float *inv = nullptr;
    cudaError_t e = cudaMalloc(&inv, rows * sizeof(float));
    if (e != cudaSuccess) return e;
    e = cudaMemcpy(inv, inv_host, rows * sizeof(float), cudaMemcpyHostToDevice);
    const long long total = (long long)rows * len;
    if (e == cudaSuccess) {
        k_decay_table<<<(unsigned)((total + 255) / 256), 256>>>(tab, inv, len, dt, total);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    cudaFree(inv);
    return e;
}
