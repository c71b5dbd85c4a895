/*
 * nbg_dense.h -- C ABI of the dense all-to-all delivery engine: many LIF
 * populations ("instances") sharing one dense recurrent weight matrix, with
 * spike delivery I_t = S_{t-1} W computed each step either as a BF16 tensor-
 * core GEMM with W split into hi + lo BF16 parts (FP32 accumulation) or as an
 * exact FP32 CUDA-core gather-sum (the comparison path).
 *
 * Reference counterpart: the dense-subnetwork delivery of the reference's
 * DenseRuntime -- GpuPropagationRuntime's firing-history mark and per-post
 * drain into pending channels (src/native/gpu/src/gpu_runtime/
 * GpuPropagationRuntime.cu:150-266) followed by the unified neuron update
 * (src/native/gpu/src/dense_subnetwork/DenseUnifiedNeuronRuntime.cu:45-149).
 * The reference stores dense subnetworks as sparse CSC lists; for all-to-all
 * connectivity this engine stores W densely and delivers with a GEMM.
 *
 * Neuron model: the voltage-jump LIF of nbg_layer_desc (legacy semantics);
 * the summed arrival of a step (recurrent + drive) is added to V once when
 * the neuron is not refractory.  Drive: each neuron receives a PoissonRate
 * source (hash index = instance * neurons + neuron) with delay 1.
 */
#ifndef NBG_DENSE_H
#define NBG_DENSE_H

#include "nbg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Delivery paths: SPLIT_BF16 = tcgen05 tensor cores (TMEM accumulator, bulk
 * copies); FP32 = exact CUDA-core gather-sum; SPLIT_BF16_SYNC = the same
 * split-precision GEMM on the legacy mma.sync tensor path (for comparison). */
enum { NBG_DENSE_SPLIT_BF16 = 0, NBG_DENSE_FP32 = 1, NBG_DENSE_SPLIT_BF16_SYNC = 2 };

typedef struct nbg_dense nbg_dense;

/* w: neurons x neurons FP32, row = pre-synaptic, column = post-synaptic.
 * neurons must be a multiple of 128 and instances 64 (the GEMM tile). */
nbg_status nbg_dense_create(int instances, int neurons, const float *w, const nbg_layer_desc *lif,
                            float drive_rate_hz, float drive_weight, float dt_ms, int precision, int device,
                            nbg_dense **out);
nbg_status nbg_dense_destroy(nbg_dense *d);
/* same step schedule as nbg_run: the first call performs steps + 1 updates */
nbg_status nbg_dense_run(nbg_dense *d, int steps);
nbg_status nbg_dense_reset(nbg_dense *d);
/* V and refractory counters, instance-major (instances x neurons) */
nbg_status nbg_dense_get_state(nbg_dense *d, float *v, int32_t *last);
/* spikes per update of all run calls so far */
nbg_status nbg_dense_num_steps(nbg_dense *d, int64_t *n);
nbg_status nbg_dense_spike_counts(nbg_dense *d, int32_t *counts);
/* current binary spike matrix S (instances x neurons, 0/1) of the last update */
nbg_status nbg_dense_get_spikes(nbg_dense *d, uint8_t *s);
/* One delivery through this engine's path on a caller-supplied binary S
 * (instances x neurons, host): out = S W (instances x neurons). */
nbg_status nbg_dense_deliver(nbg_dense *d, const uint8_t *s, float *out);
/* milliseconds of the last run call: all launches, and the delivery kernel
 * alone (CUDA events on the engine stream) */
nbg_status nbg_dense_profile(nbg_dense *d, double *total_ms, double *delivery_ms, int64_t *launches);

/* One split-BF16 spike delivery that allocates nothing -- no counterpart in
 * the reference.
 *
 * For callers that cannot call cudaMalloc: a host that owns all device memory
 * and hands the library its own buffers, a real-time control loop (the
 * reference's closed-loop robot mode) where an allocator call may stall the
 * device mid-run, or code whose stream is being captured in the global
 * capture mode, where cudaMalloc is refused.  The caller passes every input
 * and output as device pointers; the split-K partial sums live in a file-scope
 * __device__ array of NBG_DENSE_NOALLOC_MAX_NEURONS * 64 * 2 floats (4 MiB),
 * which every GPU that loads the library holds until the process exits.
 *
 *   w_hi_t, w_lo_t  BF16, neurons x neurons, row = post-synaptic neuron, column
 *                   = pre-synaptic neuron (W transposed): W_hi = bf16(W),
 *                   W_lo = bf16(W - W_hi), both round-to-nearest-even
 *   spikes          BF16 0/1, 64 x neurons (instance-major)
 *   out             FP32, 64 x neurons: out = spikes W
 *   neurons         a multiple of 128, at most NBG_DENSE_NOALLOC_MAX_NEURONS
 *                   (larger sizes are rejected with NBG_ERR_INVALID)
 *
 * w_hi_t, w_lo_t and spikes must be 16-byte aligned (the kernel reads them
 * with 16-byte copies) and out 4-byte aligned; a misaligned pointer, such as
 * an offset view into a larger tensor, is rejected with NBG_ERR_INVALID before
 * anything is launched.
 *
 * The first call on a device looks up the scratch array's device address
 * there (with that device current) and keeps it for the life of the process;
 * make that first call before any stream capture.  The address is not valid
 * across cudaDeviceReset (the module is loaded again and the array may move),
 * so do not use this function after resetting a device it has already run
 * on.  Every call shares the one scratch array, so calls that overlap on
 * the GPU (different streams, or different host threads on the same device)
 * race: order them on one stream.  The scratch needs no clearing -- each call
 * writes every partial sum it reads. */
#define NBG_DENSE_NOALLOC_MAX_NEURONS 8192
nbg_status nbg_dense_deliver_noalloc(const void *w_hi_t, const void *w_lo_t, const void *spikes, float *out,
                                     int neurons, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* NBG_DENSE_H */
