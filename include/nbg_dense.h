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

enum { NBG_DENSE_SPLIT_BF16 = 0, NBG_DENSE_FP32 = 1 };

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

#ifdef __cplusplus
}
#endif

#endif /* NBG_DENSE_H */
