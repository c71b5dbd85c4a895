/*
 * nbg.h -- C ABI of the GB300 spiking-network step engine.
 *
 * This is the boundary the reference's C++ host (and its pybind11 module)
 * calls instead of the legacy per-model GPU interfaces and the dense runtime.
 * Plain C types only: no torch, no C++ objects cross it.  Every entry point
 * returns an nbg_status; nbg_last_error() gives a readable reason for the
 * last failure on the calling thread (the reference reports reasons through
 * `bool + std::string* reason`, e.g. src/native/gpu/src/gpu_runtime/
 * GpuPropagationRuntime.cu:19-29).
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   nbg_create      Simulation::Simulation(NeuronLayerDescription...,
 *                   ConnectionDescription..., LearningRuleDescription...)
 *                   src/native/legacy/source_file_realtime_v1_async/
 *                   Simulation/inc/Simulation.h:187-250, and the network
 *                   compile Network::CaculateOutputConnection /
 *                   CaculateInputConnection (Network/src/Network.cu:483-735)
 *   nbg_run         Simulation::RunSimulationStep(int) (Simulation.h:182,
 *                   Simulation/src/Simulation.cu:383-474) together with the
 *                   CoreCuda per-model UpdateState launches
 *                   (TimeDrivenLIF_Voltage_jump_GPU_Interface.cu:70-104) and
 *                   DenseSubnetworkRuntimeGpu::RunStep
 *                   (src/native/gpu/src/dense_subnetwork/
 *                   DenseSubnetworkRuntimeGpu.cpp:625-665)
 *   nbg_get_state   the per-neuron state read of _core.Simulation.neuron_state
 *                   (python/bindings/neuronbridge_core.cpp:940-975)
 *   nbg_get_spikes  _core.Simulation.output_spikes (neuronbridge_core.cpp:490-508)
 *   nbg_get_weights / nbg_set_weight
 *                   Simulation::Get/SetConnectionWeight (Simulation.h:367-373)
 *   nbg_reset       Simulation::ResetForNextRound
 */
#ifndef NBG_H
#define NBG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int nbg_status;
enum {
    NBG_OK = 0,
    NBG_ERR_INVALID = 1,  /* bad argument or network description */
    NBG_ERR_CUDA = 2,     /* a CUDA runtime call failed */
    NBG_ERR_OOM = 3,      /* device allocation failed */
    NBG_ERR_OVERFLOW = 4, /* a recording buffer filled up */
    NBG_ERR_STATE = 5,    /* call not valid in the engine's current state */
    NBG_ERR_TIMEOUT = 6,  /* a bounded device wait gave up */
    NBG_ERR_UNSUPPORTED = 7
};

/* Neuron models (catalog names in parentheses, aliases as in the reference's
 * src/native/shared/src/neuron_model/NeuronModelCatalog.cpp:60-200). */
enum {
    NBG_MODEL_LIF_VJ = 0,   /* TimeDrivenLIF_Voltage_jump[_GPU] */
    NBG_MODEL_IZH_COND = 1, /* TimeDrivenIzhikevic_[I_]Exponential_Decay[_GPU] */
    NBG_MODEL_IZH_RK4 = 2,  /* IzhikevichCurrentRK4: current pulses, noise, RK4 */
    NBG_MODEL_POISSON = 3,  /* PoissonRate[_GPU] */
    /* Event-driven input layers (InputSpikeNeuronModel,
     * InputCurrentNeuronModel; python/src/neuronbridge/model.py:162-185): no
     * dynamics, never fire by themselves.  Their neurons are the sources of
     * nbg_add_external_spikes / nbg_add_external_currents. */
    NBG_MODEL_INPUT_SPIKE = 4,
    NBG_MODEL_INPUT_CURRENT = 5
};

/* Synapse types: 0 excitatory, 1 inhibitory (spike synapses), 3 current
 * synapse (carries the latched current of its input-current source, see
 * nbg_add_external_currents; never a learning rule). */
enum { NBG_SYN_EXC = 0, NBG_SYN_INH = 1, NBG_SYN_CURRENT = 3 };

/* Semantics profile: LEGACY_CPU is the parity target (strict '>' LIF
 * threshold, refractory-gated arrivals); DENSE follows the reference's dense
 * GPU runtime for the voltage-jump LIF ('>=' threshold, ungated arrivals,
 * v starts at V_rest). */
enum { NBG_SEM_LEGACY_CPU = 0, NBG_SEM_DENSE = 1 };

#define NBG_NFP 16
#define NBG_NIP 4

/* Per-layer parameters.  Slot meaning by model:
 *  LIF_VJ:   f[0] V_rest, f[1] tau, f[2] V_th, f[3] R, f[4] V_reset,
 *            f[5] random_mu[0], f[6] I_ext;          ip[0] t_ref (steps)
 *  IZH_COND: f[0] a, f[1] b, f[2] c, f[3] d, f[4] V_rest, f[5] V_th, f[6] R,
 *            f[7] E_ampa, f[8] ampa_tau, f[9] E_gaba, f[10] gaba_tau,
 *            f[11] I_ext
 *  IZH_RK4:  f[0] a, f[1] b, f[2] c, f[3] d, f[4] v0, f[5] V_th,
 *            f[6] noise sigma, f[7] I_bias
 *  POISSON:  f[0] rate_bias_hz, f[1] rate_gain_hz_per_current, f[2] I_ext
 *  INPUT_SPIKE, INPUT_CURRENT: no parameters */
typedef struct {
    int model;
    int count;
    float f[NBG_NFP];
    int ip[NBG_NIP];
    int output; /* record this layer's spikes (NeuronLayer.output) */
} nbg_layer_desc;

/* Pair STDP parameters (STDP::SetParameters keys Max_LTP, LTP_tau, Max_LTD,
 * LTD_tau; src/native/legacy/.../LearningRule/src/Rule/STDP.cpp:63-87). */
typedef struct {
    float max_ltp, ltp_tau, max_ltd, ltd_tau;
} nbg_stdp_desc;

/* Network description: layers in creation order (global neuron ids are
 * assigned layer by layer), then connections as parallel arrays in original
 * connection order (the reference's ConnectionDescription,
 * Network/inc/NetworkConstructStructure.h:18-74).  type 0 = excitatory,
 * 1 = inhibitory, 3 = current; delay in steps (>= 1); rule = index into
 * rules or -1 (always -1 for a current synapse). */
typedef struct {
    int n_layers;
    const nbg_layer_desc *layers;
    int64_t n_conn;
    const int32_t *source;
    const int32_t *target;
    const int32_t *type;
    const float *weight;
    const float *max_weight;
    const int32_t *delay;
    const int32_t *rule;
    int n_rules;
    const nbg_stdp_desc *rules;
    float dt_ms;
    int semantics;
    uint64_t seed; /* noise seed for IZH_RK4 layers */
} nbg_net_desc;

/* Engine options (no reference counterpart; the reference's SimulationConfig
 * queues/event_queue have no meaning on the device). */
typedef struct {
    int device;            /* CUDA device ordinal */
    int block_steps;       /* max steps per update launch (0 = auto: min delay) */
    int threads_per_block; /* 0 = auto */
    int64_t spike_capacity;/* device raster capacity per run call (0 = auto) */
    int use_graph;         /* capture the per-block launches in a CUDA graph */
    int64_t event_log_capacity; /* >0: log delivered events (testing aid) */
    int kernel_timing;     /* bracket every launch with CUDA events (nbg_profile) */
} nbg_options;

typedef struct nbg_engine nbg_engine;

const char *nbg_last_error(void);
const char *nbg_version(void);

void nbg_default_options(nbg_options *opt);
nbg_status nbg_create(const nbg_net_desc *desc, const nbg_options *opt, nbg_engine **out);
nbg_status nbg_destroy(nbg_engine *e);

/* One engine over n independent networks (the batched form of nbg_create:
 * one step loop and one launch per block for all of them).  Layers,
 * connections and learning rules are concatenated, instance k's neuron ids
 * offset by the neurons of instances 0..k-1 and its rule ids by their rules;
 * ids are checked per instance.  first_neuron (n + 1 entries, may be null)
 * receives each instance's first engine neuron id and the total.  All
 * instances share dt_ms, semantics and seed; PoissonRate draws are local to
 * their layer, so every instance behaves exactly as when created alone,
 * except the noise of IZH_RK4 layers, which is keyed by the engine-wide
 * neuron id.  The reference creates one Simulation per network
 * (src/native/legacy/source_file_realtime_v1_async/Simulation/inc/Simulation.h:187-250). */
nbg_status nbg_create_batch(const nbg_net_desc *const *descs, int n, const nbg_options *opt, nbg_engine **out,
                            int64_t *first_neuron);

/* Advance the network.  The first call performs steps+1 updates (t=0..steps),
 * later calls perform `steps` updates, matching the reference's run(). */
nbg_status nbg_run(nbg_engine *e, int steps);
nbg_status nbg_reset(nbg_engine *e);
/* Put neurons [first, first + count) back to their initial state and drop
 * the arrivals pending for them; synapses keep their weights and traces and
 * the simulation time goes on.  Replaces the reset of one dense subnetwork
 * (DenseSubnetworkModel::Reset, src/native/gpu/src/simulation_dense/
 * DenseSubnetworkModel.cpp:173-183, reached from Simulation.reset_dense_subnetwork,
 * python/bindings/neuronbridge_core.cpp:627-632). */
nbg_status nbg_reset_neurons(nbg_engine *e, int first, int count);
nbg_status nbg_next_time(const nbg_engine *e, int *t);
nbg_status nbg_num_neurons(const nbg_engine *e, int *n);
nbg_status nbg_num_synapses(const nbg_engine *e, int64_t *s);
/* minimum delay over synapses (the temporal-blocking window) */
nbg_status nbg_block_steps(const nbg_engine *e, int *b);
/* Change the launch shape of a live engine: threads per block (multiple of
 * 32, <= 256) and steps per update launch (1 .. min delay; 0 = the min
 * delay).  Results do not depend on either; only speed does. */
nbg_status nbg_set_launch(nbg_engine *e, int threads_per_block, int block_steps);

/* State fields for nbg_get_state / nbg_set_state. */
enum {
    NBG_FIELD_V = 0,
    NBG_FIELD_U = 1,
    NBG_FIELD_G_EXC = 2,
    NBG_FIELD_G_INH = 3,
    NBG_FIELD_I_EXT = 4,
    NBG_FIELD_LAST_SPIKE = 6 /* written as float */
};
nbg_status nbg_get_state(nbg_engine *e, int field, float *out /* n_neurons */);
nbg_status nbg_set_state(nbg_engine *e, int field, const float *in /* n_neurons */);

/* Spikes of output layers recorded by all run calls so far, ordered by
 * (time, neuron id) -- the reference's output spike buffer
 * (ArrayOutputSpikeDriver, read by _core.Simulation.output_spikes). */
nbg_status nbg_num_spikes(nbg_engine *e, int64_t *n);
nbg_status nbg_get_spikes(nbg_engine *e, int32_t *times, int32_t *ids, int64_t capacity);
nbg_status nbg_clear_spikes(nbg_engine *e);
/* The STDP decay factors the engine applies for a gap of k steps:
 * out[k] = factor of trace `which` (0: Apre / LTP_tau, 1: Apost / LTD_tau) of
 * rule `rule`, for k < *len (longer gaps decay to 0).  Legacy profile: host
 * libm expf of -((float)k * dt) * (float)(1.0 / (double)tau)
 * (STDP_State.cpp:5-26); dense profile: CUDA expf with 1.0f / max(1e-6f, tau)
 * (DenseLearningDeviceRuntime.cuh:65-77).  Copies min(capacity, *len). */
nbg_status nbg_get_decay_table(nbg_engine *e, int rule, int which, int64_t capacity, float *out, int64_t *len);
/* Entries [offset, offset + count) of the recorded spikes (a monitor reading
 * only what the last run call added). */
nbg_status nbg_get_spikes_from(nbg_engine *e, int64_t offset, int64_t count, int32_t *times, int32_t *ids);
/* Record (or stop recording) the spikes of layer `layer` in the raster.  At
 * create a layer is recorded iff it is an output; the DebugMonitor also
 * records the layers of the neurons it watches (the reference's
 * Simulation::WriteSpike feeds the monitor for every spike,
 * Simulation.cu:611-633).  Takes effect from the next run call. */
nbg_status nbg_set_layer_record(nbg_engine *e, int layer, int record);
/* delivered synaptic events accumulated over all run calls */
nbg_status nbg_num_events(nbg_engine *e, int64_t *n);

/* Weights and STDP state in original connection order. */
nbg_status nbg_get_weights(nbg_engine *e, float *w, float *apre, float *apost, int32_t *last);
nbg_status nbg_set_weight(nbg_engine *e, int64_t conn, float w);
/* All weights at once, original connection order (weight snapshot load,
 * the reference's Simulation::LoadWeight, Simulation.h:363). */
nbg_status nbg_set_weights(nbg_engine *e, const float *w);

/* Set neuron `id`'s external current to `value` at the start of step t
 * (before that step's arrivals), as a delay-d current connection from an
 * input-current neuron does in the reference (ProcessCurrent sets the
 * target's total current, e.g. TimeDrivenLIF_Voltage_jump.cpp:117-124;
 * PROPOGATEDCURRENT outranks PROPOGATEDSPIKE, Event.h:10). */
nbg_status nbg_set_current_at(nbg_engine *e, int t, int id, float value);

/* External spikes (Simulation::AddExternalSpikeActivity, Simulation.h:256;
 * ArrayInputSpikeDriver.cpp:15-24; InputSpike.cpp:12-29): neuron ids[k]
 * emits a spike at step times[k].  It is recorded in the raster (if its layer
 * is an output) and delivered over its out-going spike synapses at
 * times[k] + delay, with the pre-synaptic learning hook, exactly like a spike
 * of the update; the neuron's own state and the post-synaptic hook are not
 * touched.  The delivery is fused into the propagation kernel of the block
 * that contains times[k] (no per-step host work).  Sources must belong to an
 * NBG_MODEL_INPUT_SPIKE layer (such a neuron never fires by itself, so one
 * spike per step is all it can carry); a (time, neuron) pair given twice, or
 * a time before nbg_next_time, is rejected.  Events after the current call
 * stay pending for later calls; nbg_reset drops them. */
nbg_status nbg_add_external_spikes(nbg_engine *e, int64_t n, const int32_t *times, const int32_t *ids);

/* External currents (Simulation::AddExternalCurrentActivity, Simulation.h:258;
 * ArrayInputCurrentDriver.cpp:12-19; InputCurrent.cpp:13-24;
 * PropogatedCurrent.cpp:13-24): input-current neuron ids[k] sends currents[k]
 * at step times[k] over each of its current synapses (type 3).  At
 * times[k] + delay the synapse latches the value, and its target's external
 * current becomes the float sum of the latched values of all its current
 * synapses (in the target's synapse order: source, delay, connection index),
 * as CurrentSynapse::GetTotalInputCurrentPerNeuron does before
 * ProcessCurrent stores it (TimeDrivenLIF_Voltage_jump.cpp:117-124).  Applied
 * at the start of that step, after any nbg_set_current_at value for it. */
nbg_status nbg_add_external_currents(nbg_engine *e, int64_t n, const int32_t *times, const int32_t *ids,
                                     const float *currents);
/* A PoissonRate layer without incoming synapses is a generator: its spikes
 * are a pure function of (local index, step), so targets evaluate them inline
 * instead of through the delay ring.  Timed currents into generator neurons
 * are rejected with NBG_ERR_UNSUPPORTED. */

/* Membrane (field 0) traces of selected neurons, one row per update. */
nbg_status nbg_set_trace(nbg_engine *e, int n, const int32_t *ids);
nbg_status nbg_num_trace_rows(nbg_engine *e, int64_t *rows);
nbg_status nbg_get_traces(nbg_engine *e, float *out /* rows * n */);

/* Delivered-event log (testing aid, enabled by options.event_log_capacity):
 * (time, original connection index, delivered weight). */
nbg_status nbg_num_logged_events(nbg_engine *e, int64_t *n);
nbg_status nbg_get_logged_events(nbg_engine *e, int32_t *t, int64_t *conn, float *w);

/* Device timings of the last run call, from CUDA events on the engine's
 * stream: total_ms spans all launches of the call; with options.kernel_timing
 * update_ms / propagate_ms sum the per-launch durations of the update (drain
 * + neuron step) and spike-propagation kernels (else 0).  launches counts the
 * kernels launched.  Mirrors the phase split of the reference's
 * bench_profiling_snapshot (neuronbridge_core.cpp:1887). */
nbg_status nbg_profile(nbg_engine *e, double *total_ms, double *update_ms, double *propagate_ms,
                       int64_t *launches);

/* Raster phases of the last nbg_run call: the device ordering of its spike
 * raster into (step, id) order (CUDA events; order_launches kernels), the
 * download to the host and the append to the recorded raster (host wall
 * time).  The reference records output spikes from its host event loop
 * (communication/src/ArrayOutputSpikeDriver.cpp); here they are this
 * separate phase after the step loop.  If the device ordering fails (its
 * buffers cannot be allocated), nbg_run downloads the unordered entries and
 * orders them on the host instead, and order_launches reads -1. */
nbg_status nbg_raster_profile(nbg_engine *e, double *order_ms, double *download_ms, double *append_ms,
                              int64_t *order_launches);

#ifdef __cplusplus
}
#endif

#endif /* NBG_H */
