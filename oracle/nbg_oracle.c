/*
 * nbg_oracle.c -- CPU restatement of NeuronBridge's legacy time-driven step
 * loop.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the
 * CPU-baseline leg of the benchmark call it as the checker.  The product never
 * links or calls this file.
 *
 * The same source is compiled twice: REAL=float (symbols orc32_*) restates the
 * reference's FP32 arithmetic operation by operation; REAL=double (orc64_*) is
 * the FP64 oracle used to state FP32 error.  Build with -ffp-contract=off and
 * no fast-math so that every float operation rounds exactly once, as in the
 * reference's own scalar C++.
 *
 * Reference semantics restated here (paths relative to the reference project;
 * L/ = src/native/legacy/source_file_realtime_v1_async/):
 *  - step order at time t: every propagated spike group due at t (priority
 *    PROPOGATEDSPIKE) before every time-driven update (TIMEEVENT), Event.h:10;
 *    a spike emitted by the update at t is due at t+delay.
 *  - the first run(N) performs N+1 updates (t = 0..N), later runs N updates:
 *    an update event is inserted at t=0 and EndSimulationTime has the lowest
 *    priority (gpu/src/simulation_dense/SimulationCommonHost.cpp:918-924).
 *  - per arrival: target ProcessSpike, then the pre-synaptic learning hook
 *    (L/Event/src/Spike/PropogatedSpikeGroup.cpp:41-68).
 *  - per update: model Euler step in index order, then for each spiking neuron
 *    its out-going groups are scheduled and the post-synaptic learning hook
 *    runs (L/Event/src/Spike/TimeDrivenInternalSpike.cpp:37-86).
 *
 * Canonical arrival order.  The reference applies the arrivals that fall on
 * one step in event-heap order, which is not a function of the network alone.
 * This restatement applies them per target in CSC order: ascending source id,
 * then delay, then original connection index.  For a single delay group (one
 * queue) that is exactly the reference's order, because spike lists are built
 * in ascending neuron index and each source's synapses are sorted by target
 * (L/Network/src/Network.cu:485-502).
 */
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL float
#endif
#ifndef ORC
#define ORC(name) orc32_##name
#endif
/* literal constants: float literals in the FP32 build (as the reference's
 * source writes them), exact double literals in the FP64 build */
#ifdef REAL_IS_DOUBLE
#define K(x) (x)
#else
#define K(x) (x##f)
#endif

/* model ids and parameter slots: identical numbering to include/nbg.h */
enum { M_LIF_VJ = 0, M_IZH_COND = 1, M_IZH_RK4 = 2, M_POISSON = 3, M_INPUT_SPIKE = 4, M_INPUT_CURRENT = 5 };
enum { SYN_CURRENT = 3 };
enum { SEM_LEGACY = 0, SEM_DENSE = 1 };
#define NFP 16
#define NIP 4

typedef struct {
    int model, start, count;
    REAL f[NFP];
    int ip[NIP];
    int has_exc, has_inh; /* CheckType flags: any type-0 / type-1 input */
    REAL decay_ampa, decay_gaba;
} layer_t;

typedef struct {
    int64_t *v;
    int64_t n, cap;
} vec64_t;

typedef struct {
    int n_layers, n_neurons, semantics;
    REAL dt;
    float dt_f; /* dt as the reference's float basetimesteps */
    uint64_t seed;
    layer_t *layers;
    int *layer_of; /* neuron -> layer index */
    /* neuron state (SoA) */
    REAL *v, *u, *g_ampa, *g_gaba, *i_ext, *rate;
    REAL *pend_e, *pend_i; /* dense profile: arrivals of the current step */
    int *last;
    /* synapses in CSC order (by target, source, delay, original index) */
    int64_t n_syn;
    int64_t *csc_ptr;    /* n_neurons+1 */
    int *csc_src, *csc_tgt, *csc_type, *csc_delay, *csc_rule;
    int64_t *csc_orig;   /* original connection index */
    REAL *csc_w, *csc_wmax;
    /* STDP state per synapse (only used when csc_rule >= 0) */
    REAL *apre, *apost;
    int *slast;
    /* CSR by source over CSC positions */
    int64_t *out_ptr, *out_pos;
    int n_rules;
    REAL *rp; /* per rule: MaxLTP, LTP_tau, MaxLTD, LTD_tau */
    REAL *inv_ltp, *inv_ltd;
    /* delay buckets indexed by arrival time modulo ring */
    int ring;
    vec64_t *bucket;
    /* time */
    int next_t, ran;
    /* recording */
    vec64_t spk; /* packed (t << 32 | id) */
    int n_trace, *trace_ids;
    REAL *trace;
    int64_t trace_n, trace_cap;
    int log_events;
    vec64_t ev_t, ev_pos; /* delivered events: time, csc position */
    REAL *ev_w;
    int64_t ev_wcap;
    int64_t n_events;
    /* timed external currents (t, neuron, value), applied before the arrivals
     * of step t: PROPOGATEDCURRENT outranks PROPOGATEDSPIKE (Event.h:10) and
     * ProcessCurrent sets the target's total current (e.g.
     * TimeDrivenLIF_Voltage_jump.cpp:117-124) */
    vec64_t cur_t, cur_id;
    REAL *cur_v;
    int64_t cur_vcap;
    /* external spikes (t, neuron) of input-spike neurons: InputSpike events
     * (L/InputSpikeDriver/src/ArrayInputSpikeDriver.cpp:15-24,
     * L/Event/src/Spike/InputSpike.cpp:12-29) */
    vec64_t ext_t, ext_id;
    /* external currents: one latch event (time of arrival, CSC position of the
     * current synapse, value) per current synapse of the sending input-current
     * neuron (L/Event/src/Current/InputCurrent.cpp:13-24,
     * PropogatedCurrent.cpp:13-24); each synapse keeps its latched value and
     * the target's current is the float sum over its current synapses
     * (CurrentSynapse::GetTotalInputCurrentPerNeuron) */
    vec64_t lat_t, lat_p;
    REAL *lat_v;
    int64_t lat_vcap;
    REAL *latch; /* per CSC position (only current synapses used) */
    /* decay factors supplied by the caller ([rule][2][len], factor of a gap of
     * k steps; longer gaps decay to 0): the dense-runtime profile's factors
     * come from CUDA's expf, which this file does not restate */
    float *dtab_ext;
    int64_t dtab_ext_len;
    int threads;          /* OpenMP threads for the per-step loops (1 = serial) */
    unsigned char *fired; /* per-neuron spike flags of the current update */
    int64_t *seg;         /* target segment starts of the sorted bucket */
    int64_t seg_cap;
} net_t;

static void vpush(vec64_t *a, int64_t x) {
    if (a->n == a->cap) {
        a->cap = a->cap ? a->cap * 2 : 64;
        a->v = (int64_t *)realloc(a->v, (size_t)a->cap * sizeof(int64_t));
    }
    a->v[a->n++] = x;
}

static int cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/* PoissonRate hash: L/NeuralModel/src/TimeDriven/PoissonRate.cpp:12-22 */
static float hash_uniform01(int neuron_index, int time_step) {
    uint32_t x = (uint32_t)neuron_index * 747796405u + (uint32_t)(time_step + 1) * 2891336453u + 0x9e3779b9u;
    x ^= x >> 16;
    x *= 2246822519u;
    x ^= x >> 13;
    x *= 3266489917u;
    x ^= x >> 16;
    return (float)(x & 0x00FFFFFFu) / (float)0x01000000u;
}

/* Counter-based N(0,1) approximation for the Izhikevich noise current: the
 * Irwin-Hall sum of twelve 16-bit uniforms (u + 1/2) / 2^16 minus 6, summed in
 * integers and converted once (exact in float).  Bits come from the PCG
 * RXS-M-XS 32-bit output permutation used as a hash (Jarzynski and Olano,
 * "Hash Functions for GPU Rendering", JCGT 9(3), 2020): a per-neuron key
 * from (seed, neuron), a per-step key from (neuron key, step), then six
 * 32-bit words (two uniforms each).  Not part of the reference (it has no
 * seeded noise). */
static uint32_t pcg_hash(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
static uint32_t noise_key(uint64_t seed, int neuron) {
    return pcg_hash((uint32_t)neuron ^ pcg_hash((uint32_t)seed ^ (uint32_t)(seed >> 32)));
}
static REAL gauss12(uint64_t seed, int neuron, int t) {
    uint32_t tk = pcg_hash(noise_key(seed, neuron) ^ ((uint32_t)t * 0x9E3779B9u));
    int32_t m = 0;
    for (uint32_t k = 0; k < 6; ++k) {
        uint32_t h = pcg_hash(tk + k);
        m += (int32_t)(h & 0xFFFFu) + (int32_t)(h >> 16);
    }
    return (REAL)(m + 6 - 6 * 65536) * (REAL)(1.0 / 65536.0);
}

static void set_err(char *err, int errlen, const char *msg) {
    if (err && errlen > 0) {
        strncpy(err, msg, (size_t)errlen - 1);
        err[errlen - 1] = 0;
    }
}

typedef struct {
    int tgt, src, delay;
    int64_t idx;
} sortkey_t;
static int cmp_csc(const void *a, const void *b) {
    const sortkey_t *x = (const sortkey_t *)a, *y = (const sortkey_t *)b;
    if (x->tgt != y->tgt) return x->tgt < y->tgt ? -1 : 1;
    if (x->src != y->src) return x->src < y->src ? -1 : 1;
    if (x->delay != y->delay) return x->delay < y->delay ? -1 : 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

void ORC(destroy)(void *hp);

/* Initial state of neuron i of layer L. */
static void init_neuron(net_t *n, const layer_t *L, int i) {
    n->last[i] = 10000;
    switch (L->model) {
    case M_LIF_VJ:
        /* legacy: V = V_reset + random_mu (TimeDrivenLIF_Voltage_jump.cpp:37);
         * dense profile: v = v_rest (gpu DenseLifVoltageJumpModel.h ResetStateFields) */
        n->v[i] = n->semantics == SEM_DENSE ? L->f[0] : L->f[4] + L->f[5];
        n->i_ext[i] = L->f[6];
        break;
    case M_IZH_COND:
        /* v = V_rest, u = b*V_rest (TimeDrivenIzhikevic_Exponential_Decay.cpp:50) */
        n->v[i] = L->f[4];
        n->u[i] = L->f[1] * L->f[4];
        n->i_ext[i] = L->f[11];
        break;
    case M_IZH_RK4:
        n->v[i] = L->f[4];
        n->u[i] = L->f[1] * L->f[4];
        n->i_ext[i] = L->f[7];
        break;
    case M_POISSON:
        n->i_ext[i] = L->f[2];
        break;
    }
}

void *ORC(create)(int n_layers, const int *model, const int *count, const float *fparams, const int *iparams,
                  int64_t n_conn, const int *src, const int *tgt, const int *type, const float *w,
                  const float *wmax, const int *delay, const int *rule, int n_rules, const float *rparams,
                  float dt, int semantics, uint64_t seed, char *err, int errlen) {
    net_t *n = (net_t *)calloc(1, sizeof(net_t));
    n->n_layers = n_layers;
    n->dt = (REAL)dt;
    n->dt_f = dt;
    n->seed = seed;
    n->semantics = semantics;
    n->layers = (layer_t *)calloc((size_t)n_layers, sizeof(layer_t));
    int total = 0;
    for (int l = 0; l < n_layers; ++l) {
        layer_t *L = &n->layers[l];
        L->model = model[l];
        L->start = total;
        L->count = count[l];
        for (int k = 0; k < NFP; ++k) L->f[k] = (REAL)fparams[l * NFP + k];
        for (int k = 0; k < NIP; ++k) L->ip[k] = iparams[l * NIP + k];
        if (L->model < 0 || L->model > M_INPUT_CURRENT || L->count <= 0) {
            set_err(err, errlen, "bad layer");
            ORC(destroy)(n);
            return NULL;
        }
        total += count[l];
    }
    n->n_neurons = total;
    n->layer_of = (int *)malloc((size_t)total * sizeof(int));
    for (int l = 0; l < n_layers; ++l)
        for (int i = 0; i < n->layers[l].count; ++i) n->layer_of[n->layers[l].start + i] = l;

    /* CSC order */
    n->n_syn = n_conn;
    sortkey_t *keys = (sortkey_t *)malloc((size_t)(n_conn > 0 ? n_conn : 1) * sizeof(sortkey_t));
    int dmax = 1;
    for (int64_t s = 0; s < n_conn; ++s) {
        if (src[s] < 0 || src[s] >= total || tgt[s] < 0 || tgt[s] >= total || delay[s] < 1 ||
            !(type[s] == 0 || type[s] == 1 || type[s] == SYN_CURRENT) || (rule[s] >= n_rules) ||
            ((type[s] == SYN_CURRENT) != (n->layers[n->layer_of[src[s]]].model == M_INPUT_CURRENT)) ||
            (type[s] == SYN_CURRENT && rule[s] >= 0)) {
            set_err(err, errlen, "bad connection");
            free(keys);
            ORC(destroy)(n);
            return NULL;
        }
        keys[s].tgt = tgt[s];
        keys[s].src = src[s];
        keys[s].delay = delay[s];
        keys[s].idx = s;
        if (delay[s] > dmax) dmax = delay[s];
        layer_t *L = &n->layers[n->layer_of[tgt[s]]];
        if (type[s] == 0) L->has_exc = 1;
        if (type[s] == 1) L->has_inh = 1;
    }
    qsort(keys, (size_t)n_conn, sizeof(sortkey_t), cmp_csc);
    n->csc_ptr = (int64_t *)calloc((size_t)total + 1, sizeof(int64_t));
    size_t ns = (size_t)(n_conn > 0 ? n_conn : 1);
    n->csc_src = (int *)malloc(ns * sizeof(int));
    n->csc_tgt = (int *)malloc(ns * sizeof(int));
    n->csc_type = (int *)malloc(ns * sizeof(int));
    n->csc_delay = (int *)malloc(ns * sizeof(int));
    n->csc_rule = (int *)malloc(ns * sizeof(int));
    n->csc_orig = (int64_t *)malloc(ns * sizeof(int64_t));
    n->csc_w = (REAL *)malloc(ns * sizeof(REAL));
    n->csc_wmax = (REAL *)malloc(ns * sizeof(REAL));
    n->apre = (REAL *)calloc(ns, sizeof(REAL));
    n->apost = (REAL *)calloc(ns, sizeof(REAL));
    n->slast = (int *)calloc(ns, sizeof(int));
    n->latch = (REAL *)calloc(ns, sizeof(REAL));
    for (int64_t p = 0; p < n_conn; ++p) {
        int64_t s = keys[p].idx;
        n->csc_ptr[keys[p].tgt + 1]++;
        n->csc_src[p] = src[s];
        n->csc_tgt[p] = tgt[s];
        n->csc_type[p] = type[s];
        n->csc_delay[p] = delay[s];
        n->csc_rule[p] = rule[s];
        n->csc_orig[p] = s;
        n->csc_w[p] = (REAL)w[s];
        n->csc_wmax[p] = (REAL)wmax[s];
    }
    free(keys);
    for (int i = 0; i < total; ++i) n->csc_ptr[i + 1] += n->csc_ptr[i];
    /* CSR by source over CSC positions (order within a source is irrelevant:
     * every bucket is sorted by CSC position before it is applied) */
    n->out_ptr = (int64_t *)calloc((size_t)total + 1, sizeof(int64_t));
    n->out_pos = (int64_t *)malloc(ns * sizeof(int64_t));
    for (int64_t p = 0; p < n_conn; ++p) n->out_ptr[n->csc_src[p] + 1]++;
    for (int i = 0; i < total; ++i) n->out_ptr[i + 1] += n->out_ptr[i];
    {
        int64_t *fill = (int64_t *)malloc(((size_t)total + 1) * sizeof(int64_t));
        memcpy(fill, n->out_ptr, ((size_t)total + 1) * sizeof(int64_t));
        for (int64_t p = 0; p < n_conn; ++p) n->out_pos[fill[n->csc_src[p]]++] = p;
        free(fill);
    }
    /* learning rules: STDP(Max_LTP, LTP_tau, Max_LTD, LTD_tau); inverse taus
     * as STDP_State.cpp:5-7 (double division stored to float) */
    n->n_rules = n_rules;
    n->rp = (REAL *)malloc((size_t)(n_rules > 0 ? n_rules : 1) * 4 * sizeof(REAL));
    n->inv_ltp = (REAL *)malloc((size_t)(n_rules > 0 ? n_rules : 1) * sizeof(REAL));
    n->inv_ltd = (REAL *)malloc((size_t)(n_rules > 0 ? n_rules : 1) * sizeof(REAL));
    for (int r = 0; r < n_rules; ++r) {
        for (int k = 0; k < 4; ++k) n->rp[r * 4 + k] = (REAL)rparams[r * 4 + k];
        n->inv_ltp[r] = (REAL)(1.0 / (double)rparams[r * 4 + 1]);
        n->inv_ltd[r] = (REAL)(1.0 / (double)rparams[r * 4 + 3]);
    }
    n->ring = dmax + 1;
    n->bucket = (vec64_t *)calloc((size_t)n->ring, sizeof(vec64_t));

    /* state init: Neuron_State_Vector::InitNeuronState with sigma = 0,
     * LastSpike = 10000 (L/NeuralModel/src/NeuralStateVector/Neuron_State_Vector.cpp:43-69) */
    size_t nn = (size_t)total;
    n->v = (REAL *)calloc(nn, sizeof(REAL));
    n->u = (REAL *)calloc(nn, sizeof(REAL));
    n->g_ampa = (REAL *)calloc(nn, sizeof(REAL));
    n->g_gaba = (REAL *)calloc(nn, sizeof(REAL));
    n->i_ext = (REAL *)calloc(nn, sizeof(REAL));
    n->rate = (REAL *)calloc(nn, sizeof(REAL));
    n->pend_e = (REAL *)calloc(nn, sizeof(REAL));
    n->pend_i = (REAL *)calloc(nn, sizeof(REAL));
    n->last = (int *)malloc(nn * sizeof(int));
    n->fired = (unsigned char *)calloc(nn, 1);
    n->threads = 1;
    for (int l = 0; l < n_layers; ++l) {
        layer_t *L = &n->layers[l];
        for (int i = L->start; i < L->start + L->count; ++i) init_neuron(n, L, i);
        if (L->model == M_IZH_COND) {
            /* conductance decay factors: host std::exp(-dt * (1/tau)) in float
             * (TimeDrivenIzhikevic_Exponential_Decay.cpp:32-39) */
            float inv_a = (float)L->f[8] != 0.0f ? 1.0f / (float)L->f[8] : 0.0f;
            float inv_g = (float)L->f[10] != 0.0f ? 1.0f / (float)L->f[10] : 0.0f;
            if (sizeof(REAL) == sizeof(float) && semantics == SEM_DENSE) {
                /* dense runtime: std::exp(-dt_ms / tau) (DenseIzhikevichExponentialDecayModel.h:139-141) */
                L->decay_ampa = (REAL)expf(-dt / (float)L->f[8]);
                L->decay_gaba = (REAL)expf(-dt / (float)L->f[10]);
            } else if (sizeof(REAL) == sizeof(float)) {
                L->decay_ampa = (REAL)expf(-dt * inv_a);
                L->decay_gaba = (REAL)expf(-dt * inv_g);
            } else {
                L->decay_ampa = (REAL)exp(-(double)dt / (double)L->f[8]);
                L->decay_gaba = (REAL)exp(-(double)dt / (double)L->f[10]);
            }
        }
    }
    return n;
}

void ORC(destroy)(void *hp) {
    net_t *n = (net_t *)hp;
    if (!n) return;
    free(n->layers);
    free(n->layer_of);
    free(n->v);
    free(n->u);
    free(n->g_ampa);
    free(n->g_gaba);
    free(n->i_ext);
    free(n->rate);
    free(n->pend_e);
    free(n->pend_i);
    free(n->last);
    free(n->csc_ptr);
    free(n->csc_src);
    free(n->csc_tgt);
    free(n->csc_type);
    free(n->csc_delay);
    free(n->csc_rule);
    free(n->csc_orig);
    free(n->csc_w);
    free(n->csc_wmax);
    free(n->apre);
    free(n->apost);
    free(n->slast);
    free(n->out_ptr);
    free(n->out_pos);
    free(n->rp);
    free(n->inv_ltp);
    free(n->inv_ltd);
    if (n->bucket)
        for (int r = 0; r < n->ring; ++r) free(n->bucket[r].v);
    free(n->bucket);
    free(n->spk.v);
    free(n->trace_ids);
    free(n->trace);
    free(n->ev_t.v);
    free(n->ev_pos.v);
    free(n->ev_w);
    free(n->cur_t.v);
    free(n->cur_id.v);
    free(n->cur_v);
    free(n->ext_t.v);
    free(n->ext_id.v);
    free(n->lat_t.v);
    free(n->lat_p.v);
    free(n->lat_v);
    free(n->latch);
    free(n->dtab_ext);
    free(n->fired);
    free(n->seg);
    free(n);
}

/* STDP_State::SetUpdate (L/LearningRule/src/State/STDP_State.cpp:17-26):
 * deltaTime = (float)(t - last) * dt; A *= exp(-deltaTime * inv_tau). */
static void stdp_decay(net_t *n, int64_t p, int t) {
    int r = n->csc_rule[p];
    if (n->dtab_ext) {
        int64_t gap = (int64_t)t - n->slast[p];
        float fp = gap < n->dtab_ext_len ? n->dtab_ext[(size_t)(r * 2 + 0) * n->dtab_ext_len + gap] : 0.0f;
        float fm = gap < n->dtab_ext_len ? n->dtab_ext[(size_t)(r * 2 + 1) * n->dtab_ext_len + gap] : 0.0f;
        n->apre[p] *= (REAL)fp;
        n->apost[p] *= (REAL)fm;
    } else if (sizeof(REAL) == sizeof(float)) {
        float dtime = (float)(t - n->slast[p]) * n->dt_f;
        n->apre[p] *= (REAL)expf(-dtime * (float)n->inv_ltp[r]);
        n->apost[p] *= (REAL)expf(-dtime * (float)n->inv_ltd[r]);
    } else {
        double dtime = (double)(t - n->slast[p]) * (double)n->dt;
        n->apre[p] *= exp(-dtime / (double)n->rp[r * 4 + 1]);
        n->apost[p] *= exp(-dtime / (double)n->rp[r * 4 + 3]);
    }
    n->slast[p] = t;
}

static void clamp_w(net_t *n, int64_t p) {
    if (n->csc_w[p] < 0) n->csc_w[p] = 0;
    else if (n->csc_w[p] > n->csc_wmax[p]) n->csc_w[p] = n->csc_wmax[p];
}

/* STDP::ApplyPreSynaticSpike (L/LearningRule/src/Rule/STDP.cpp:19-35) */
static void stdp_pre(net_t *n, int64_t p, int t) {
    int r = n->csc_rule[p];
    stdp_decay(n, p, t);
    n->apre[p] += K(1.0);
    n->csc_w[p] += -n->rp[r * 4 + 2] * n->apost[p];
    clamp_w(n, p);
}

/* STDP::ApplyPostSynaticSpike (L/LearningRule/src/Rule/STDP.cpp:37-61) */
static void stdp_post(net_t *n, int j, int t) {
    for (int64_t p = n->csc_ptr[j]; p < n->csc_ptr[j + 1]; ++p) {
        int r = n->csc_rule[p];
        if (r < 0) continue;
        stdp_decay(n, p, t);
        n->apost[p] += K(1.0);
        n->csc_w[p] += n->rp[r * 4 + 0] * n->apre[p];
        clamp_w(n, p);
    }
}

/* Target-side arrival (ProcessSpike of each model). */
static void deliver(net_t *n, int64_t p, int t) {
    int j = n->csc_tgt[p];
    layer_t *L = &n->layers[n->layer_of[j]];
    REAL w = n->csc_w[p];
    int type = n->csc_type[p];
    if (n->log_events) {
        vpush(&n->ev_t, t);
        vpush(&n->ev_pos, p);
        if (n->ev_t.n > n->ev_wcap) {
            n->ev_wcap = n->ev_t.cap;
            n->ev_w = (REAL *)realloc(n->ev_w, (size_t)n->ev_wcap * sizeof(REAL));
        }
        n->ev_w[n->ev_t.n - 1] = w;
    }
    switch (L->model) {
    case M_LIF_VJ:
        /* TimeDrivenLIF_Voltage_jump::ProcessSpike (.cpp:100-113): gated by
         * LastSpike > t_ref.  The dense profile does not gate arrivals
         * (gpu DenseLifVoltageJumpDeviceUpdate.cuh:34); it accumulates them
         * separately (see update_lif). */
        if (n->semantics == SEM_DENSE) {
            if (type == 0) n->g_ampa[j] += w;
            else n->g_gaba[j] += w;
        } else if (n->last[j] > L->ip[0]) {
            if (type == 0) n->v[j] += w;
            else n->v[j] += -w;
        }
        break;
    case M_IZH_COND:
        /* legacy: g += w, not gated (TimeDrivenIzhikevic_Exponential_Decay.cpp:119-131);
         * dense profile: summed into the step's pending channels (i_pend) */
        if (n->semantics == SEM_DENSE) {
            if (type == 0) n->pend_e[j] += w;
            else n->pend_i[j] += w;
        } else if (type == 0) n->g_ampa[j] += w;
        else n->g_gaba[j] += w;
        break;
    case M_IZH_RK4:
        /* current pulse: accumulated into this step's synaptic current */
        if (type == 0) n->g_ampa[j] += w;
        else n->g_ampa[j] += -w;
        break;
    case M_POISSON:
        /* PoissonRate::ProcessSpike (PoissonRate.cpp:80-88) */
        if (type == 0) n->rate[j] += w;
        else n->rate[j] += -w;
        break;
    }
    if (n->csc_rule[p] >= 0) stdp_pre(n, p, t);
}

static int spiked_lif(net_t *n, layer_t *L, int i) {
    REAL eff_dt = n->dt; /* stride 1 */
    if (n->semantics == SEM_DENSE) {
        /* gpu DenseLifVoltageJumpDeviceUpdate.cuh:33-49, DenseIntegrationKernels.cuh:24-44 */
        REAL alpha = (REAL)(float)((float)n->dt_f / (float)L->f[1]);
        if (sizeof(REAL) == sizeof(double)) alpha = n->dt / L->f[1];
        REAL nv = n->v[i] + n->g_ampa[i] - n->g_gaba[i];
        n->g_ampa[i] = 0;
        n->g_gaba[i] = 0;
        if (n->last[i] >= L->ip[0]) nv = nv + alpha * (L->f[0] - nv + L->f[3] * n->i_ext[i]);
        n->last[i] += 1;
        int s = 0;
        if (nv >= L->f[2]) {
            nv = L->f[4];
            n->last[i] = 0;
            s = 1;
        }
        n->v[i] = nv;
        return s;
    }
    /* TimeDrivenLIF_Voltage_jump::CaculateDifferentialEquation (.cpp:49-63),
     * ForwardEulerMethod::CaculateIncreament (ForwardEulerMethod.h:29-55),
     * CaculateSpike (.cpp:74-86) */
    REAL cur = K(0.0);
    cur += L->f[3] * n->i_ext[i] / L->f[1];
    REAL aux;
    if (n->last[i] > L->ip[0]) aux = cur + (L->f[0] - n->v[i]) / L->f[1];
    else aux = 0;
    n->v[i] += aux * eff_dt;
    n->last[i] += 1;
    if (n->v[i] > L->f[2]) {
        n->v[i] = L->f[4];
        n->last[i] = 0;
        return 1;
    }
    return 0;
}

/* Dense-runtime Izhikevich (gpu DenseIzhikevichExponentialDecayDeviceUpdate.cuh
 * :10-68, DenseIntegrationKernels.cuh:10-75): decay-then-add conductances,
 * Euler step with u updated from the new v, no refractory gate. */
static int spiked_izh_dense(net_t *n, layer_t *L, int i) {
    const REAL ge = n->g_ampa[i] * L->decay_ampa + n->pend_e[i];
    const REAL gi = n->g_gaba[i] * L->decay_gaba + n->pend_i[i];
    n->pend_e[i] = 0;
    n->pend_i[i] = 0;
    const REAL V = n->v[i], U = n->u[i];
    const REAL total = ge * (L->f[7] - V) + gi * (L->f[9] - V) + n->i_ext[i];
    REAL v = V + n->dt * (K(0.04) * V * V + K(5.0) * V + K(140.0) - U + L->f[6] * total);
    REAL u = U + n->dt * (L->f[0] * (L->f[1] * v - U));
    n->g_ampa[i] = ge;
    n->g_gaba[i] = gi;
    n->last[i] += 1;
    int s = 0;
    if (v >= L->f[5]) {
        v = L->f[2];
        u += L->f[3];
        n->last[i] = 0;
        s = 1;
    }
    n->v[i] = v;
    n->u[i] = u;
    return s;
}

static int spiked_izh_cond(net_t *n, layer_t *L, int i) {
    if (n->semantics == SEM_DENSE) return spiked_izh_dense(n, L, i);
    /* TimeDrivenIzhikevic_Exponential_Decay.cpp:59-110 */
    const REAL V = n->v[i], U = n->u[i];
    REAL total = K(0.0);
    if (L->has_exc) total += n->g_ampa[i] * (L->f[7] - V);
    if (L->has_inh) total += n->g_gaba[i] * (L->f[9] - V);
    total += n->i_ext[i];
    REAL dv, du;
    if (n->last[i] > 0) {
        dv = K(0.04) * V * V + K(5.0) * V + K(140.0) - U + L->f[6] * total;
        du = L->f[0] * (L->f[1] * V - U);
    } else {
        dv = 0;
        du = 0;
    }
    n->v[i] += dv * n->dt;
    n->u[i] += du * n->dt;
    if (L->has_exc) n->g_ampa[i] *= L->decay_ampa;
    if (L->has_inh) n->g_gaba[i] *= L->decay_gaba;
    n->last[i] += 1;
    if (n->v[i] >= L->f[5]) {
        n->v[i] = L->f[2];
        n->u[i] += L->f[3];
        n->last[i] = 0;
        return 1;
    }
    return 0;
}

/* Current-based Izhikevich with classic RK4 over one step, synaptic current
 * plus Gaussian noise held constant over the step.  The reference registers
 * only forward Euler (L/ModelFactory/IntegrationMethodList.inc:9-12); this
 * model follows its Izhikevich equations, reset and LastSpike gating. */
/* Current-based Izhikevich right-hand side (config 1; the reference has only
 * the conductance/Euler form).  Written with explicit fused multiply-adds,
 * each rounded once, identically in the CUDA kernel:
 *   f = (fma(fma(0.04, v, 5), v, 140) - u) + I,   g = a * fma(b, v, -u). */
#ifdef REAL_IS_DOUBLE
#define FMA(x, y, z) fma((x), (y), (z))
#else
#define FMA(x, y, z) fmaf((x), (y), (z))
#endif
static REAL izh_f(REAL v, REAL u, REAL I) { return (FMA(FMA(K(0.04), v, K(5.0)), v, K(140.0)) - u) + I; }
static REAL izh_g(REAL a, REAL b, REAL v, REAL u) { return a * FMA(b, v, -u); }
static int spiked_izh_rk4(net_t *n, layer_t *L, int i, int t) {
    REAL a = L->f[0], b = L->f[1];
    REAL I = n->g_ampa[i] + n->i_ext[i];
    if (L->f[6] != (REAL)0) I = I + L->f[6] * gauss12(n->seed, i, t);
    n->g_ampa[i] = 0;
    if (n->last[i] > 0) {
        REAL h = n->dt, hh = K(0.5) * n->dt, h6 = n->dt / K(6.0);
        REAL v = n->v[i], u = n->u[i];
        /* classical RK4; stage combinations as fused multiply-adds */
        REAL k1v = izh_f(v, u, I), k1u = izh_g(a, b, v, u);
        REAL v2 = FMA(hh, k1v, v), u2 = FMA(hh, k1u, u);
        REAL k2v = izh_f(v2, u2, I), k2u = izh_g(a, b, v2, u2);
        REAL v3 = FMA(hh, k2v, v), u3 = FMA(hh, k2u, u);
        REAL k3v = izh_f(v3, u3, I), k3u = izh_g(a, b, v3, u3);
        REAL v4 = FMA(h, k3v, v), u4 = FMA(h, k3u, u);
        REAL k4v = izh_f(v4, u4, I), k4u = izh_g(a, b, v4, u4);
        n->v[i] = FMA(h6, FMA(K(2.0), k3v, FMA(K(2.0), k2v, k1v)) + k4v, v);
        n->u[i] = FMA(h6, FMA(K(2.0), k3u, FMA(K(2.0), k2u, k1u)) + k4u, u);
    }
    n->last[i] += 1;
    if (n->v[i] >= L->f[5]) {
        n->v[i] = L->f[2];
        n->u[i] += L->f[3];
        n->last[i] = 0;
        return 1;
    }
    return 0;
}

static int spiked_poisson(net_t *n, layer_t *L, int i, int t) {
    /* PoissonRate::UpdateState (PoissonRate.cpp:55-78), local neuron index */
    float dt_ms = n->dt_f;
    float rate = (float)L->f[0] + (float)n->rate[i] + (float)L->f[1] * (float)n->i_ext[i];
    rate = rate > 0.0f ? rate : 0.0f;
    float prob = rate * dt_ms * 0.001f;
    prob = prob < 1.0f ? prob : 1.0f;
    int s = 0;
    if (hash_uniform01(i - L->start, t) < prob) {
        n->last[i] = 0;
        s = 1;
    } else {
        n->last[i] += 1;
    }
    n->rate[i] = 0;
    return s;
}

static int spiked(net_t *n, layer_t *L, int i, int t) {
    switch (L->model) {
    case M_LIF_VJ: return spiked_lif(n, L, i);
    case M_IZH_COND: return spiked_izh_cond(n, L, i);
    case M_IZH_RK4: return spiked_izh_rk4(n, L, i, t);
    case M_INPUT_SPIKE:
    case M_INPUT_CURRENT: return 0; /* event-driven: no time-driven update */
    default: return spiked_poisson(n, L, i, t);
    }
}

/* One step.  With threads > 1 the arrivals of different targets, the neuron
 * updates and the post-synaptic passes of different spiking neurons run in
 * parallel; each touches only its own neuron and synapses, so the results
 * are identical to the serial order. */
static void schedule_spike(net_t *n, int i, int t) {
    for (int64_t q = n->out_ptr[i]; q < n->out_ptr[i + 1]; ++q) {
        int64_t p = n->out_pos[q];
        if (n->csc_type[p] == SYN_CURRENT) continue; /* carries currents only */
        vpush(&n->bucket[(t + n->csc_delay[p]) % n->ring], p);
    }
}

static void step(net_t *n, int t) {
    for (int64_t k = 0; k < n->cur_t.n; ++k)
        if (n->cur_t.v[k] == t) n->i_ext[n->cur_id.v[k]] = n->cur_v[k];
    /* latched external currents arriving at t (insertion order), then the
     * total of every touched target */
    {
        int any = 0;
        for (int64_t k = 0; k < n->lat_t.n; ++k)
            if (n->lat_t.v[k] == t) {
                n->latch[n->lat_p.v[k]] = n->lat_v[k];
                any = 1;
            }
        if (any)
            for (int64_t k = 0; k < n->lat_t.n; ++k) {
                if (n->lat_t.v[k] != t) continue;
                int j = n->csc_tgt[n->lat_p.v[k]];
                float total = 0.0f;
                for (int64_t p = n->csc_ptr[j]; p < n->csc_ptr[j + 1]; ++p)
                    if (n->csc_type[p] == SYN_CURRENT) total += (float)n->latch[p];
                n->i_ext[j] = (REAL)total;
            }
    }
    /* external spikes at t: recorded and scheduled like a spike of the
     * update, before it (PROPOGATEDSPIKE outranks TIMEEVENT) */
    for (int64_t k = 0; k < n->ext_t.n; ++k)
        if (n->ext_t.v[k] == t) {
            int i = (int)n->ext_id.v[k];
            vpush(&n->spk, ((int64_t)t << 32) | (int64_t)(uint32_t)i);
            schedule_spike(n, i, t);
        }
    /* 1. arrivals due at t, per target in CSC order */
    vec64_t *b = &n->bucket[t % n->ring];
    qsort(b->v, (size_t)b->n, sizeof(int64_t), cmp_i64);
    n->n_events += b->n;
    if (n->threads <= 1 || n->log_events || b->n < 4096) {
        for (int64_t e = 0; e < b->n; ++e) deliver(n, b->v[e], t);
    } else {
        if (b->n + 1 > n->seg_cap) {
            n->seg_cap = 2 * (b->n + 1);
            n->seg = (int64_t *)realloc(n->seg, (size_t)n->seg_cap * sizeof(int64_t));
        }
        int64_t ns = 0;
        for (int64_t e = 0; e < b->n; ++e)
            if (e == 0 || n->csc_tgt[b->v[e]] != n->csc_tgt[b->v[e - 1]]) n->seg[ns++] = e;
        n->seg[ns] = b->n;
#pragma omp parallel for schedule(dynamic, 64) num_threads(n->threads)
        for (int64_t g = 0; g < ns; ++g)
            for (int64_t e = n->seg[g]; e < n->seg[g + 1]; ++e) deliver(n, b->v[e], t);
    }
    b->n = 0;
    /* 2. model updates in layer creation order */
    for (int l = 0; l < n->n_layers; ++l) {
        layer_t *L = &n->layers[l];
        const int i0 = L->start, i1 = L->start + L->count;
#pragma omp parallel for schedule(static) num_threads(n->threads) if (n->threads > 1 && L->count >= 4096)
        for (int i = i0; i < i1; ++i) n->fired[i] = (unsigned char)spiked(n, L, i, t);
        int64_t first = n->spk.n;
        for (int i = i0; i < i1; ++i) {
            if (!n->fired[i]) continue;
            vpush(&n->spk, ((int64_t)t << 32) | (int64_t)(uint32_t)i);
            schedule_spike(n, i, t);
        }
        const int64_t last = n->spk.n;
#pragma omp parallel for schedule(dynamic, 4) num_threads(n->threads) if (n->threads > 1 && last - first > 8)
        for (int64_t k = first; k < last; ++k) stdp_post(n, (int)(n->spk.v[k] & 0xFFFFFFFF), t);
    }
    if (n->n_trace > 0) {
        if (n->trace_n + n->n_trace > n->trace_cap) {
            n->trace_cap = (n->trace_cap + n->n_trace) * 2;
            n->trace = (REAL *)realloc(n->trace, (size_t)n->trace_cap * sizeof(REAL));
        }
        for (int k = 0; k < n->n_trace; ++k) n->trace[n->trace_n++] = n->v[n->trace_ids[k]];
    }
}

void ORC(set_threads)(void *hp, int threads) { ((net_t *)hp)->threads = threads > 0 ? threads : 1; }

/* Simulation::RunSimulationStep(steps) as seen through _core.Simulation.run:
 * N+1 updates on the first call, N afterwards. */
int ORC(run)(void *hp, int steps) {
    net_t *n = (net_t *)hp;
    if (steps <= 0) return 1;
    int count = n->ran ? steps : steps + 1;
    for (int k = 0; k < count; ++k) step(n, n->next_t + k);
    n->next_t += count;
    n->ran = 1;
    return 0;
}

int ORC(next_time)(void *hp) { return ((net_t *)hp)->next_t; }
int64_t ORC(num_spikes)(void *hp) { return ((net_t *)hp)->spk.n; }
int64_t ORC(num_events)(void *hp) { return ((net_t *)hp)->n_events; }
int64_t ORC(num_synapses)(void *hp) { return ((net_t *)hp)->n_syn; }

void ORC(get_spikes)(void *hp, int *t, int *id) {
    net_t *n = (net_t *)hp;
    for (int64_t k = 0; k < n->spk.n; ++k) {
        t[k] = (int)(n->spk.v[k] >> 32);
        id[k] = (int)(n->spk.v[k] & 0xFFFFFFFF);
    }
}

/* field: 0 v, 1 u, 2 g_ampa (also the synaptic-current accumulator), 3 g_gaba,
 * 4 i_ext, 5 rate, 6 last_spike */
void ORC(get_state)(void *hp, int field, double *out) {
    net_t *n = (net_t *)hp;
    for (int i = 0; i < n->n_neurons; ++i) {
        switch (field) {
        case 0: out[i] = (double)n->v[i]; break;
        case 1: out[i] = (double)n->u[i]; break;
        case 2: out[i] = (double)n->g_ampa[i]; break;
        case 3: out[i] = (double)n->g_gaba[i]; break;
        case 4: out[i] = (double)n->i_ext[i]; break;
        case 5: out[i] = (double)n->rate[i]; break;
        default: out[i] = (double)n->last[i]; break;
        }
    }
}

void ORC(set_state)(void *hp, int field, const double *in) {
    net_t *n = (net_t *)hp;
    for (int i = 0; i < n->n_neurons; ++i) {
        switch (field) {
        case 0: n->v[i] = (REAL)in[i]; break;
        case 1: n->u[i] = (REAL)in[i]; break;
        case 4: n->i_ext[i] = (REAL)in[i]; break;
        default: break;
        }
    }
}

/* weights and STDP state in original connection order */
void ORC(get_weights)(void *hp, double *w, double *apre, double *apost, int *last) {
    net_t *n = (net_t *)hp;
    for (int64_t p = 0; p < n->n_syn; ++p) {
        int64_t s = n->csc_orig[p];
        if (w) w[s] = (double)n->csc_w[p];
        if (apre) apre[s] = (double)n->apre[p];
        if (apost) apost[s] = (double)n->apost[p];
        if (last) last[s] = n->slast[p];
    }
}

void ORC(set_trace)(void *hp, int count, const int *ids) {
    net_t *n = (net_t *)hp;
    free(n->trace_ids);
    n->n_trace = count;
    n->trace_ids = (int *)malloc((size_t)(count > 0 ? count : 1) * sizeof(int));
    for (int k = 0; k < count; ++k) n->trace_ids[k] = ids[k];
    n->trace_n = 0;
}

int64_t ORC(get_traces)(void *hp, double *out) {
    net_t *n = (net_t *)hp;
    if (out)
        for (int64_t k = 0; k < n->trace_n; ++k) out[k] = (double)n->trace[k];
    return n->trace_n;
}

void ORC(set_event_log)(void *hp, int on) { ((net_t *)hp)->log_events = on; }
int64_t ORC(num_logged_events)(void *hp) { return ((net_t *)hp)->ev_t.n; }

/* delivered events as (time, original connection index, delivered weight) */
void ORC(get_events)(void *hp, int *t, int64_t *conn, double *w) {
    net_t *n = (net_t *)hp;
    for (int64_t k = 0; k < n->ev_t.n; ++k) {
        t[k] = (int)n->ev_t.v[k];
        conn[k] = n->csc_orig[n->ev_pos.v[k]];
        w[k] = (double)n->ev_w[k];
    }
}

/* Neurons [first, first + count) back to their initial state, with the
 * arrivals pending for them dropped; synapses and time are kept (the reset
 * of one dense subnetwork: DenseSubnetworkModel::Reset,
 * src/native/gpu/src/simulation_dense/DenseSubnetworkModel.cpp:173-183). */
void ORC(reset_neurons)(void *hp, int first, int count) {
    net_t *n = (net_t *)hp;
    for (int i = first; i < first + count; ++i) {
        n->g_ampa[i] = n->g_gaba[i] = n->rate[i] = n->pend_e[i] = n->pend_i[i] = 0;
        n->u[i] = 0;
        n->fired[i] = 0;
        init_neuron(n, &n->layers[n->layer_of[i]], i);
    }
    for (int r = 0; r < n->ring; ++r) {
        vec64_t *b = &n->bucket[r];
        int64_t k = 0;
        for (int64_t q = 0; q < b->n; ++q) {
            const int j = n->csc_tgt[b->v[q]];
            if (j < first || j >= first + count) b->v[k++] = b->v[q];
        }
        b->n = k;
    }
}

void ORC(set_decay_table)(void *hp, int64_t len, const float *vals) {
    net_t *n = (net_t *)hp;
    free(n->dtab_ext);
    n->dtab_ext = NULL;
    n->dtab_ext_len = 0;
    if (len <= 0 || !vals) return;
    size_t count = (size_t)(n->n_rules > 0 ? n->n_rules : 1) * 2 * (size_t)len;
    n->dtab_ext = (float *)malloc(count * sizeof(float));
    memcpy(n->dtab_ext, vals, count * sizeof(float));
    n->dtab_ext_len = len;
}

void ORC(add_external_spike)(void *hp, int t, int id) {
    net_t *n = (net_t *)hp;
    vpush(&n->ext_t, t);
    vpush(&n->ext_id, id);
}

void ORC(add_external_current)(void *hp, int t, int id, double value) {
    net_t *n = (net_t *)hp;
    for (int64_t q = n->out_ptr[id]; q < n->out_ptr[id + 1]; ++q) {
        int64_t p = n->out_pos[q];
        if (n->csc_type[p] != SYN_CURRENT) continue;
        vpush(&n->lat_t, t + n->csc_delay[p]);
        vpush(&n->lat_p, p);
        if (n->lat_t.n > n->lat_vcap) {
            n->lat_vcap = n->lat_t.cap;
            n->lat_v = (REAL *)realloc(n->lat_v, (size_t)n->lat_vcap * sizeof(REAL));
        }
        n->lat_v[n->lat_t.n - 1] = (REAL)value;
    }
}

void ORC(add_current)(void *hp, int t, int id, double value) {
    net_t *n = (net_t *)hp;
    vpush(&n->cur_t, t);
    vpush(&n->cur_id, id);
    if (n->cur_t.n > n->cur_vcap) {
        n->cur_vcap = n->cur_t.cap;
        n->cur_v = (REAL *)realloc(n->cur_v, (size_t)n->cur_vcap * sizeof(REAL));
    }
    n->cur_v[n->cur_t.n - 1] = (REAL)value;
}

/* ------------------------------------------------------------------------
 * Dense all-to-all populations (the GPU dense delivery engine's semantics):
 * B instances x N voltage-jump LIF neurons sharing W (N x N, row = pre).
 * Step t: a = sum over spiking pre i (ascending) of W[i][j], plus the drive
 * weight when the delay-1 PoissonRate source (hash index b*N+j) fired at t-1;
 * if not refractory V += a; then the legacy Euler update
 * (TimeDrivenLIF_Voltage_jump.cpp:49-86).  The first run performs N+1 updates.
 * ------------------------------------------------------------------------ */
typedef struct {
    int B, N, t_ref, next_t, ran, threads;
    REAL v_rest, tau, v_th, r, v_reset, i_ext, dt, drive_w;
    float drive_p;
    const float *w; /* borrowed: N x N */
    REAL *v;
    int *last;
    unsigned char *s, *s_next;
    vec64_t counts;
} dense_t;

void *ORC(dense_create)(int B, int N, const float *w, const float *f, const int *ip, float drive_rate_hz,
                        float drive_w, float dt) {
    dense_t *d = (dense_t *)calloc(1, sizeof(dense_t));
    d->B = B;
    d->N = N;
    d->w = w;
    d->v_rest = (REAL)f[0];
    d->tau = (REAL)f[1];
    d->v_th = (REAL)f[2];
    d->r = (REAL)f[3];
    d->v_reset = (REAL)f[4] + (REAL)f[5];
    d->i_ext = (REAL)f[6];
    d->t_ref = ip[0];
    d->dt = (REAL)dt;
    d->drive_w = (REAL)drive_w;
    float rate = drive_rate_hz > 0.0f ? drive_rate_hz : 0.0f;
    float p = rate * dt * 0.001f;
    d->drive_p = p < 1.0f ? p : 1.0f;
    size_t tot = (size_t)B * N;
    d->v = (REAL *)malloc(tot * sizeof(REAL));
    d->last = (int *)malloc(tot * sizeof(int));
    d->s = (unsigned char *)calloc(tot, 1);
    d->s_next = (unsigned char *)calloc(tot, 1);
    for (size_t i = 0; i < tot; ++i) {
        d->v[i] = d->v_reset;
        d->last[i] = 10000;
    }
    return d;
}

void ORC(dense_destroy)(void *hp) {
    dense_t *d = (dense_t *)hp;
    if (!d) return;
    free(d->v);
    free(d->last);
    free(d->s);
    free(d->s_next);
    free(d->counts.v);
    free(d);
}

/* Instances are independent (each its own V, LastSpike and spike row), so
 * they run on OpenMP threads; every instance's arithmetic is the same
 * sequential sum as on one thread. */
static void dense_step(dense_t *d, int t) {
    const int N = d->N;
    int64_t nspk = 0;
#pragma omp parallel num_threads(d->threads > 0 ? d->threads : 1) reduction(+ : nspk)
    {
    REAL *col = (REAL *)malloc((size_t)N * sizeof(REAL));
#pragma omp for schedule(static)
    for (int b = 0; b < d->B; ++b) {
        const unsigned char *sb = d->s + (size_t)b * N;
        for (int j = 0; j < N; ++j) col[j] = K(0.0);
        for (int i = 0; i < N; ++i) {
            if (!sb[i]) continue;
            const float *row = d->w + (size_t)i * N;
            for (int j = 0; j < N; ++j) col[j] = col[j] + (REAL)row[j];
        }
        for (int j = 0; j < N; ++j) {
            const size_t idx = (size_t)b * N + j;
            REAL a = col[j];
            if (t >= 1 && hash_uniform01((int)idx, t - 1) < d->drive_p) a = a + d->drive_w;
            REAL vv = d->v[idx];
            int ls = d->last[idx];
            if (ls > d->t_ref) vv = vv + a;
            REAL cur = K(0.0);
            cur = cur + d->r * d->i_ext / d->tau;
            REAL aux = (ls > d->t_ref) ? cur + (d->v_rest - vv) / d->tau : K(0.0);
            vv = vv + aux * d->dt;
            ls += 1;
            unsigned char spk = 0;
            if (vv > d->v_th) {
                vv = d->v_reset;
                ls = 0;
                spk = 1;
                ++nspk;
            }
            d->v[idx] = vv;
            d->last[idx] = ls;
            d->s_next[idx] = spk;
        }
    }
    free(col);
    }
    unsigned char *tmp = d->s;
    d->s = d->s_next;
    d->s_next = tmp;
    vpush(&d->counts, nspk);
}

int ORC(dense_run)(void *hp, int steps) {
    dense_t *d = (dense_t *)hp;
    if (steps <= 0) return 1;
    int count = d->ran ? steps : steps + 1;
    for (int k = 0; k < count; ++k) dense_step(d, d->next_t + k);
    d->next_t += count;
    d->ran = 1;
    return 0;
}

void ORC(dense_set_threads)(void *hp, int threads) { ((dense_t *)hp)->threads = threads; }
int64_t ORC(dense_num_steps)(void *hp) { return ((dense_t *)hp)->counts.n; }
void ORC(dense_counts)(void *hp, int *out) {
    dense_t *d = (dense_t *)hp;
    for (int64_t k = 0; k < d->counts.n; ++k) out[k] = (int)d->counts.v[k];
}
void ORC(dense_state)(void *hp, double *v, int *last, unsigned char *s) {
    dense_t *d = (dense_t *)hp;
    size_t tot = (size_t)d->B * d->N;
    for (size_t i = 0; i < tot; ++i) {
        if (v) v[i] = (double)d->v[i];
        if (last) last[i] = d->last[i];
        if (s) s[i] = d->s[i];
    }
}

/* standalone helpers for known-answer tests */
float ORC(poisson_hash)(int neuron_index, int time_step) { return hash_uniform01(neuron_index, time_step); }
double ORC(gauss12)(uint64_t seed, int neuron, int t) { return (double)gauss12(seed, neuron, t); }
