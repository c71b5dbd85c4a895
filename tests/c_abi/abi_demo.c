/* A C host driving the engine through include/nbg.h only, as the reference's
 * C++ host would (its NativeSimulation, python/bindings/neuronbridge_core.cpp
 * :152-300).  Network: 200 voltage-jump LIF neurons (output layer), each
 * driven 1:1 by a PoissonRate source at 4 kHz (delay 1) and by 20 recurrent
 * excitatory synapses (delay 5, deterministic pattern).  Prints one line:
 * "status <create> <run> spikes <n> events <m> first <t> <id>".
 * Test infrastructure for tests/test_c_abi.py. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nbg.h"

#define N 200
#define FAN 20

int main(int argc, char **argv) {
    const int steps = argc > 1 ? atoi(argv[1]) : 500;
    nbg_layer_desc layers[2];
    memset(layers, 0, sizeof layers);
    layers[0].model = NBG_MODEL_LIF_VJ;
    layers[0].count = N;
    layers[0].f[0] = -65.0f; /* V_rest */
    layers[0].f[1] = 20.0f;  /* tau */
    layers[0].f[2] = -50.0f; /* V_th */
    layers[0].f[3] = 1.0f;   /* R */
    layers[0].f[4] = -65.0f; /* V_reset */
    layers[0].ip[0] = 20;    /* t_ref (steps) */
    layers[0].output = 1;
    layers[1].model = NBG_MODEL_POISSON;
    layers[1].count = N;
    layers[1].f[0] = 4000.0f; /* rate_bias_hz */
    const int64_t m = (int64_t)N + (int64_t)N * FAN;
    int32_t *src = malloc(m * sizeof(int32_t)), *tgt = malloc(m * sizeof(int32_t));
    int32_t *type = malloc(m * sizeof(int32_t)), *delay = malloc(m * sizeof(int32_t));
    int32_t *rule = malloc(m * sizeof(int32_t));
    float *w = malloc(m * sizeof(float)), *wmax = malloc(m * sizeof(float));
    int64_t c = 0;
    for (int i = 0; i < N; ++i, ++c) { /* Poisson drive */
        src[c] = N + i; tgt[c] = i; type[c] = 0; w[c] = 2.0f; wmax[c] = 2.0f; delay[c] = 1; rule[c] = -1;
    }
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < FAN; ++k, ++c) { /* recurrent */
            src[c] = i; tgt[c] = (i * 7 + k * 13 + 1) % N; type[c] = (k % 5 == 0); w[c] = 0.8f; wmax[c] = 0.8f;
            delay[c] = 5; rule[c] = -1;
        }
    nbg_net_desc d;
    memset(&d, 0, sizeof d);
    d.n_layers = 2; d.layers = layers; d.n_conn = m;
    d.source = src; d.target = tgt; d.type = type; d.weight = w; d.max_weight = wmax; d.delay = delay; d.rule = rule;
    d.dt_ms = 0.1f; d.semantics = NBG_SEM_LEGACY_CPU;
    nbg_options o;
    nbg_default_options(&o);
    nbg_engine *e = NULL;
    const nbg_status sc = nbg_create(&d, &o, &e);
    if (sc != NBG_OK) {
        printf("status %d -1 error %s\n", (int)sc, nbg_last_error());
        return 0;
    }
    const nbg_status sr = nbg_run(e, steps);
    int64_t ns = 0, ne = 0;
    nbg_num_spikes(e, &ns);
    nbg_num_events(e, &ne);
    int32_t t0 = -1, i0 = -1;
    if (ns > 0) {
        int32_t *ts = malloc(ns * sizeof(int32_t)), *ids = malloc(ns * sizeof(int32_t));
        nbg_get_spikes(e, ts, ids, ns);
        t0 = ts[0];
        i0 = ids[0];
        free(ts);
        free(ids);
    }
    printf("status %d %d spikes %lld events %lld first %d %d\n", (int)sc, (int)sr, (long long)ns, (long long)ne,
           t0, i0);
    nbg_destroy(e);
    free(src); free(tgt); free(type); free(delay); free(rule); free(w); free(wmax);
    return 0;
}
