// nbg_engine.cu -- GB300 (sm_103a) step engine for NeuronBridge's time-driven
// spiking networks: network compile on the host, one kernel launch per block
// of steps on the device, C ABI in include/nbg.h.
//
// Execution model (owner computes by target neuron):
//   * Every synapse has a bit in a per-step "arrival mask" ring:
//       mask[slot][woff[j] + p/32] bit p%32   for in-synapse p of target j
//     (p is the synapse's rank in j's CSC list, sorted by source id).
//   * k_update: one thread per target neuron advances it `B` steps.  At each
//     step it reads its own mask words for slot t % D, applies the marked
//     arrivals in ascending CSC order (the canonical order of the oracle),
//     runs the pre-synaptic STDP hook of each plastic arrival, integrates the
//     neuron, and on a spike runs the post-synaptic STDP pass over its own
//     CSC list and propagates the spike: the warp strides over the spiking
//     neuron's out-synapses (CSR by source) and sets each one's bit in slot
//     (t + delay) % D with a fire-and-forget atomicOr.  OR is commutative, so
//     the mask -- and therefore every later sum -- does not depend on the
//     order in which threads run: results are bit-exact and reproducible
//     without floating-point atomics.
//   * Temporal blocking: a spike at t reaches its targets at t + d >= t + dmin,
//     so B <= dmin steps can be advanced per target with no global exchange.
//     The ring has D = dmax + Bmax slots, so a mark made during a block
//     (for a step >= the block's end) never lands in a slot the block is
//     still draining: the marks of a launch are read only by later launches.
//
// Reference counterparts (paths inside the reference project):
//   LIF update     .../NeuralModel/src/TimeDriven/TimeDrivenLIF_Voltage_jump.cpp:49-113
//                  .../Intergration/inc/FixStep/ForwardEulerMethod.h:29-55
//   Izhikevich     .../TimeDrivenIzhikevic_Exponential_Decay.cpp:59-131
//   Poisson        .../TimeDriven/PoissonRate.cpp:12-22,55-78
//   delivery       .../Event/src/Spike/PropogatedSpikeGroup.cpp:33-72,
//                  .../Event/src/Spike/TimeDrivenInternalSpike.cpp:37-145,
//                  src/native/gpu/src/gpu_runtime/GpuPropagationRuntime.cu:150-266
//   STDP           .../LearningRule/src/Rule/STDP.cpp:19-61,
//                  .../LearningRule/src/State/STDP_State.cpp:17-26
//   dense profile  src/native/gpu/include/dense_subnetwork/model/
//                  DenseLifVoltageJumpDeviceUpdate.cuh:10-51
//
// Built with -fmad=false: every float operation rounds once, as in the
// reference's scalar C++ and the oracle (-ffp-contract=off).

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <memory>
#include <thread>
#include <type_traits>
#include <utility>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <unordered_set>
#include <vector>

#include "nbg.h"
#include "nbg_common.cuh"

namespace {
thread_local std::string g_err;
}

nbg_status nbg_fail(nbg_status code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

namespace {

inline nbg_status fail(nbg_status code, const char *msg) { return nbg_fail(code, "%s", msg); }
template <typename... A>
inline nbg_status fail(nbg_status code, const char *fmt, A... a) {
    return nbg_fail(code, fmt, a...);
}

constexpr int kMaxBlockSteps = 32;
constexpr int kErrOverflow = 1;
constexpr int kErrEventLog = 2;

// ---------------------------------------------------------------- device data

struct LayerDev {
    int model, start, count, has_exc, has_inh;
    int record;    // output layer: spikes go to the raster
    int generator; // source-free PoissonRate: targets evaluate its spikes inline
    float f[NBG_NFP];
    int ip[NBG_NIP];
    float decay_exc, decay_inh; // IZH_COND conductance decay per step
    float alpha;                // DENSE LIF: dt / tau
};

// Synapse records, in CSC order.  A plastic network keeps every field an
// arrival touches in one 32-byte record -- one DRAM sector per arrival, read
// by two 16-byte loads and written back by one -- instead of one sector in
// each of six arrays.  The rule's two jump sizes ride along in the record, so
// an arrival has no further dependent load besides its decay factors.  A static network keeps weight and meta in 8 bytes.
//   meta: bit 0 synapse type (1 = subtract), bits 1..7 learning rule + 1
struct alignas(32) SynRec {
    float w, apre, apost; // weight, the pre- and post-synaptic traces
    int last;             // step of the last trace update
    unsigned int meta;
    float wmax;           // upper weight bound of the rule's clamp
    float a_pre, a_post;  // the rule's Max_LTD and Max_LTP (its pre and post jumps)
};
struct alignas(8) SynStatic {
    float w;
    unsigned int meta;
};

struct NetDev {
    int N, D, Wt, n_layers, semantics;
    float dt;
    unsigned long long seed;
    const unsigned short *pop;
    const LayerDev *layers;
    float *v, *u, *gexc, *ginh, *iext;
    int *last;
    const int *csc_ptr, *woff;
    // synapses in CSC order: SynRec (plastic networks) or SynStatic (static
    // ones); exactly one of the two is set
    SynRec *rec;
    SynStatic *wst;
    const float2 *dtab; // [rule][dtab_len] {LTP factor, LTD factor} per step gap
    int dtab_len;
    int sdtab_len; // entries of rule 0's table copied into shared memory per CTA (0: none)
    unsigned int *mask;
    unsigned int *wsum; // per slot: one bit per mask word, set while that word is non-zero
    int Ws;             // summary words per slot (ceil(Wt / 32) + 1 padding word)
    const int *out_ptr;
    // out lists (CSR by source): packed (mask bit << out_dbits | delay -
    // out_dmin) when that fits 32 bits, else bit and delay in two arrays
    const unsigned int *out_pk;
    int out_dbits, out_dmin;
    const unsigned int *out_bit;
    const unsigned short *out_delay;
    // in-synapses from generator layers, per target, sorted by CSC rank
    const int *gen_ptr, *gen_pos, *gen_src;
    const unsigned short *gen_delay;
    int *out_ids, *out_t; // raster of output-layer spikes (unordered; sorted on the host)
    unsigned int *cursor;
    long long out_cap;
    int *err;
    int *run_t0;
    const int *trace_slot;
    float *trace;
    int ntrace;
    int *ev_t, *ev_pos;
    float *ev_w;
    unsigned long long *ev_cursor;
    long long ev_cap;
    unsigned long long *n_events;
    // external spikes of the current run call: ext_ids[ext_ptr[k] .. ext_ptr[k+1])
    // spike at call step k (null until the first nbg_add_external_spikes)
    const int *ext_ptr, *ext_ids;
    // thread -> neuron: the first N_upd threads update upd_ids[thread] (the
    // thread's own index when null); generator neurons gen_ids[0 .. N_gen)
    // follow in trailing CTAs, kGenPerThread per thread
    int N_upd, N_gen;
    const int *upd_ids, *gen_ids;
};

__device__ __forceinline__ float hash_uniform01(int neuron_index, int time_step) {
    return nbg_hash_uniform01(neuron_index, time_step);
}

// Spike of generator neuron k at step ts (PoissonRate::UpdateState with no
// inputs: the rate is bias + gain * I_ext, identical to update_neuron below).
__device__ __forceinline__ bool generator_fired(const NetDev &n, int k, int ts);

// Noise current: Irwin-Hall sum of twelve 16-bit uniforms (u + 1/2) / 2^16
// minus 6, summed in integers and converted once (exact in float).  Bits
// from the PCG RXS-M-XS 32-bit output permutation used as a hash (Jarzynski
// and Olano, "Hash Functions for GPU Rendering", JCGT 2020): a per-neuron key
// from (seed, neuron), a per-step key from (neuron key, step), then six
// 32-bit words of two uniforms each.  Identical arithmetic in the oracle.
__device__ __forceinline__ unsigned int pcg_hash(unsigned int v) {
    const unsigned int state = v * 747796405u + 2891336453u;
    const unsigned int word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
__device__ __forceinline__ unsigned int noise_key(unsigned long long seed, int neuron) {
    return pcg_hash((unsigned int)neuron ^ pcg_hash((unsigned int)seed ^ (unsigned int)(seed >> 32)));
}
__device__ __forceinline__ float gauss12(unsigned int key, int t) {
    const unsigned int tk = pcg_hash(key ^ ((unsigned int)t * 0x9E3779B9u));
    int m = 0;
#pragma unroll
    for (unsigned int k = 0; k < 6; ++k) {
        const unsigned int h = pcg_hash(tk + k);
        m += (int)(h & 0xFFFFu) + (int)(h >> 16);
    }
    return (float)(m + 6 - 6 * 65536) * (1.0f / 65536.0f);
}

// Current-based Izhikevich right-hand side with explicit fused multiply-adds
// (each rounded once; the oracle writes the same fmaf calls):
//   f = (fma(fma(0.04, v, 5), v, 140) - u) + I,   g = a * fma(b, v, -u)
__device__ __forceinline__ float izh_f(float v, float u, float I) {
    return (__fmaf_rn(__fmaf_rn(0.04f, v, 5.0f), v, 140.0f) - u) + I;
}
__device__ __forceinline__ float izh_g(float a, float b, float v, float u) { return a * __fmaf_rn(b, v, -u); }

struct NeuronRegs {
    float v, u, gexc, ginh, iext;
    float lif_cur; // legacy LIF: 0 + R * I_ext / tau, constant over a launch (I_ext changes between launches)
    int last;
};

// Per-thread copy of the parameters its neuron's model uses (a compact
// subset of LayerDev, to keep the update kernel's register count low).
//   LIF_VJ   p: V_rest tau V_th R V_reset alpha        ip: t_ref
//   IZH_COND p: a b c d V_th R E_ampa E_gaba dexc dinh  flags: has_exc has_inh
//   IZH_RK4  p: a b c d V_th sigma
//   POISSON  p: rate_bias gain                         ip: layer start
struct Model {
    int model, ip, flags, record;
    float p[10];
};

__device__ __forceinline__ Model load_model(const LayerDev &L) {
    Model m;
    m.model = L.model;
    m.record = L.record;
    m.ip = 0;
    m.flags = (L.has_exc ? 1 : 0) | (L.has_inh ? 2 : 0);
#pragma unroll
    for (int k = 0; k < 10; ++k) m.p[k] = 0.0f;
    switch (L.model) {
    case NBG_MODEL_LIF_VJ:
        m.p[0] = L.f[0]; m.p[1] = L.f[1]; m.p[2] = L.f[2]; m.p[3] = L.f[3]; m.p[4] = L.f[4]; m.p[5] = L.alpha;
        m.ip = L.ip[0];
        break;
    case NBG_MODEL_IZH_COND:
        m.p[0] = L.f[0]; m.p[1] = L.f[1]; m.p[2] = L.f[2]; m.p[3] = L.f[3]; m.p[4] = L.f[5]; m.p[5] = L.f[6];
        m.p[6] = L.f[7]; m.p[7] = L.f[9]; m.p[8] = L.decay_exc; m.p[9] = L.decay_inh;
        break;
    case NBG_MODEL_IZH_RK4:
        m.p[0] = L.f[0]; m.p[1] = L.f[1]; m.p[2] = L.f[2]; m.p[3] = L.f[3]; m.p[4] = L.f[5]; m.p[5] = L.f[6];
        break;
    default:
        m.p[0] = L.f[0]; m.p[1] = L.f[1];
        m.ip = L.start;
        break;
    }
    return m;
}

// Compile-time network profile of an update-kernel instance: the neuron
// models that may occur (bit m = model m) and whether synapses learn
// (1 yes, 0 no, -1 decided per launch from the STDP arrays).  With one model
// the per-neuron dispatch folds away; without learning the STDP loads and
// the post-synaptic pass are not compiled.
template <unsigned kModels, int kPlastic>
struct Spec {
    static constexpr bool has(int m) { return (kModels >> m) & 1u; }
    // resident 256-thread CTAs per SM the register budget is sized for: the
    // static instances fit in 64 registers, which matters when a large
    // network runs in several waves
    static constexpr int min_blocks = kPlastic == 0 ? 4 : 3;
    static constexpr int single() {
        return (kModels != 0u && (kModels & (kModels - 1u)) == 0u) ? __builtin_ctz(kModels) : -1;
    }
    __device__ static int model(int m) { return single() >= 0 ? single() : m; }
    __device__ static bool plastic(const NetDev &n) { return kPlastic < 0 ? n.rec != nullptr : kPlastic > 0; }
    // Shape of the arrival drain.  Deep: one mask word per step, three steps
    // ahead, for networks whose neurons receive a few arrivals per hundred
    // steps (the current-based Izhikevich + STDP profile).  Wide: every
    // flagged word one step ahead and arrivals loaded several at a time, for
    // networks with arrivals at most steps (Poisson-driven static LIF).
    static constexpr bool deep = kPlastic > 0;
};
constexpr unsigned kAllModels = 0x3fu;
using GenericSpec = Spec<kAllModels, -1>;

__device__ __forceinline__ float clamp_w(float w, float wmax) {
    if (w < 0.0f) return 0.0f;
    if (w > wmax) return wmax;
    return w;
}

// One synapse as loaded for an arrival or a post-synaptic pass.
struct Syn {
    float w, apre, apost, wmax, a_pre, a_post;
    int last;
    unsigned int meta;
};

// A plastic synapse record from its two 16-byte halves.
__device__ __forceinline__ Syn syn_decode(const uint4 a, const uint4 b) {
    Syn y;
    y.w = __uint_as_float(a.x);
    y.apre = __uint_as_float(a.y);
    y.apost = __uint_as_float(a.z);
    y.last = (int)a.w;
    y.meta = b.x;
    y.wmax = __uint_as_float(b.y);
    y.a_pre = __uint_as_float(b.z);
    y.a_post = __uint_as_float(b.w);
    return y;
}

// Load synapse s: the whole 32-byte record of a plastic network (two 16-byte
// loads of one sector, issued together), or the 8-byte static record.
template <class S>
__device__ __forceinline__ Syn load_syn(const NetDev &n, int s) {
    Syn y;
    if (S::plastic(n)) {
        y = syn_decode(reinterpret_cast<const uint4 *>(n.rec + s)[0], reinterpret_cast<const uint4 *>(n.rec + s)[1]);
    } else {
        const uint2 a = reinterpret_cast<const uint2 *>(n.wst)[s];
        y.w = __uint_as_float(a.x);
        y.meta = a.y;
        y.apre = y.apost = y.wmax = y.a_pre = y.a_post = 0.0f;
        y.last = 0;
    }
    return y;
}

// Request synapse s's record ahead of its load (no register, no wait).  The
// later load finds the line in L2 rather than in this SM's L1 (measured: about
// 750 cycles instead of about 1,100 from DRAM, not the 40 of an L1 hit).
template <class S>
__device__ __forceinline__ void prefetch_syn(const NetDev &n, int s) {
    const void *p = S::plastic(n) ? (const void *)(n.rec + s) : (const void *)(n.wst + s);
    asm volatile("prefetch.global.L1 [%0];" ::"l"(__cvta_generic_to_global(p)));
}

// Decay factors {LTP, LTD} of rule `rule` for a gap of `gap` steps; gaps past
// the table decay to 0 (the table runs until expf underflows).
// The first entries of rule 0's decay table, copied into each CTA's shared
// memory at the start of a launch (the table does not change within a run
// call): most gaps are short, so most lookups leave the L2 round trip out
// of the arrival's dependent chain.
extern __shared__ float2 s_dtab[];
constexpr int kSharedDecayEntries = 4096; // 32 KiB

__device__ __forceinline__ float2 decay_pair(const NetDev &n, int rule, int gap) {
    if (rule == 0 && gap < n.sdtab_len) return s_dtab[gap];
    return gap < n.dtab_len ? n.dtab[(size_t)rule * n.dtab_len + gap] : make_float2(0.0f, 0.0f);
}

// Pair STDP (L/LearningRule/src/Rule/STDP.cpp:19-61, State/STDP_State.cpp:
// 17-26): decay both traces from the host table by the integer step gap
// (STDP_State::SetUpdate), then the pre (Apre += 1, w -= A- Apost) or post
// (Apost += 1, w += A+ Apre) jump and the clamp to [0, wmax]; the updated
// weight, traces and step go back as one 16-byte store.
template <bool kPre>
__device__ __forceinline__ void stdp_apply(const NetDev &n, int s, const Syn &y, float2 f, float a, int t) {
    float xpre = y.apre * f.x, xpost = y.apost * f.y, w = y.w;
    if (kPre) {
        xpre = xpre + 1.0f;
        w = clamp_w(w + (-a * xpost), y.wmax);
    } else {
        xpost = xpost + 1.0f;
        w = clamp_w(w + a * xpre, y.wmax);
    }
    reinterpret_cast<uint4 *>(n.rec + s)[0] =
        make_uint4(__float_as_uint(w), __float_as_uint(xpre), __float_as_uint(xpost), (unsigned int)t);
}

__device__ __forceinline__ int rule_of(unsigned int meta) { return (int)((meta >> 1) & 0x7fu) - 1; }

// Synapses per lane per round of a post-synaptic pass: every lane loads the
// records of kPostChunk synapses, then their decay factors, then stores, so
// a pass over up to 32 * kPostChunk in-synapses costs two memory round trips.
constexpr int kPostChunk = 2;

// This lane's share of a post-synaptic STDP pass over in-synapses
// [s, s1) of a spiking neuron, striding by the warp size.
template <class S>
__device__ __forceinline__ void post_stdp_lane(const NetDev &n, int s, int s1, int t) {
    // every record of this lane's share requested first: the rounds after the
    // first find theirs in L2
    for (int q = s + 32 * kPostChunk; q < s1; q += 32) prefetch_syn<S>(n, q);
    for (; s < s1; s += 32 * kPostChunk) {
        Syn y[kPostChunk];
        float2 f[kPostChunk];
        float a[kPostChunk];
#pragma unroll
        for (int k = 0; k < kPostChunk; ++k) {
            const int sk = s + 32 * k;
            if (sk < s1) y[k] = load_syn<S>(n, sk);
            else y[k].meta = 0u;
        }
#pragma unroll
        for (int k = 0; k < kPostChunk; ++k) {
            f[k] = make_float2(0.0f, 0.0f);
            a[k] = 0.0f;
            if (y[k].meta >= 2u) {
                const int rule = rule_of(y[k].meta);
                f[k] = decay_pair(n, rule, t - y[k].last);
                a[k] = y[k].a_post;
            }
        }
#pragma unroll
        for (int k = 0; k < kPostChunk; ++k)
            if (y[k].meta >= 2u) stdp_apply<false>(n, s + 32 * k, y[k], f[k], a[k], t);
    }
}

// Apply one arrival on synapse s of a target, its record y already loaded:
// its ProcessSpike with the weight as it is before this step's pre hook,
// then the pre hook if the synapse is plastic (the decay factors of its gap,
// one 8-byte load, then one 16-byte store).
template <class S>
__device__ __forceinline__ void apply_loaded(const NetDev &n, const Model &M, NeuronRegs &r, float &acc_a,
                                             float &acc_b, bool gate, int s, const Syn &y, int t) {
    const float w = y.w;
    const int type = y.meta & 1u;
    switch (S::model(M.model)) {
    case NBG_MODEL_LIF_VJ:
        if constexpr (S::has(NBG_MODEL_LIF_VJ)) {
            if (n.semantics == NBG_SEM_DENSE) {
                if (type == 0) acc_a = acc_a + w;
                else acc_b = acc_b + w;
            } else if (gate) {
                r.v = r.v + (type ? -w : w);
            }
        }
        break;
    case NBG_MODEL_IZH_COND:
        if constexpr (S::has(NBG_MODEL_IZH_COND)) {
            if (n.semantics == NBG_SEM_DENSE) { // summed into the step's pending channels
                if (type == 0) acc_a = acc_a + w;
                else acc_b = acc_b + w;
            } else if (type == 0) {
                r.gexc = r.gexc + w;
            } else {
                r.ginh = r.ginh + w;
            }
        }
        break;
    case NBG_MODEL_INPUT_SPIKE:
    case NBG_MODEL_INPUT_CURRENT: // event-driven inputs: ProcessSpike has no effect
        break;
    default: // IZH_RK4 current pulse, POISSON rate increment
        acc_a = acc_a + (type ? -w : w);
        break;
    }
    if (n.ev_t) {
        const unsigned long long pos = atomicAdd(n.ev_cursor, 1ull);
        if (pos < (unsigned long long)n.ev_cap) {
            n.ev_t[pos] = t;
            n.ev_pos[pos] = s;
            n.ev_w[pos] = w;
        } else {
            atomicOr(n.err, kErrEventLog);
        }
    }
    if (S::plastic(n) && y.meta >= 2u) { // pre-synaptic pair STDP (STDP::ApplyPreSynaticSpike)
        const int rule = rule_of(y.meta);
        const float2 f = decay_pair(n, rule, t - y.last);
        stdp_apply<true>(n, s, y, f, y.a_pre, t);
    }
}

template <class S>
__device__ __forceinline__ void apply_arrival(const NetDev &n, const Model &M, NeuronRegs &r, float &acc_a,
                                              float &acc_b, bool gate, int s, int t) {
    apply_loaded<S>(n, M, r, acc_a, acc_b, gate, s, load_syn<S>(n, s), t);
}

// Arrivals loaded per round by the wide drain.
constexpr int kBatch = 2;

// The set bits of `word` (first = the CSC position of bit 0), in ascending
// order, for a neuron with arrivals at most steps: the records of up to
// kBatch arrivals are loaded before any of them is applied (distinct
// synapses, so no load depends on an earlier apply), one memory round trip
// per round instead of one per arrival.
template <class S>
__device__ __forceinline__ void apply_word_batched(const NetDev &n, const Model &M, NeuronRegs &r, float &acc_a,
                                                   float &acc_b, bool gate, unsigned int word, int first, int t) {
    while (word) {
        int sk[kBatch];
        Syn y[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; ++k) {
            sk[k] = -1;
            if (word) {
                sk[k] = first + __ffs(word) - 1;
                word &= word - 1u;
            }
        }
#pragma unroll
        for (int k = 0; k < kBatch; ++k)
            if (sk[k] >= 0) y[k] = load_syn<S>(n, sk[k]);
#pragma unroll
        for (int k = 0; k < kBatch; ++k)
            if (sk[k] >= 0) apply_loaded<S>(n, M, r, acc_a, acc_b, gate, sk[k], y[k], t);
    }
}

// Apply every set bit of `word` (word index wi of this target) in ascending
// order.
template <class S>
__device__ __forceinline__ void apply_word(const NetDev &n, const Model &M, NeuronRegs &r, float &acc_a,
                                           float &acc_b, bool gate, unsigned int word, int first, int t) {
    for (; word; word &= word - 1u) apply_arrival<S>(n, M, r, acc_a, acc_b, gate, first + __ffs(word) - 1, t);
}

// apply_word for the deep drain: the record of synapse pos_cur was copied
// into shared memory (srec) a step ahead; an arrival on pos_nxt, the synapse
// whose copy for the next step is in flight, makes that copy stale.
template <class S>
__device__ __forceinline__ void apply_word_staged(const NetDev &n, const Model &M, NeuronRegs &r, float &acc_a,
                                                  float &acc_b, bool gate, unsigned int word, int first, int t,
                                                  int pos_cur, const uint4 *srec, int &pos_nxt) {
    for (; word; word &= word - 1u) {
        const int s = first + __ffs(word) - 1;
        Syn y;
        if (s == pos_cur) y = syn_decode(srec[0], srec[1]);
        else y = load_syn<S>(n, s);
        if (s == pos_nxt) pos_nxt = -1;
        apply_loaded<S>(n, M, r, acc_a, acc_b, gate, s, y, t);
    }
}

// One neuron update; returns true on a spike.  `noise` is
// sigma * gauss12(noise_key(seed, j), t) for noisy IZH_RK4 layers (else 0).
template <class S>
__device__ __forceinline__ bool update_neuron(const NetDev &n, const Model &M, NeuronRegs &r, float acc_a,
                                             float acc_b, float noise, int j, int t) {
    switch (S::model(M.model)) {
    case NBG_MODEL_LIF_VJ: {
        if constexpr (!S::has(NBG_MODEL_LIF_VJ)) return false;
        if (n.semantics == NBG_SEM_DENSE) {
            float nv = r.v + acc_a - acc_b;
            if (r.last >= M.ip) nv = nv + M.p[5] * (M.p[0] - nv + M.p[3] * r.iext);
            r.last += 1;
            if (nv >= M.p[2]) {
                r.v = M.p[4];
                r.last = 0;
                return true;
            }
            r.v = nv;
            return false;
        }
        float aux = (r.last > M.ip) ? r.lif_cur + (M.p[0] - r.v) / M.p[1] : 0.0f;
        r.v = r.v + aux * n.dt;
        r.last += 1;
        if (r.v > M.p[2]) {
            r.v = M.p[4];
            r.last = 0;
            return true;
        }
        return false;
    }
    case NBG_MODEL_IZH_COND: {
        if constexpr (!S::has(NBG_MODEL_IZH_COND)) return false;
        if (n.semantics == NBG_SEM_DENSE) {
            // dense runtime (DenseIzhikevichExponentialDecayDeviceUpdate.cuh:10-68):
            // decay-then-add conductances, u from the new v, no refractory gate
            const float ge = r.gexc * M.p[8] + acc_a;
            const float gi = r.ginh * M.p[9] + acc_b;
            const float V = r.v, U = r.u;
            const float total = ge * (M.p[6] - V) + gi * (M.p[7] - V) + r.iext;
            float v = V + n.dt * (0.04f * V * V + 5.0f * V + 140.0f - U + M.p[5] * total);
            float u = U + n.dt * (M.p[0] * (M.p[1] * v - U));
            r.gexc = ge;
            r.ginh = gi;
            r.last += 1;
            bool s = false;
            if (v >= M.p[4]) {
                v = M.p[2];
                u = u + M.p[3];
                r.last = 0;
                s = true;
            }
            r.v = v;
            r.u = u;
            return s;
        }
        const float V = r.v, U = r.u;
        float total = 0.0f;
        if (M.flags & 1) total = total + r.gexc * (M.p[6] - V);
        if (M.flags & 2) total = total + r.ginh * (M.p[7] - V);
        total = total + r.iext;
        float dv = 0.0f, du = 0.0f;
        if (r.last > 0) {
            dv = 0.04f * V * V + 5.0f * V + 140.0f - U + M.p[5] * total;
            du = M.p[0] * (M.p[1] * V - U);
        }
        r.v = r.v + dv * n.dt;
        r.u = r.u + du * n.dt;
        if (M.flags & 1) r.gexc = r.gexc * M.p[8];
        if (M.flags & 2) r.ginh = r.ginh * M.p[9];
        r.last += 1;
        if (r.v >= M.p[4]) {
            r.v = M.p[2];
            r.u = r.u + M.p[3];
            r.last = 0;
            return true;
        }
        return false;
    }
    case NBG_MODEL_IZH_RK4: {
        if constexpr (!S::has(NBG_MODEL_IZH_RK4)) return false;
        const float a = M.p[0], b = M.p[1];
        float I = acc_a + r.iext;
        if (M.p[5] != 0.0f) I = I + noise;
        if (r.last > 0) {
            const float h = n.dt, hh = 0.5f * n.dt, h6 = n.dt / 6.0f;
            const float v = r.v, u = r.u;
            const float k1v = izh_f(v, u, I), k1u = izh_g(a, b, v, u);
            const float v2 = __fmaf_rn(hh, k1v, v), u2 = __fmaf_rn(hh, k1u, u);
            const float k2v = izh_f(v2, u2, I), k2u = izh_g(a, b, v2, u2);
            const float v3 = __fmaf_rn(hh, k2v, v), u3 = __fmaf_rn(hh, k2u, u);
            const float k3v = izh_f(v3, u3, I), k3u = izh_g(a, b, v3, u3);
            const float v4 = __fmaf_rn(h, k3v, v), u4 = __fmaf_rn(h, k3u, u);
            const float k4v = izh_f(v4, u4, I), k4u = izh_g(a, b, v4, u4);
            r.v = __fmaf_rn(h6, __fmaf_rn(2.0f, k3v, __fmaf_rn(2.0f, k2v, k1v)) + k4v, v);
            r.u = __fmaf_rn(h6, __fmaf_rn(2.0f, k3u, __fmaf_rn(2.0f, k2u, k1u)) + k4u, u);
        }
        r.last += 1;
        if (r.v >= M.p[4]) {
            r.v = M.p[2];
            r.u = r.u + M.p[3];
            r.last = 0;
            return true;
        }
        return false;
    }
    case NBG_MODEL_INPUT_SPIKE:
    case NBG_MODEL_INPUT_CURRENT: // no time-driven dynamics
        return false;
    default: { // POISSON
        if constexpr (!S::has(NBG_MODEL_POISSON)) return false;
        float rate = M.p[0] + acc_a + M.p[1] * r.iext;
        rate = rate > 0.0f ? rate : 0.0f;
        float prob = rate * n.dt * 0.001f;
        prob = prob < 1.0f ? prob : 1.0f;
        if (hash_uniform01(j - M.ip, t) < prob) {
            r.last = 0;
            return true;
        }
        r.last += 1;
        return false;
    }
    }
}

// Firing probability and local hash index of generator neuron k; constant
// within a launch (its rate has no inputs; I_ext changes only between runs).
__device__ __forceinline__ float generator_prob(const NetDev &n, int k, int *local) {
    const LayerDev &G = n.layers[n.pop[k]];
    float rate = G.f[0] + 0.0f + G.f[1] * n.iext[k];
    rate = rate > 0.0f ? rate : 0.0f;
    float prob = rate * n.dt * 0.001f;
    *local = k - G.start;
    return prob < 1.0f ? prob : 1.0f;
}

__device__ __forceinline__ bool generator_fired(const NetDev &n, int k, int ts) {
    if (ts < 0) return false;
    int local;
    const float prob = generator_prob(n, k, &local);
    return hash_uniform01(local, ts) < prob;
}

// The first kGenCached generator inputs of a target, hoisted out of the step
// loop: local hash index, delay, CSC rank and probability.
constexpr int kGenCached = 1;
struct GenIn {
    int local, delay, pos;
    float prob;
};

// Advance every neuron B steps (drain arrivals, integrate, compact spikes,
// post-synaptic STDP).  One thread per neuron; all lanes stay in the loop so
// the per-step warp collectives are full-warp.  The post-synaptic STDP pass
// of a spiking neuron is spread over its warp: the 32 lanes stride over that
// neuron's CSC list.

// x mod D for x < 2D: ring slots are advanced by adding and wrapping once
// instead of an integer division per step and per mark (every step and
// delay offset added to a slot is below D: B + d_max <= D).
__device__ __forceinline__ unsigned int wrap_slot(unsigned int x, unsigned int D) { return x >= D ? x - D : x; }

// Bits [woff, woff+nw) of a summary row (nw <= 32), as an nw-bit mask.
__device__ __forceinline__ unsigned int summary_bits(const unsigned int *srow, int woff, int nw) {
    const int w0 = woff >> 5, sh = woff & 31;
    unsigned long long x = srow[w0];
    if (sh + nw > 32) x |= (unsigned long long)srow[w0 + 1] << 32;
    x >>= sh;
    return nw >= 32 ? (unsigned int)x : (unsigned int)x & ((1u << nw) - 1u);
}

// The same bits from the one or two summary words already read (lo = word
// woff / 32 of the row, hi = the next word, used when the range crosses it).
__device__ __forceinline__ unsigned int summary_decode(unsigned int lo, unsigned int hi, int woff, int nw) {
    const unsigned long long x = ((unsigned long long)hi << 32 | lo) >> (woff & 31);
    return nw >= 32 ? (unsigned int)x : (unsigned int)x & ((1u << nw) - 1u);
}

// Asynchronous 4-byte copy global -> shared (zero-filled when !valid, which
// reads nothing): the drain's look-ahead words land in shared memory instead
// of registers, so no instruction waits on them until they are read a step
// later.
__device__ __forceinline__ void stage_u32(unsigned int *dst, const unsigned int *src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"((unsigned int)__cvta_generic_to_shared(dst)),
                 "l"(__cvta_generic_to_global(src)), "r"(valid ? 4 : 0)
                 : "memory");
}
__device__ __forceinline__ void stage_16(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"((unsigned int)__cvta_generic_to_shared(dst)),
                 "l"(__cvta_generic_to_global(src))
                 : "memory");
}
__device__ __forceinline__ void stage_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Stage the summary words of [woff, woff+nw) in row srow.
__device__ __forceinline__ void stage_summary(unsigned int *lo, unsigned int *hi, const unsigned int *srow, int woff,
                                              int nw, bool valid) {
    const int w0 = woff >> 5;
    const bool two = valid && (woff & 31) + nw > 32;
    stage_u32(lo, srow + w0, valid);
    stage_u32(hi, srow + w0 + (two ? 1 : 0), two); // an address inside the row even when nothing is read
}

// Clear `bits` (relative to woff) in a summary row; neighbours share words.
__device__ __forceinline__ void summary_clear(unsigned int *srow, int woff, unsigned int bits) {
    const int w0 = woff >> 5, sh = woff & 31;
    const unsigned long long x = (unsigned long long)bits << sh;
    if ((unsigned int)x) atomicAnd(&srow[w0], ~(unsigned int)x);
    if (x >> 32) atomicAnd(&srow[w0 + 1], ~(unsigned int)(x >> 32));
}

// Clear the summary bits of words [woff, woff+nw) for any nw.
__device__ __forceinline__ void summary_clear_range(unsigned int *srow, int woff, int nw) {
    for (int w = woff; w < woff + nw;) {
        const int take = min(32 - (w & 31), woff + nw - w);
        const unsigned int m = take == 32 ? 0xffffffffu : ((1u << take) - 1u) << (w & 31);
        if (srow[w >> 5] & m) atomicAnd(&srow[w >> 5], ~m);
        w += take;
    }
}

// Out-synapse q of the CSR by source: its mask bit and delay.
__device__ __forceinline__ void out_entry(const NetDev &n, int q, unsigned int &bit, unsigned int &dl) {
    if (n.out_pk) {
        const unsigned int pk = n.out_pk[q];
        bit = pk >> n.out_dbits;
        dl = (pk & ((1u << n.out_dbits) - 1u)) + (unsigned int)n.out_dmin;
    } else {
        bit = n.out_bit[q];
        dl = n.out_delay[q];
    }
}

// Mark the out-synapses [q0, q1) of a spike at step t (the calling lanes
// stride over them): bit of the synapse in slot (t + delay) % D and the
// summary bit of its word.  No return values are used, so the atomics are
// fire-and-forget reductions.
__device__ __forceinline__ void mark_out(const NetDev &n, int q, int q1, unsigned int t) {
#pragma unroll 4
    for (; q < q1; q += 32) {
        unsigned int bit, dl;
        out_entry(n, q, bit, dl);
        const unsigned int slot = (t + dl) % (unsigned int)n.D;
        const unsigned int wd = bit >> 5;
        atomicOr(&n.mask[(size_t)slot * n.Wt + wd], 1u << (bit & 31u));
        atomicOr(&n.wsum[(size_t)slot * n.Ws + (wd >> 5)], 1u << (wd & 31u));
    }
}

// Generator neurons (PoissonRate layers without inputs: their targets draw
// their spikes inline) need only their own spike draws, for the raster and
// their LastSpike counter.  kGenPerThread of them per thread keeps them from
// occupying a thread slot each.
constexpr int kGenPerThread = 8;

// The B steps of the generator neurons of thread g: PoissonRate::UpdateState
// with no inputs (as update_neuron's POISSON case with acc = 0), raster
// entries of recorded layers reserved once per warp.
__device__ __forceinline__ void generator_steps(const NetDev &n, int g, int B, int T0, int run_t0, int lane) {
    unsigned int fired[kGenPerThread];
    int nrec = 0;
#pragma unroll
    for (int q = 0; q < kGenPerThread; ++q) {
        fired[q] = 0u;
        const int x = g * kGenPerThread + q;
        if (x < n.N_gen) {
            const int k = n.gen_ids[x];
            int local;
            const float prob = generator_prob(n, k, &local);
            int last = n.last[k];
            const int tslot = n.trace_slot ? n.trace_slot[k] : -1;
            for (int b = 0; b < B; ++b) {
                if (hash_uniform01(local, T0 + b) < prob) {
                    last = 0;
                    fired[q] |= 1u << b;
                } else {
                    last += 1;
                }
                if (tslot >= 0) n.trace[(size_t)(T0 + b - run_t0) * n.ntrace + tslot] = n.v[k];
            }
            n.last[k] = last;
            if (n.layers[n.pop[k]].record) nrec += __popc(fired[q]);
            else fired[q] = 0u;
        }
    }
    int incl = nrec;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0) return;
    unsigned int pos = 0;
    if (lane == 31) pos = atomicAdd(n.cursor, (unsigned int)total);
    pos = __shfl_sync(0xffffffffu, pos, 31) + (unsigned int)(incl - nrec);
    if (nrec == 0) return;
    if (pos + (unsigned int)nrec > (unsigned int)n.out_cap) {
        atomicOr(n.err, kErrOverflow);
        return;
    }
#pragma unroll
    for (int q = 0; q < kGenPerThread; ++q)
        for (unsigned int m = fired[q]; m; m &= m - 1u, ++pos) {
            n.out_ids[pos] = n.gen_ids[g * kGenPerThread + q];
            n.out_t[pos] = T0 + __ffs(m) - 1;
        }
}

// One block of B steps starting toff steps after the run call's first step.
template <class S>
__global__ void __launch_bounds__(256, S::min_blocks) k_update(const __grid_constant__ NetDev n, int B, int toff) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int reg_blocks = (n.N_upd + (int)blockDim.x - 1) / (int)blockDim.x;
    const bool gen_block = (int)blockIdx.x >= reg_blocks;
    const bool active = !gen_block && tid < n.N_upd;
    const int j = active && n.upd_ids ? n.upd_ids[tid] : tid;
    const int lane = threadIdx.x & 31;
    const int run_t0 = *n.run_t0;
    const int T0 = run_t0 + toff;
    // Programmatic dependent launch: the next block's launch may start once
    // every CTA of this one has; its prologue up to griddepcontrol.wait reads
    // only what no launch writes (network structure, parameters, generator
    // inputs), overlapping this launch's tail.
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    for (int k = threadIdx.x; k < n.sdtab_len; k += blockDim.x) s_dtab[k] = n.dtab[k];
    if (n.sdtab_len) __syncthreads();

    Model L;
    NeuronRegs r;
    int base = 0, end = 0, woff = 0, nw = 0, tslot = -1, g0 = 0, g1 = 0;
    if (active) {
        L = load_model(n.layers[n.pop[j]]);
        base = n.csc_ptr[j];
        end = n.csc_ptr[j + 1];
        woff = n.woff[j];
        nw = n.woff[j + 1] - woff;
        if (n.trace_slot) tslot = n.trace_slot[j];
        g0 = n.gen_ptr[j];
        g1 = n.gen_ptr[j + 1];
    }
    GenIn gin[kGenCached];
#pragma unroll
    for (int q = 0; q < kGenCached; ++q) {
        gin[q].local = 0;
        gin[q].delay = 0;
        gin[q].pos = 0;
        gin[q].prob = -1.0f; // never fires
        if (active && g0 + q < g1) {
            gin[q].prob = generator_prob(n, n.gen_src[g0 + q], &gin[q].local);
            gin[q].delay = n.gen_delay[g0 + q];
            gin[q].pos = n.gen_pos[g0 + q];
        }
    }
    // everything below reads or writes what the previous block's launch wrote
    asm volatile("griddepcontrol.wait;" ::: "memory");
    // external spikes of the block's steps (InputSpike::ProcessEvent): one
    // warp per spike marks its out-synapses like a spike of the update (their
    // arrivals fall after this block, so marking first is safe); the raster
    // entries are added on the host, which holds the list
    if (n.ext_ptr) {
        const int e0 = n.ext_ptr[toff], e1 = n.ext_ptr[toff + B];
        const int nwarps = (gridDim.x * blockDim.x) >> 5;
        for (int g = tid >> 5; g < e1 - e0; g += nwarps) {
            const int x = e0 + g;
            int b = 0;
            while (b + 1 < B && n.ext_ptr[toff + b + 1] <= x) ++b;
            const int src = n.ext_ids[x];
            mark_out(n, n.out_ptr[src] + lane, n.out_ptr[src + 1], (unsigned int)(T0 + b));
        }
    }
    if (gen_block) { // whole CTAs of generator threads
        generator_steps(n, tid - reg_blocks * (int)blockDim.x, B, T0, run_t0, lane);
        return;
    }
    if (active) {
        r.v = n.v[j];
        r.u = n.u[j];
        r.gexc = n.gexc[j];
        r.ginh = n.ginh[j];
        r.iext = n.iext[j];
        r.last = n.last[j];
        r.lif_cur = 0.0f;
        if (S::has(NBG_MODEL_LIF_VJ) && L.model == NBG_MODEL_LIF_VJ) // current_dV += R * I / tau (two roundings)
            r.lif_cur = r.lif_cur + L.p[3] * r.iext / L.p[1];
    }
    // noisy RK4 neurons: per-neuron noise key (the per-step draw is made in the step loop)
    const bool noisy = S::has(NBG_MODEL_IZH_RK4) && active && L.model == NBG_MODEL_IZH_RK4 && L.p[5] != 0.0f;
    const unsigned int nkey = noisy ? noise_key(n.seed, j) : 0u;
    // Fast path (in-degree <= 1024, <= 32 generator inputs): the L2-resident
    // word summary says which of this neuron's mask words hold arrivals, so
    // only those words are loaded.  Every mark for the block's slots was made
    // by earlier launches, so summary bits and words can be loaded early.
    // * Deep drain (S::deep): a pipeline three steps deep keeps the memory
    //   latency off the step.  At the top of step b the summary bits of step
    //   b + 3 and the first flagged mask word of step b + 2 are requested,
    //   and the synapse record of the first arrival of step b + 1 (whose word
    //   arrived during step b - 1); the second arrival's record is requested
    //   into the cache.  Further flagged words of a step (rare at a few
    //   arrivals per hundred steps) are loaded when it runs.  The requested
    //   words and record travel by asynchronous copy into shared memory and
    //   are read at the top of the next step: a load into a register would
    //   stall the step at its first use (the summary's shift, the move that
    //   rotates the pipeline), one memory round trip per step.
    // * Wide drain: the summary of step b + 3 (through shared memory, as
    //   above) and the first kWide flagged words of step b + 1 are requested
    //   while step b runs, and the arrivals of a word are applied kBatch per
    //   memory round trip.  (Prefetching step b + 1's records at the end of
    //   step b, and keeping the generator synapse's record in registers, both
    //   made the static networks slower.)
    const bool fast = nw <= 32 && (g1 - g0) <= 32;
    const unsigned int D = (unsigned int)n.D;
    const unsigned int slot0 = (unsigned int)T0 % D; // the block's first slot; later ones by wrap_slot
    constexpr int kWide = 4;
    // deep: summary bits of steps b, b+1, b+2 and the first flagged word of b, b+1
    unsigned int sbA = 0u, sbB = 0u, sbC = 0u, fwA = 0u, fwB = 0u;
    // wide: summary bits of steps b, b+1 and the first kWide words of step b (loads in flight)
    unsigned int sb_cur = 0u, sb_nxt = 0u;
    unsigned int w_cur[kWide] = {0u, 0u, 0u, 0u};
    // Look-ahead words in flight: [parity of the step that requested them]
    // [summary word lo, summary word hi, first flagged mask word][thread].
    // Each step waits for the words the step before requested, reads them
    // and requests the next ones into the other half.
    __shared__ unsigned int s_stage[2][3][256];
    unsigned int *const st_lo = &s_stage[0][0][threadIdx.x];
    constexpr int kStageHalf = 3 * 256, kStageHi = 256, kStageFw = 512;
    // deep: the record of the next step's first arrival, [parity][thread][two
    // 16-byte halves]; pos_nxt is its CSC position (-1: none, or stale)
    __shared__ uint4 s_rec[S::deep ? 2 * 256 * 2 : 1];
    int pos_nxt = -1;
    const bool staged = active && fast && nw > 0;
    if (staged) {
        if constexpr (S::deep) {
            sbA = summary_bits(n.wsum + (size_t)slot0 * n.Ws, woff, nw);
            if (B > 1) sbB = summary_bits(n.wsum + (size_t)wrap_slot(slot0 + 1u, D) * n.Ws, woff, nw);
            if (sbA) fwA = n.mask[(size_t)slot0 * n.Wt + woff + __ffs(sbA) - 1];
            // for step 0: the summary of step 2 and the first word of step 1
            unsigned int *const h = st_lo + kStageHalf;
            stage_summary(h, h + kStageHi, n.wsum + (size_t)wrap_slot(slot0 + 2u, D) * n.Ws, woff, nw, B > 2);
            stage_u32(h + kStageFw, n.mask + (size_t)wrap_slot(slot0 + 1u, D) * n.Wt + woff + (sbB ? __ffs(sbB) - 1 : 0),
                      sbB != 0u);
            stage_commit();
        } else {
            sb_cur = summary_bits(n.wsum + (size_t)slot0 * n.Ws, woff, nw);
            if (B > 1) sb_nxt = summary_bits(n.wsum + (size_t)wrap_slot(slot0 + 1u, D) * n.Ws, woff, nw);
            const unsigned int *r0 = n.mask + (size_t)slot0 * n.Wt + woff;
#pragma unroll
            for (int k = 0; k < kWide; ++k)
                if ((sb_cur >> k) & 1u) w_cur[k] = r0[k];
            unsigned int *const h = st_lo + kStageHalf; // for step 0: the summary of step 2
            stage_summary(h, h + kStageHi, n.wsum + (size_t)wrap_slot(slot0 + 2u, D) * n.Ws, woff, nw, B > 2);
            stage_commit();
        }
    }
    unsigned long long delivered = 0;
    unsigned int spk_steps = 0u; // bit b: this neuron spiked at step T0 + b
    for (int b = 0; b < B; ++b) {
        const int t = T0 + b;
        bool spk = false;
        const int pos_cur = pos_nxt; // deep: the staged record of this step, if any
        pos_nxt = -1;
        if (active) {
            const unsigned int slot = wrap_slot(slot0 + (unsigned int)b, D);
            unsigned int *mrow = n.mask + (size_t)slot * n.Wt + woff;
            float acc_a = 0.0f, acc_b = 0.0f;
            const bool gate = r.last > L.ip;
            if (fast) {
                unsigned int sb, fw = 0u;
                unsigned int wc[kWide];
                if constexpr (S::deep) {
                    sb = sbA;
                    fw = fwA;
                    if (staged) {
                        // the words step b - 1 requested: the summary of step
                        // b + 2 and the first flagged word of step b + 1
                        stage_wait();
                        const unsigned int *const h = st_lo + ((b + 1) & 1) * kStageHalf;
                        sbC = summary_decode(h[0], h[kStageHi], woff, nw);
                        fwB = h[kStageFw];
                        if (b + 1 < B) { // request the summary of step b + 3 and the first word of step b + 2
                            unsigned int *const q = st_lo + (b & 1) * kStageHalf;
                            stage_summary(q, q + kStageHi, n.wsum + (size_t)wrap_slot(slot + 3u, D) * n.Ws, woff,
                                          nw, b + 3 < B);
                            stage_u32(q + kStageFw,
                                      n.mask + (size_t)wrap_slot(slot + 2u, D) * n.Wt + woff +
                                          (sbC ? __ffs(sbC) - 1 : 0),
                                      b + 2 < B && sbC != 0u);
                            if (fwB) { // the record of step b + 1's first arrival
                                pos_nxt = base + (__ffs(sbB) - 1) * 32 + __ffs(fwB) - 1;
                                uint4 *const d = s_rec + ((b & 1) * 256 + threadIdx.x) * 2;
                                stage_16(d, n.rec + pos_nxt);
                                stage_16(d + 1, reinterpret_cast<const uint4 *>(n.rec + pos_nxt) + 1);
                            }
                            stage_commit();
                        }
                    }
                    if (fwB) { // the record of its second arrival into L2
                        const unsigned int rest = fwB & (fwB - 1u);
                        if (rest) prefetch_syn<S>(n, base + (__ffs(sbB) - 1) * 32 + __ffs(rest) - 1);
                    }
                    sbA = sbB;
                    fwA = fwB;
                    sbB = sbC;
                } else {
                    sb = sb_cur;
#pragma unroll
                    for (int k = 0; k < kWide; ++k) wc[k] = w_cur[k];
                    if (b + 1 < B) { // words of step b + 1
                        const unsigned int *rn = n.mask + (size_t)wrap_slot(slot + 1u, D) * n.Wt + woff;
#pragma unroll
                        for (int k = 0; k < kWide; ++k) w_cur[k] = ((sb_nxt >> k) & 1u) ? rn[k] : 0u;
                        sb_cur = sb_nxt;
                    }
                    if (staged) { // the summary of step b + 2 (requested by step b - 1); request b + 3's
                        stage_wait();
                        const unsigned int *const h = st_lo + ((b + 1) & 1) * kStageHalf;
                        sb_nxt = summary_decode(h[0], h[kStageHi], woff, nw);
                        if (b + 1 < B) {
                            unsigned int *const q = st_lo + (b & 1) * kStageHalf;
                            stage_summary(q, q + kStageHi, n.wsum + (size_t)wrap_slot(slot + 3u, D) * n.Ws, woff,
                                          nw, b + 3 < B);
                            stage_commit();
                        }
                    }
                }
                // generator arrivals of this step (pure functions of source and time)
                unsigned int gfired = 0u, gwords = 0u;
#pragma unroll
                for (int q = 0; q < kGenCached; ++q) {
                    const int ts = t - gin[q].delay;
                    if (g0 + q < g1 && ts >= 0 && hash_uniform01(gin[q].local, ts) < gin[q].prob) {
                        gfired |= 1u << q;
                        gwords |= 1u << (gin[q].pos >> 5);
                    }
                }
                for (int g = g0 + kGenCached; g < g1; ++g)
                    if (generator_fired(n, n.gen_src[g], t - (int)n.gen_delay[g])) {
                        gfired |= 1u << (g - g0);
                        gwords |= 1u << (n.gen_pos[g] >> 5);
                    }
                unsigned int need = sb | gwords;
                if (sb) summary_clear(n.wsum + (size_t)slot * n.Ws, woff, sb);
                const int wfirst = __ffs(sb) - 1; // deep: the word already loaded (fw), -1 if none
                while (need) {
                    const int wi = __ffs(need) - 1;
                    need &= need - 1u;
                    unsigned int word = 0u;
                    if ((sb >> wi) & 1u) {
                        if constexpr (S::deep) {
                            word = wi == wfirst ? fw : mrow[wi];
                        } else if (wi < kWide) {
                            word = wc[0];
#pragma unroll
                            for (int k = 1; k < kWide; ++k)
                                if (wi == k) word = wc[k];
                        } else {
                            word = mrow[wi];
                        }
                        mrow[wi] = 0u;
                    }
                    for (unsigned int gf = gfired; gf; gf &= gf - 1u) {
                        const int q = __ffs(gf) - 1;
                        const int gp = q == 0 ? gin[0].pos : n.gen_pos[g0 + q];
                        if ((gp >> 5) == wi) word |= 1u << (gp & 31);
                    }
                    delivered += __popc(word);
                    if constexpr (S::deep)
                        apply_word_staged<S>(n, L, r, acc_a, acc_b, gate, word, base + wi * 32, t, pos_cur,
                                             s_rec + (((b + 1) & 1) * 256 + threadIdx.x) * 2, pos_nxt);
                    else
                        apply_word_batched<S>(n, L, r, acc_a, acc_b, gate, word, base + wi * 32, t);
                }
            } else {
                int gq = g0;
                for (int wi = 0; wi < nw; ++wi) {
                    unsigned int word = mrow[wi];
                    if (word) mrow[wi] = 0u;
                    for (; gq < g1 && (n.gen_pos[gq] >> 5) == wi; ++gq)
                        if (generator_fired(n, n.gen_src[gq], t - (int)n.gen_delay[gq]))
                            word |= 1u << (n.gen_pos[gq] & 31);
                    if (!word) continue;
                    delivered += __popc(word);
                    apply_word<S>(n, L, r, acc_a, acc_b, gate, word, base + wi * 32, t);
                }
                // this neuron's summary bits (set while its words were non-zero)
                summary_clear_range(n.wsum + (size_t)slot * n.Ws, woff, nw);
            }
            spk = update_neuron<S>(n, L, r, acc_a, acc_b, noisy ? L.p[5] * gauss12(nkey, t) : 0.0f, j, t);
            if (tslot >= 0) n.trace[(size_t)(t - run_t0) * n.ntrace + tslot] = r.v;
        }
        if (spk) {
            pos_nxt = -1; // the post-synaptic pass below rewrites every record of this neuron
            // the out-list bounds the propagation reads after the last step
            if (!spk_steps)
                asm volatile("prefetch.global.L1 [%0];" ::"l"(__cvta_generic_to_global(n.out_ptr + j)));
            spk_steps |= 1u << b;
        }
        // post-synaptic STDP (STDP::ApplyPostSynaticSpike) of every spiking
        // lane, the warp striding over that neuron's in-synapses
        unsigned int sbal = S::plastic(n) ? __ballot_sync(0xffffffffu, spk && end > base) : 0u;
        while (sbal) {
            const int l = __ffs(sbal) - 1;
            sbal &= sbal - 1u;
            const int s0 = __shfl_sync(0xffffffffu, base, l), s1 = __shfl_sync(0xffffffffu, end, l);
            post_stdp_lane<S>(n, s0 + lane, s1, t);
        }
        __syncwarp(); // the owners read these synapses at their next arrivals
    }
    if (active) {
        n.v[j] = r.v;
        n.u[j] = r.u;
        n.gexc[j] = r.gexc;
        n.ginh[j] = r.ginh;
        n.last[j] = r.last;
    }
    // The block's spikes leave the warp after its last step: nothing in this
    // launch reads their marks (arrivals fall at or after T0 + B, and the
    // ring never aliases this block's slots), so the loads they need overlap
    // with other warps' steps instead of stalling every step.
    // Raster: output-layer spikes, one cursor reservation per warp; the
    // reservation is requested here and its result used after the
    // propagation, so that its round trip overlaps the marks.
    const int nrec = (active && L.record) ? __popc(spk_steps) : 0;
    int rincl = nrec;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, rincl, o);
        if (lane >= o) rincl += y;
    }
    const int rtotal = __shfl_sync(0xffffffffu, rincl, 31);
    unsigned int rpos = 0;
    if (rtotal > 0 && lane == 31) rpos = atomicAdd(n.cursor, (unsigned int)rtotal);
    // Propagation: the out-lists of all the warp's spiking lanes form one
    // range that the 32 lanes stride over together (entry e belongs to the
    // first lane whose inclusive prefix of list lengths exceeds e).  The
    // list bounds of every spiking lane come in one round trip, and the
    // entry loads of four rounds are issued before their marks.  Each
    // synapse is loaded once and marked for every step its source spiked in.
    {
        int q0 = 0, cnt = 0;
        if (spk_steps) {
            q0 = n.out_ptr[j];
            cnt = n.out_ptr[j + 1] - q0;
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        constexpr int kRounds = 4;
        for (int e0 = 0; e0 < total; e0 += 32 * kRounds) {
            unsigned int bit[kRounds], dl[kRounds], steps[kRounds];
#pragma unroll
            for (int k = 0; k < kRounds; ++k) {
                const int e = e0 + 32 * k + lane;
                int owner = 0; // first lane with incl > e (binary search over the warp's prefix)
#pragma unroll
                for (int w = 16; w > 0; w >>= 1) {
                    const int c = __shfl_sync(0xffffffffu, incl, owner + w - 1);
                    if (c <= e) owner += w;
                }
                const int oq = __shfl_sync(0xffffffffu, q0, owner & 31);
                const int oe = __shfl_sync(0xffffffffu, incl - cnt, owner & 31);
                steps[k] = __shfl_sync(0xffffffffu, spk_steps, owner & 31);
                bit[k] = dl[k] = 0u;
                if (e < total) out_entry(n, oq + (e - oe), bit[k], dl[k]);
                else steps[k] = 0u;
            }
#pragma unroll
            for (int k = 0; k < kRounds; ++k) {
                const unsigned int wd = bit[k] >> 5;
                for (unsigned int m = steps[k]; m; m &= m - 1u) {
                    const unsigned int slot = wrap_slot(slot0 + (unsigned int)(__ffs(m) - 1) + dl[k], D);
                    atomicOr(&n.mask[(size_t)slot * n.Wt + wd], 1u << (bit[k] & 31u));
                    atomicOr(&n.wsum[(size_t)slot * n.Ws + (wd >> 5)], 1u << (wd & 31u));
                }
            }
        }
    }
    if (rtotal > 0) {
        unsigned int pos = __shfl_sync(0xffffffffu, rpos, 31) + (unsigned int)(rincl - nrec);
        if (nrec > 0) {
            if (pos + (unsigned int)nrec <= (unsigned int)n.out_cap) {
                for (unsigned int m = spk_steps; m; m &= m - 1u, ++pos) {
                    n.out_ids[pos] = j;
                    n.out_t[pos] = T0 + __ffs(m) - 1;
                }
            } else {
                atomicOr(n.err, kErrOverflow);
            }
        }
    }
    // warp-aggregated delivered-event count
    for (int o = 16; o > 0; o >>= 1) delivered += __shfl_down_sync(0xffffffffu, delivered, o);
    if (lane == 0 && delivered) atomicAdd(n.n_events, delivered);
}

// ------------------------------------------------------------------ host side

} // namespace

NBG_HIDDEN cudaError_t nbg_device_decay_table(float *tab, const float *inv_host, int rows, int len, float dt);

// Largest spike bitmap of the raster ordering, in 32-bit words (1 GiB); the
// environment variable NBG_RASTER_BITMAP_WORDS overrides it at creation.
constexpr size_t kRasterBitmapWords = (size_t)1 << 28;

// Allocator whose value-initialisation leaves trivially constructible
// elements uninitialised: the raster vectors grow by up to hundreds of MB per
// run call and are overwritten right after.
template <class T> struct NoInitAlloc : std::allocator<T> {
    template <class U> struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <class U> NoInitAlloc(const NoInitAlloc<U> &) noexcept {}
    template <class U> void construct(U *p) noexcept(std::is_nothrow_default_constructible<U>::value) {
        ::new ((void *)p) U;
    }
    template <class U, class... A> void construct(U *p, A &&...a) { ::new ((void *)p) U(std::forward<A>(a)...); }
};

struct nbg_engine {
    int device = 0;
    int N = 0;
    int64_t S = 0;
    int D = 1, Wt = 0, dmin = 1, dmax = 1, B = 1;
    int threads = 256;
    int n_rules = 0;
    bool plastic = false; // any synapse with a learning rule
    void (*update_kernel)(NetDev, int, int) = nullptr; // k_update instance for this network's profile
    float dt = 1.0f;
    int semantics = 0;
    unsigned long long seed = 0;
    bool use_graph = true;
    int64_t spike_capacity = 0;
    int64_t ev_cap = 0;
    // host copies
    std::vector<LayerDev> layers;
    std::vector<unsigned short> pop_host;
    std::vector<int> csc_ptr;
    std::vector<int64_t> csc_orig; // CSC position -> original connection index
    std::vector<int64_t> orig_pos; // original connection index -> CSC position
    std::vector<nbg_stdp_desc> rules;
    std::vector<float> init_v, init_u, init_iext;
    std::vector<int> woff_host; // first mask word of each neuron (N + 1 entries)
    int *pin_ids = nullptr, *pin_t = nullptr; // pinned staging of the raster download
    size_t pin_cap = 0;
    int sm_count = 1;
    size_t raster_bitmap_words = kRasterBitmapWords;
    // host-side fault injection (NBG_RASTER_ORDER_FAIL, read at creation):
    // the device ordering reports an allocation failure, which exercises the
    // host fallback of nbg_run
    bool raster_order_fail = false;
    // raster ordering: per-step spike bitmap, tile sums / positions, running
    // base, ordered entries; timings of the last run call's raster phases
    DevBuf<unsigned int> rbm, rtile, rbase;
    DevBuf<int> ord_ids, ord_t;
    cudaEvent_t evr0 = nullptr, evr1 = nullptr;
    double last_order_ms = 0.0, last_download_ms = 0.0, last_append_ms = 0.0;
    int64_t last_order_launches = 0;
    std::vector<float> init_w;
    // device buffers
    DevBuf<unsigned short> pop;
    DevBuf<LayerDev> d_layers;
    DevBuf<SynRec> rec;    // plastic network: synapse records
    DevBuf<SynStatic> wst; // static network: weight + meta
    DevBuf<float> init_w_d; // weights reset returns to, CSC order
    DevBuf<float> v, u, gexc, ginh, iext, trace, ev_w;
    DevBuf<float2> dtab;
    DevBuf<int> gen_ptr, gen_pos, gen_src;
    DevBuf<unsigned short> gen_delay;
    DevBuf<int> last, csc_ptr_d, woff, out_ptr, out_ids, out_t, err, run_t0, trace_slot, ev_t, ev_pos;
    DevBuf<unsigned int> mask, wsum, out_bit, out_pk;
    int out_dbits = 0, out_dmin = 0;
    int Ws = 1;
    DevBuf<unsigned short> out_delay;
    DevBuf<unsigned int> cursor;
    DevBuf<unsigned long long> ev_cursor, n_events;
    int dtab_len = 0;
    bool dtab_complete = false; // table reached exact zero: longer gaps decay to 0
    // time / recording
    int next_t = 0;
    bool ran = false;
    std::vector<int32_t, NoInitAlloc<int32_t>> spk_t, spk_id; // growth does not zero-fill
    std::vector<int32_t> trace_ids;
    std::vector<float> trace_rows;
    int64_t trace_nrows = 0;
    struct CurrentEvent {
        int t, id;
        float value;
    };
    std::vector<CurrentEvent> currents; // pending, sorted by time
    // external spikes: pending (time, neuron) pairs, and the device list of
    // the current call
    std::vector<std::pair<int, int>> ext_pending;
    std::unordered_set<uint64_t> ext_keys;
    std::vector<int> ext_ptr_h, ext_ids_h;
    DevBuf<int> ext_ptr_d, ext_ids_d;
    DevBuf<int> upd_ids_d, gen_ids_d; // thread map (NetDev::upd_ids, gen_ids)
    int N_upd = 0, N_gen = 0;
    // current synapses (type 3): per source the out-going ones (target,
    // delay, latch slot); latch slots are grouped by target in CSC order
    std::vector<int> cur_out_ptr, cur_out_tgt, cur_out_delay, cur_out_slot;
    std::vector<int> cur_tgt_ptr; // target j: latch slots [cur_tgt_ptr[j], cur_tgt_ptr[j+1])
    std::vector<float> cur_latch;
    struct LatchEvent {
        int t, slot;
        float value;
        int64_t seq;
    };
    std::vector<LatchEvent> latches; // pending
    int64_t latch_seq = 0;
    std::vector<int32_t> log_t;
    std::vector<int64_t> log_conn;
    std::vector<float> log_w;
    // launch resources
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_blocks = 0, graph_tail = 0, graph_B = 0, graph_threads = 0;
    NetDev graph_nd{}; // kernel arguments baked into the graph
    double last_ms = 0.0, last_upd_ms = 0.0, last_prop_ms = 0.0;
    int64_t last_launches = 0;
    bool kernel_timing = false;
    std::vector<cudaEvent_t> tev; // 3 per block of one graph / launch batch
    int tev_used = 0;             // blocks bracketed since the last harvest

    NetDev dev() {
        NetDev n{};
        n.N = N;
        n.D = D;
        n.Wt = Wt;
        n.n_layers = (int)layers.size();
        n.semantics = semantics;
        n.dt = dt;
        n.seed = seed;
        n.pop = pop.p;
        n.layers = d_layers.p;
        n.v = v.p;
        n.u = u.p;
        n.gexc = gexc.p;
        n.ginh = ginh.p;
        n.iext = iext.p;
        n.last = last.p;
        n.csc_ptr = csc_ptr_d.p;
        n.woff = woff.p;
        n.rec = rec.p;
        n.wst = wst.p;
        n.dtab = dtab.p;
        n.dtab_len = dtab_len;
        n.sdtab_len = plastic && n_rules > 0 ? std::min(dtab_len, kSharedDecayEntries) : 0;
        n.mask = mask.p;
        n.wsum = wsum.p;
        n.Ws = Ws;
        n.out_ptr = out_ptr.p;
        n.out_pk = out_pk.p;
        n.out_dbits = out_dbits;
        n.out_dmin = out_dmin;
        n.out_bit = out_bit.p;
        n.out_delay = out_delay.p;
        n.gen_ptr = gen_ptr.p;
        n.gen_pos = gen_pos.p;
        n.gen_src = gen_src.p;
        n.gen_delay = gen_delay.p;
        n.out_ids = out_ids.p;
        n.out_t = out_t.p;
        n.cursor = cursor.p;
        n.out_cap = (long long)out_ids.n;
        n.err = err.p;
        n.run_t0 = run_t0.p;
        n.trace_slot = trace_ids.empty() ? nullptr : trace_slot.p;
        n.trace = trace.p;
        n.ntrace = (int)trace_ids.size();
        n.ev_t = ev_cap > 0 ? ev_t.p : nullptr;
        n.ev_pos = ev_pos.p;
        n.ev_w = ev_w.p;
        n.ev_cursor = ev_cursor.p;
        n.ev_cap = ev_cap;
        n.n_events = n_events.p;
        n.ext_ptr = ext_ptr_d.p;
        n.ext_ids = ext_ids_d.p;
        n.N_upd = N_upd;
        n.N_gen = N_gen;
        n.upd_ids = upd_ids_d.p;
        n.gen_ids = gen_ids_d.p;
        return n;
    }
};

namespace {

// Host decay table: table[k] = expf(-((float)k * dt) * inv_tau), the exact
// float expression of STDP_State::SetUpdate evaluated with the host libm.
// Dense-runtime profile: the table is built on the device with CUDA's expf
// and inv_tau = 1.0f / max(1e-6f, tau) (DenseStdpLearningModel.h:115,
// DenseLearningDeviceRuntime.cuh:65-77), long enough that its last entry is
// 0 (expf of an argument below -104 is 0 in float).
nbg_status dense_decay_table(nbg_engine *e) {
    std::vector<float> inv((size_t)e->n_rules * 2);
    int64_t len = 1;
    for (int r = 0; r < e->n_rules; ++r) {
        inv[r * 2 + 0] = 1.0f / std::max(1.0e-6f, e->rules[r].ltp_tau);
        inv[r * 2 + 1] = 1.0f / std::max(1.0e-6f, e->rules[r].ltd_tau);
        for (int w = 0; w < 2; ++w) {
            int64_t k = 1;
            while ((float)k * e->dt * inv[r * 2 + w] <= 104.0f && k < ((int64_t)1 << 24)) k *= 2;
            len = std::max(len, k + 1);
        }
    }
    if (len > ((int64_t)1 << 24)) return fail(NBG_ERR_UNSUPPORTED, "STDP decay table would exceed 2^24 entries");
    NBG_CUDA(e->dtab.alloc((size_t)e->n_rules * len));
    NBG_CUDA(nbg_device_decay_table(reinterpret_cast<float *>(e->dtab.p), inv.data(), e->n_rules * 2, (int)len,
                                    e->dt));
    e->dtab_len = (int)len;
    e->dtab_complete = true;
    for (int r = 0; r < e->n_rules; ++r) { // verify the underflow to 0
        float2 last = make_float2(1.0f, 1.0f);
        NBG_CUDA(cudaMemcpy(&last, e->dtab.p + (size_t)r * len + len - 1, sizeof(float2), cudaMemcpyDeviceToHost));
        if (last.x != 0.0f || last.y != 0.0f) e->dtab_complete = false;
    }
    if (!e->dtab_complete) return fail(NBG_ERR_UNSUPPORTED, "dense STDP decay table did not reach 0");
    return NBG_OK;
}

nbg_status ensure_decay_table(nbg_engine *e, int64_t needed) {
    if (e->n_rules == 0) return NBG_OK;
    if (e->dtab_complete || e->dtab_len >= needed) return NBG_OK;
    if (e->semantics == NBG_SEM_DENSE) return dense_decay_table(e);
    // Entry k does not depend on the table's length, so the table is grown
    // ahead of need: at least doubled, and at once to the length where every
    // row has underflowed to 0 when that is at most 2^22 entries.  It (and the
    // CUDA graph holding its address) is then rebuilt a few times per
    // simulation instead of at every run call.
    int64_t full = 1;
    for (int r = 0; r < e->n_rules; ++r)
        for (const float tau : {e->rules[r].ltp_tau, e->rules[r].ltd_tau}) {
            const float inv = (float)(1.0 / (double)tau);
            int64_t k = 1;
            while ((float)k * e->dt * inv <= 104.0f && k < ((int64_t)1 << 24)) k *= 2;
            full = std::max(full, k + 1);
        }
    int64_t len = std::max<int64_t>({needed, (int64_t)4096, 2 * (int64_t)e->dtab_len});
    if (full <= ((int64_t)1 << 22)) len = std::max(len, full);
    len = std::min<int64_t>(len, (int64_t)1 << 24);
    std::vector<float2> tab((size_t)e->n_rules * len);
    bool complete = true;
    for (int r = 0; r < e->n_rules; ++r) {
        const float inv_p = (float)(1.0 / (double)e->rules[r].ltp_tau);
        const float inv_m = (float)(1.0 / (double)e->rules[r].ltd_tau);
        bool zp = false, zm = false;
        for (int64_t k = 0; k < len; ++k) {
            const float dtime = (float)k * e->dt;
            const float vp = std::exp(-dtime * inv_p);
            const float vm = std::exp(-dtime * inv_m);
            tab[(size_t)r * len + k] = make_float2(vp, vm);
            if (k == len - 1) {
                zp = vp == 0.0f;
                zm = vm == 0.0f;
            }
        }
        complete = complete && zp && zm;
    }
    if (!complete && needed > len) return fail(NBG_ERR_UNSUPPORTED, "STDP decay table would exceed 2^24 entries");
    NBG_CUDA(e->dtab.upload(tab));
    e->dtab_len = (int)len;
    e->dtab_complete = complete;
    return NBG_OK;
}

// Weights from `w` (CSC order); with `traces`, also Apre = Apost = 0 and
// last = 0.  meta and wmax are left as they are.
__global__ void k_set_synapses(SynRec *rec, SynStatic *wst, const float *__restrict__ w, long long S, int traces) {
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= S) return;
    if (rec) {
        if (traces) {
            reinterpret_cast<uint4 *>(rec + p)[0] = make_uint4(__float_as_uint(w[p]), 0u, 0u, 0u);
        } else {
            rec[p].w = w[p];
        }
    } else {
        wst[p].w = w[p];
    }
}

// Every synapse's weight back to init_w_d (and, with `traces`, its STDP state
// to zero), on the engine's stream, synchronously.
cudaError_t reset_synapses(nbg_engine *e, bool traces) {
    const long long S = e->S;
    k_set_synapses<<<(unsigned)((S + 255) / 256), 256, 0, e->stream>>>(e->rec.p, e->wst.p, e->init_w_d.p, S,
                                                                       traces ? 1 : 0);
    const cudaError_t ce = cudaGetLastError();
    return ce != cudaSuccess ? ce : cudaStreamSynchronize(e->stream);
}

nbg_status upload_layers(nbg_engine *e) {
    NBG_CUDA(e->d_layers.alloc(e->layers.size()));
    NBG_CUDA(cudaMemcpy(e->d_layers.p, e->layers.data(), e->layers.size() * sizeof(LayerDev),
                        cudaMemcpyHostToDevice));
    return NBG_OK;
}

nbg_status reset_state(nbg_engine *e) {
    NBG_CUDA(cudaMemcpy(e->v.p, e->init_v.data(), e->N * sizeof(float), cudaMemcpyHostToDevice));
    NBG_CUDA(cudaMemcpy(e->u.p, e->init_u.data(), e->N * sizeof(float), cudaMemcpyHostToDevice));
    NBG_CUDA(cudaMemcpy(e->iext.p, e->init_iext.data(), e->N * sizeof(float), cudaMemcpyHostToDevice));
    NBG_CUDA(e->gexc.zero());
    NBG_CUDA(e->ginh.zero());
    std::vector<int> last0((size_t)e->N, 10000);
    NBG_CUDA(cudaMemcpy(e->last.p, last0.data(), e->N * sizeof(int), cudaMemcpyHostToDevice));
    if (e->S > 0) NBG_CUDA(reset_synapses(e, true));
    NBG_CUDA(e->mask.zero());
    NBG_CUDA(e->wsum.zero());
    NBG_CUDA(e->err.zero());
    NBG_CUDA(e->cursor.zero());
    NBG_CUDA(e->ev_cursor.zero());
    NBG_CUDA(e->n_events.zero());
    e->next_t = 0;
    e->ran = false;
    e->spk_t.clear();
    e->spk_id.clear();
    e->trace_rows.clear();
    e->trace_nrows = 0;
    e->log_t.clear();
    e->log_conn.clear();
    e->log_w.clear();
    e->currents.clear();
    e->ext_pending.clear();
    e->ext_keys.clear();
    e->latches.clear();
    std::fill(e->cur_latch.begin(), e->cur_latch.end(), 0.0f);
    return NBG_OK;
}

constexpr int kLaunchChunk = 64; // direct launches between timing harvests

// Grow the pool of event pairs used to bracket the launches.
nbg_status ensure_timing_events(nbg_engine *e, int blocks) {
    if (!e->kernel_timing) return NBG_OK;
    while ((int)e->tev.size() < 2 * blocks) {
        cudaEvent_t ev;
        NBG_CUDA(cudaEventCreate(&ev));
        e->tev.push_back(ev);
    }
    return NBG_OK;
}

// Launch one block of B steps.  With kernel timing, `slot` selects the event
// pair bracketing the launch.
// Inside stream capture an event record must be "external" to become an
// event-record node of the graph (a plain record is only a dependency).
void launch_block(nbg_engine *e, const NetDev &nd, int B, int toff, int slot, bool capturing = false) {
    const int gen_threads = (e->N_gen + kGenPerThread - 1) / kGenPerThread;
    const int grid = std::max(1, (e->N_upd + e->threads - 1) / e->threads + (gen_threads + e->threads - 1) / e->threads);
    const unsigned int flags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    if (e->kernel_timing) cudaEventRecordWithFlags(e->tev[2 * slot + 0], e->stream, flags);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(e->threads);
    cfg.dynamicSmemBytes = (size_t)nd.sdtab_len * sizeof(float2);
    cfg.stream = e->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, e->update_kernel, nd, B, toff); // errors surface at the call's cudaGetLastError
    if (e->kernel_timing) cudaEventRecordWithFlags(e->tev[2 * slot + 1], e->stream, flags);
}

// Sum the bracketed kernel durations of `blocks` event pairs.
nbg_status harvest_timing(nbg_engine *e, int blocks) {
    if (!e->kernel_timing || blocks == 0) return NBG_OK;
    NBG_CUDA(cudaEventSynchronize(e->tev[2 * (blocks - 1) + 1]));
    for (int k = 0; k < blocks; ++k) {
        float a = 0.0f;
        NBG_CUDA(cudaEventElapsedTime(&a, e->tev[2 * k + 0], e->tev[2 * k + 1]));
        e->last_upd_ms += a;
    }
    return NBG_OK;
}

// ---------------------------------------------------------------------------
// Raster ordering on the device.  The update kernel appends (step, id)
// entries in warp order; a run call returns its raster in (step, id) order.
// A spike bitmap per step gives that order without a sort: every entry sets
// its bit, a popcount scan over the bitmap words gives each word its first
// output position, and the set bits are written out word by word.  A neuron
// spikes at most once per step, so the bitmap holds every entry (the host
// checks that the emitted count equals the entry count).  Bitmap rows are
// padded to whole 16-byte groups and the bitmap to whole tiles; long calls
// are ordered in chunks of steps whose bitmap fits the budget.
constexpr int kRasterThreads = 256;
constexpr int kRasterWordsPerThread = 16;                                  // four 16-byte loads
constexpr int kRasterTileWords = kRasterThreads * kRasterWordsPerThread;  // words per CTA
constexpr int kRasterScanThreads = 1024, kRasterScanPerThread = 8;

// Exclusive prefix sum over the block of x (blockDim.x a multiple of 32, at
// most 1024); *total receives the block's sum.  wt: 33 words of shared memory.
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned x, unsigned *wt, unsigned *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wt[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const unsigned v = lane < nw ? wt[lane] : 0u;
        unsigned vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, vi, o);
            if (lane >= o) vi += y;
        }
        if (lane < nw) wt[lane] = vi - v;
        if (lane == 31) wt[32] = vi;
    }
    __syncthreads();
    *total = wt[32];
    return wt[wid] + inc - x;
}

__global__ void k_raster_mark(const int *__restrict__ ts, const int *__restrict__ ids, unsigned n, int t_lo,
                              int steps, int wp, int n_neurons, unsigned *__restrict__ bm) {
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int s = ts[i] - t_lo;
        const int id = ids[i];
        if (s < 0 || s >= steps || id < 0 || id >= n_neurons) continue;
        atomicOr(bm + (size_t)s * (size_t)wp + (size_t)(id >> 5), 1u << (id & 31));
    }
}

__global__ void __launch_bounds__(kRasterThreads) k_raster_count(const uint4 *__restrict__ bm,
                                                                 unsigned *__restrict__ tile_sum) {
    __shared__ unsigned wt[33];
    const uint4 *q = bm + ((size_t)blockIdx.x * kRasterTileWords + (size_t)threadIdx.x * kRasterWordsPerThread) / 4;
    unsigned c = 0;
#pragma unroll
    for (int k = 0; k < kRasterWordsPerThread / 4; ++k) {
        const uint4 v = q[k];
        c += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
    }
    unsigned total;
    block_exclusive_scan(c, wt, &total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// One CTA: tile sums -> first output position of each tile, continuing from
// *base (the entries of earlier chunks); *base advances by the chunk's total.
__global__ void __launch_bounds__(kRasterScanThreads) k_raster_scan(unsigned *__restrict__ tile, unsigned n_tiles,
                                                                    unsigned *__restrict__ base) {
    __shared__ unsigned wt[33];
    unsigned carry = *base;
    __syncthreads();
    for (unsigned c0 = 0; c0 < n_tiles; c0 += kRasterScanThreads * kRasterScanPerThread) {
        const unsigned i0 = c0 + threadIdx.x * kRasterScanPerThread;
        unsigned v[kRasterScanPerThread], sum = 0;
#pragma unroll
        for (int k = 0; k < kRasterScanPerThread; ++k) {
            v[k] = i0 + k < n_tiles ? tile[i0 + k] : 0u;
            sum += v[k];
        }
        unsigned total;
        unsigned run = carry + block_exclusive_scan(sum, wt, &total);
#pragma unroll
        for (int k = 0; k < kRasterScanPerThread; ++k) {
            if (i0 + k < n_tiles) tile[i0 + k] = run;
            run += v[k];
        }
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *base = carry;
}

__global__ void __launch_bounds__(kRasterThreads) k_raster_emit(const uint4 *__restrict__ bm,
                                                                const unsigned *__restrict__ tile_pos, int wp,
                                                                int t_lo, int *__restrict__ out_ids,
                                                                int *__restrict__ out_t) {
    __shared__ unsigned wt[33];
    const size_t w0 = (size_t)blockIdx.x * kRasterTileWords + (size_t)threadIdx.x * kRasterWordsPerThread;
    const uint4 *q = bm + w0 / 4;
    unsigned w[kRasterWordsPerThread], c = 0;
#pragma unroll
    for (int k = 0; k < kRasterWordsPerThread / 4; ++k) {
        const uint4 v = q[k];
        w[4 * k + 0] = v.x;
        w[4 * k + 1] = v.y;
        w[4 * k + 2] = v.z;
        w[4 * k + 3] = v.w;
        c += __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
    }
    unsigned total;
    unsigned pos = tile_pos[blockIdx.x] + block_exclusive_scan(c, wt, &total);
    if (c == 0) return;
    size_t s = w0 / (size_t)wp;
    int col = (int)(w0 - s * (size_t)wp);
#pragma unroll
    for (int k = 0; k < kRasterWordsPerThread; ++k) {
        unsigned m = w[k];
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            out_ids[pos] = (col << 5) + b;
            out_t[pos] = t_lo + (int)s;
            ++pos;
        }
        if (++col == wp) {
            col = 0;
            ++s;
        }
    }
}

// Order this call's n device raster entries by (step, id) into ord_ids /
// ord_t; returns the number of ordered entries in *n_out.
nbg_status order_raster(nbg_engine *e, unsigned n, int t0, int count, unsigned *n_out) {
    *n_out = 0;
    e->last_order_ms = 0.0;
    e->last_order_launches = 0;
    if (n == 0) return NBG_OK;
    const int wp = (((e->N + 31) >> 5) + 3) & ~3;
    const int chunk =
        (int)std::max<int64_t>(1, std::min<int64_t>(count, (int64_t)(e->raster_bitmap_words / (size_t)wp)));
    auto tiles_of = [&](int steps) {
        return (unsigned)(((size_t)steps * (size_t)wp + kRasterTileWords - 1) / kRasterTileWords);
    };
    const unsigned max_tiles = tiles_of(chunk);
    if (e->raster_order_fail)
        return fail(NBG_ERR_CUDA, "raster bitmap: %s (injected)", cudaGetErrorString(cudaErrorMemoryAllocation));
    if (e->rbm.n < (size_t)max_tiles * kRasterTileWords) NBG_CUDA(e->rbm.alloc((size_t)max_tiles * kRasterTileWords));
    if (e->rtile.n < max_tiles) NBG_CUDA(e->rtile.alloc(max_tiles));
    if (e->rbase.n < 1) NBG_CUDA(e->rbase.alloc(1));
    if (e->ord_ids.n < n) {
        NBG_CUDA(e->ord_ids.alloc(n));
        NBG_CUDA(e->ord_t.alloc(n));
    }
    NBG_CUDA(cudaEventRecord(e->evr0, e->stream));
    NBG_CUDA(cudaMemsetAsync(e->rbase.p, 0, sizeof(unsigned), e->stream));
    const unsigned mark_grid =
        (unsigned)std::min<size_t>(((size_t)n + kRasterThreads - 1) / kRasterThreads, (size_t)e->sm_count * 8);
    int64_t launches = 0;
    for (int c0 = 0; c0 < count; c0 += chunk) {
        const int steps = std::min(chunk, count - c0);
        const unsigned tiles = tiles_of(steps);
        NBG_CUDA(cudaMemsetAsync(e->rbm.p, 0, (size_t)tiles * kRasterTileWords * sizeof(unsigned), e->stream));
        k_raster_mark<<<mark_grid, kRasterThreads, 0, e->stream>>>(e->out_t.p, e->out_ids.p, n, t0 + c0, steps, wp,
                                                                   (int)e->N, e->rbm.p);
        k_raster_count<<<tiles, kRasterThreads, 0, e->stream>>>(reinterpret_cast<const uint4 *>(e->rbm.p),
                                                                e->rtile.p);
        k_raster_scan<<<1, kRasterScanThreads, 0, e->stream>>>(e->rtile.p, tiles, e->rbase.p);
        k_raster_emit<<<tiles, kRasterThreads, 0, e->stream>>>(reinterpret_cast<const uint4 *>(e->rbm.p),
                                                               e->rtile.p, wp, t0 + c0, e->ord_ids.p, e->ord_t.p);
        launches += 4;
    }
    NBG_CUDA(cudaGetLastError());
    NBG_CUDA(cudaEventRecord(e->evr1, e->stream));
    NBG_CUDA(cudaMemcpyAsync(n_out, e->rbase.p, sizeof(unsigned), cudaMemcpyDeviceToHost, e->stream));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    float ms = 0.0f;
    NBG_CUDA(cudaEventElapsedTime(&ms, e->evr0, e->evr1));
    e->last_order_ms = ms;
    e->last_order_launches = launches;
    if (*n_out != n) return fail(NBG_ERR_STATE, "raster holds %u entries but %u distinct (step, neuron) pairs", n, *n_out);
    return NBG_OK;
}

// Append one run call's raster, already in (step, id) order, to spk_t /
// spk_id, merged with ext: the external spikes of recorded neurons, sorted
// by (step, id) and never among the device entries.  Large appends copy on
// up to 16 host threads.
void append_raster(nbg_engine *e, const int *ts, const int *ids, size_t n,
                   const std::vector<std::pair<int, int>> &ext) {
    const size_t base = e->spk_id.size();
    e->spk_id.resize(base + n + ext.size());
    e->spk_t.resize(base + n + ext.size());
    int *out_id = e->spk_id.data() + base, *out_t = e->spk_t.data() + base;
    if (!ext.empty()) {
        size_t i = 0, j = 0, o = 0;
        while (i < n || j < ext.size()) {
            const bool take_dev = j == ext.size() ||
                                  (i < n && (ts[i] < ext[j].first || (ts[i] == ext[j].first && ids[i] < ext[j].second)));
            if (take_dev) {
                out_t[o] = ts[i];
                out_id[o++] = ids[i++];
            } else {
                out_t[o] = ext[j].first;
                out_id[o++] = ext[j++].second;
            }
        }
        return;
    }
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int T = n >= ((size_t)1 << 20) ? (int)std::min(16u, hw) : 1;
    auto body = [&](int k) {
        const size_t lo = n * (size_t)k / (size_t)T, hi = n * (size_t)(k + 1) / (size_t)T;
        std::memcpy(out_t + lo, ts + lo, (hi - lo) * sizeof(int));
        std::memcpy(out_id + lo, ids + lo, (hi - lo) * sizeof(int));
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < T; ++k) pool.emplace_back(body, k);
    body(0);
    for (auto &th : pool) th.join();
}

} // namespace

extern "C" {

const char *nbg_last_error(void) { return g_err.c_str(); }
const char *nbg_version(void) { return "nbg 0.1 (sm_103a)"; }

void nbg_default_options(nbg_options *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->device = 0;
    o->block_steps = 0;
    o->threads_per_block = 256;
    o->spike_capacity = 0;
    o->use_graph = 1;
    o->event_log_capacity = 0;
    o->kernel_timing = 0;
}

nbg_status nbg_create(const nbg_net_desc *d, const nbg_options *opt_in, nbg_engine **out);

nbg_status nbg_create_batch(const nbg_net_desc *const *descs, int n, const nbg_options *opt, nbg_engine **out,
                            int64_t *first_neuron) {
    if (!descs || !out || n <= 0) return fail(NBG_ERR_INVALID, "need at least one network description");
    *out = nullptr;
    std::vector<nbg_layer_desc> layers;
    std::vector<int32_t> src, tgt, type, delay, rule;
    std::vector<float> w, wmax;
    std::vector<nbg_stdp_desc> rules;
    std::vector<int64_t> first((size_t)n + 1, 0);
    int64_t off = 0;
    int roff = 0;
    for (int k = 0; k < n; ++k) {
        const nbg_net_desc *d = descs[k];
        if (!d || !d->layers || d->n_layers <= 0) return fail(NBG_ERR_INVALID, "instance %d: no layers", k);
        if (d->dt_ms != descs[0]->dt_ms || d->semantics != descs[0]->semantics || d->seed != descs[0]->seed)
            return fail(NBG_ERR_INVALID, "instance %d: every instance must share dt_ms, semantics and seed", k);
        if (d->n_conn < 0 || (d->n_conn > 0 && (!d->source || !d->target || !d->type || !d->weight ||
                                                !d->max_weight || !d->delay || !d->rule)))
            return fail(NBG_ERR_INVALID, "instance %d: connection arrays must be non-null", k);
        if (d->n_rules < 0 || (d->n_rules > 0 && !d->rules))
            return fail(NBG_ERR_INVALID, "instance %d: bad learning rules", k);
        int64_t count = 0;
        for (int l = 0; l < d->n_layers; ++l) {
            if (d->layers[l].count <= 0) return fail(NBG_ERR_INVALID, "instance %d layer %d: count must be positive", k, l);
            count += d->layers[l].count;
            layers.push_back(d->layers[l]);
        }
        // ids are checked per instance: an id past the instance's end would
        // otherwise land in the next instance
        for (int64_t c = 0; c < d->n_conn; ++c) {
            if (d->source[c] < 0 || d->source[c] >= count || d->target[c] < 0 || d->target[c] >= count)
                return fail(NBG_ERR_INVALID, "instance %d connection %lld: neuron id out of range", k, (long long)c);
            if (d->rule[c] >= d->n_rules)
                return fail(NBG_ERR_INVALID, "instance %d connection %lld: unknown learning rule", k, (long long)c);
            src.push_back((int32_t)(d->source[c] + off));
            tgt.push_back((int32_t)(d->target[c] + off));
            type.push_back(d->type[c]);
            w.push_back(d->weight[c]);
            wmax.push_back(d->max_weight[c]);
            delay.push_back(d->delay[c]);
            rule.push_back(d->rule[c] < 0 ? d->rule[c] : d->rule[c] + roff);
        }
        for (int r = 0; r < d->n_rules; ++r) rules.push_back(d->rules[r]);
        first[(size_t)k] = off;
        off += count;
        roff += d->n_rules;
        if (off > (1 << 30)) return fail(NBG_ERR_INVALID, "too many neurons");
    }
    first[(size_t)n] = off;
    if (layers.size() > 65535) return fail(NBG_ERR_INVALID, "need 1..65535 layers in all");
    nbg_net_desc u{};
    u.n_layers = (int)layers.size();
    u.layers = layers.data();
    u.n_conn = (int64_t)src.size();
    u.source = src.data();
    u.target = tgt.data();
    u.type = type.data();
    u.weight = w.data();
    u.max_weight = wmax.data();
    u.delay = delay.data();
    u.rule = rule.data();
    u.n_rules = (int)rules.size();
    u.rules = rules.data();
    u.dt_ms = descs[0]->dt_ms;
    u.semantics = descs[0]->semantics;
    u.seed = descs[0]->seed;
    const nbg_status st = nbg_create(&u, opt, out);
    if (st == NBG_OK && first_neuron) std::copy(first.begin(), first.end(), first_neuron);
    return st;
}

nbg_status nbg_create(const nbg_net_desc *d, const nbg_options *opt_in, nbg_engine **out) {
    if (!d || !out) return fail(NBG_ERR_INVALID, "null argument");
    *out = nullptr;
    nbg_options opt;
    nbg_default_options(&opt);
    if (opt_in) opt = *opt_in;
    if (d->n_layers <= 0 || d->n_layers > 65535 || !d->layers)
        return fail(NBG_ERR_INVALID, "need 1..65535 layers");
    if (!(d->dt_ms > 0.0f)) return fail(NBG_ERR_INVALID, "timestep must be positive");
    if (d->semantics != NBG_SEM_LEGACY_CPU && d->semantics != NBG_SEM_DENSE)
        return fail(NBG_ERR_INVALID, "unknown semantics %d", d->semantics);
    if (d->n_conn < 0 || d->n_conn > 0x7FFFFFFFll) return fail(NBG_ERR_INVALID, "connection count out of range");
    if (d->n_conn > 0 && (!d->source || !d->target || !d->type || !d->weight || !d->max_weight || !d->delay ||
                          !d->rule))
        return fail(NBG_ERR_INVALID, "connection arrays must be non-null");
    if (d->n_rules < 0 || d->n_rules > 126 || (d->n_rules > 0 && !d->rules))
        return fail(NBG_ERR_INVALID, "need 0..126 learning rules");
    if (opt.threads_per_block <= 0) opt.threads_per_block = 256;
    if (opt.threads_per_block % 32 || opt.threads_per_block > 256)
        return fail(NBG_ERR_INVALID, "threads_per_block must be a multiple of 32 and <= 256");

    int64_t total = 0;
    for (int l = 0; l < d->n_layers; ++l) {
        const nbg_layer_desc &ld = d->layers[l];
        if (ld.model < 0 || ld.model > NBG_MODEL_INPUT_CURRENT)
            return fail(NBG_ERR_INVALID, "layer %d: unknown model %d", l, ld.model);
        if (ld.count <= 0) return fail(NBG_ERR_INVALID, "layer %d: count must be positive", l);
        total += ld.count;
    }
    if (total > (1 << 30)) return fail(NBG_ERR_INVALID, "too many neurons");
    for (int r = 0; r < d->n_rules; ++r)
        if (!(d->rules[r].ltp_tau > 0.0f) || !(d->rules[r].ltd_tau > 0.0f))
            return fail(NBG_ERR_INVALID, "rule %d: time constants must be positive", r);

    auto *e = new nbg_engine();
    e->device = opt.device;
    e->N = (int)total;
    e->S = d->n_conn;
    e->dt = d->dt_ms;
    e->semantics = d->semantics;
    e->seed = d->seed;
    e->threads = opt.threads_per_block;
    e->use_graph = opt.use_graph != 0;
    e->ev_cap = opt.event_log_capacity;
    e->kernel_timing = opt.kernel_timing != 0;
    e->n_rules = d->n_rules;
    e->rules.assign(d->rules, d->rules + d->n_rules);
    auto bail = [&](nbg_status s) {
        delete e;
        return s;
    };
    // ---- layers
    std::vector<unsigned short> pop((size_t)e->N);
    e->layers.resize(d->n_layers);
    e->init_v.assign(e->N, 0.0f);
    e->init_u.assign(e->N, 0.0f);
    e->init_iext.assign(e->N, 0.0f);
    int start = 0;
    for (int l = 0; l < d->n_layers; ++l) {
        const nbg_layer_desc &ld = d->layers[l];
        LayerDev L{};
        L.model = ld.model;
        L.start = start;
        L.count = ld.count;
        L.record = ld.output != 0;
        std::memcpy(L.f, ld.f, sizeof(L.f));
        std::memcpy(L.ip, ld.ip, sizeof(L.ip));
        if (ld.model == NBG_MODEL_IZH_COND) {
            if (d->semantics == NBG_SEM_DENSE) {
                // dense runtime: std::exp(-dt_ms / tau) (DenseIzhikevichExponentialDecayModel.h:139-141)
                L.decay_exc = std::exp(-d->dt_ms / ld.f[8]);
                L.decay_inh = std::exp(-d->dt_ms / ld.f[10]);
            } else {
                const float inv_a = ld.f[8] != 0.0f ? 1.0f / ld.f[8] : 0.0f;
                const float inv_g = ld.f[10] != 0.0f ? 1.0f / ld.f[10] : 0.0f;
                L.decay_exc = std::exp(-d->dt_ms * inv_a);
                L.decay_inh = std::exp(-d->dt_ms * inv_g);
            }
        }
        if (ld.model == NBG_MODEL_LIF_VJ) {
            if (!(ld.f[1] != 0.0f)) return bail(fail(NBG_ERR_INVALID, "layer %d: tau must be non-zero", l));
            L.alpha = d->dt_ms / ld.f[1];
        }
        for (int i = start; i < start + ld.count; ++i) {
            pop[i] = (unsigned short)l;
            switch (ld.model) {
            case NBG_MODEL_LIF_VJ:
                e->init_v[i] = d->semantics == NBG_SEM_DENSE ? ld.f[0] : ld.f[4] + ld.f[5];
                e->init_iext[i] = ld.f[6];
                break;
            case NBG_MODEL_IZH_COND:
                e->init_v[i] = ld.f[4];
                e->init_u[i] = ld.f[1] * ld.f[4];
                e->init_iext[i] = ld.f[11];
                break;
            case NBG_MODEL_IZH_RK4:
                e->init_v[i] = ld.f[4];
                e->init_u[i] = ld.f[1] * ld.f[4];
                e->init_iext[i] = ld.f[7];
                break;
            case NBG_MODEL_POISSON:
                e->init_iext[i] = ld.f[2];
                break;
            default: // input layers: no state
                break;
            }
        }
        e->layers[l] = L;
        start += ld.count;
    }

    // ---- validate connections, CSC order by (target, source, delay, index)
    const int64_t S = d->n_conn;
    e->dmin = 0x7FFFFFFF;
    e->dmax = 1;
    std::vector<int> indeg((size_t)e->N + 1, 0);
    for (int64_t s = 0; s < S; ++s) {
        const int a = d->source[s], b = d->target[s];
        if (a < 0 || a >= e->N || b < 0 || b >= e->N)
            return bail(fail(NBG_ERR_INVALID, "connection %lld: neuron id out of range", (long long)s));
        if (d->delay[s] < 1 || d->delay[s] > 65535)
            return bail(fail(NBG_ERR_INVALID, "connection %lld: delay must be in 1..65535 steps", (long long)s));
        if (d->type[s] != NBG_SYN_EXC && d->type[s] != NBG_SYN_INH && d->type[s] != NBG_SYN_CURRENT)
            return bail(fail(NBG_ERR_UNSUPPORTED,
                             "connection %lld: synapse type %d not supported (0 exc, 1 inh, 3 current)",
                             (long long)s, d->type[s]));
        if ((d->type[s] == NBG_SYN_CURRENT) != (e->layers[pop[a]].model == NBG_MODEL_INPUT_CURRENT))
            return bail(fail(NBG_ERR_UNSUPPORTED,
                             "connection %lld: input-current neurons connect through current synapses (type 3) "
                             "and only they do", (long long)s));
        if (d->type[s] == NBG_SYN_CURRENT && d->rule[s] != -1)
            return bail(fail(NBG_ERR_UNSUPPORTED, "connection %lld: a current synapse cannot learn", (long long)s));
        if (d->rule[s] < -1 || d->rule[s] >= d->n_rules)
            return bail(fail(NBG_ERR_INVALID, "connection %lld: learning rule %d out of range", (long long)s,
                             d->rule[s]));
        if (!std::isfinite(d->weight[s]) || !std::isfinite(d->max_weight[s]))
            return bail(fail(NBG_ERR_INVALID, "connection %lld: weight must be finite", (long long)s));
        indeg[b + 1]++;
        if (d->type[s] == NBG_SYN_EXC) e->layers[pop[b]].has_exc = 1;
        else if (d->type[s] == NBG_SYN_INH) e->layers[pop[b]].has_inh = 1;
    }
    // generator layers: PoissonRate layers without incoming synapses
    {
        std::vector<int64_t> layer_in(d->n_layers, 0);
        for (int i = 0; i < e->N; ++i) layer_in[pop[i]] += indeg[i + 1];
        for (int l = 0; l < d->n_layers; ++l)
            e->layers[l].generator = e->layers[l].model == NBG_MODEL_POISSON && layer_in[l] == 0;
    }
    for (int64_t s = 0; s < S; ++s) {
        if (e->layers[pop[d->source[s]]].generator || d->type[s] == NBG_SYN_CURRENT) continue;
        e->dmin = std::min(e->dmin, d->delay[s]);
        e->dmax = std::max(e->dmax, d->delay[s]);
    }
    if (e->dmin == 0x7FFFFFFF) e->dmin = kMaxBlockSteps; // nothing goes through the ring
    std::vector<int> &cptr = e->csc_ptr;
    cptr.assign((size_t)e->N + 1, 0);
    for (int i = 0; i < e->N; ++i) cptr[i + 1] = cptr[i] + indeg[i + 1];
    e->csc_orig.assign((size_t)S, 0);
    {
        std::vector<int> fill(cptr.begin(), cptr.end() - 1);
        for (int64_t s = 0; s < S; ++s) e->csc_orig[fill[d->target[s]]++] = s; // stable by index
        for (int j = 0; j < e->N; ++j) {
            auto first = e->csc_orig.begin() + cptr[j], last_it = e->csc_orig.begin() + cptr[j + 1];
            std::sort(first, last_it, [&](int64_t x, int64_t y) {
                if (d->source[x] != d->source[y]) return d->source[x] < d->source[y];
                if (d->delay[x] != d->delay[y]) return d->delay[x] < d->delay[y];
                return x < y;
            });
        }
    }
    e->orig_pos.assign((size_t)S, 0);
    for (int64_t p = 0; p < S; ++p) e->orig_pos[e->csc_orig[p]] = p;

    // ---- mask word offsets and per-synapse arrays
    std::vector<int> woff((size_t)e->N + 1, 0);
    for (int j = 0; j < e->N; ++j) woff[j + 1] = woff[j] + (cptr[j + 1] - cptr[j] + 31) / 32;
    e->Wt = std::max(woff[e->N], 1);
    e->woff_host = woff;
    // ring slots: every delay plus the longest block, so that no mark made
    // inside a block aliases a slot the block drains
    e->D = e->dmax + std::min(e->dmin, kMaxBlockSteps);
    e->pop_host = pop;
    std::vector<float> w((size_t)S);
    std::vector<int> src_of((size_t)S);
    for (int64_t p = 0; p < S; ++p) {
        const int64_t s = e->csc_orig[p];
        w[p] = d->weight[s];
        src_of[p] = d->source[s];
    }
    e->init_w = w;
    e->plastic = false;
    for (int64_t s = 0; s < S && !e->plastic; ++s) e->plastic = d->rule[s] >= 0;
    // synapse records: 32 bytes with the STDP state when anything learns
    std::vector<SynRec> recs;
    std::vector<SynStatic> wsts;
    if (e->plastic) recs.resize((size_t)S);
    else wsts.resize((size_t)S);
    for (int64_t p = 0; p < S; ++p) {
        const int64_t s = e->csc_orig[p];
        const unsigned int meta = (unsigned int)((d->type[s] & 1) | ((d->rule[s] + 1) << 1));
        if (e->plastic) {
            SynRec &r = recs[(size_t)p];
            r = SynRec{};
            r.w = w[p];
            r.meta = meta;
            r.wmax = d->max_weight[s];
            if (d->rule[s] >= 0) {
                r.a_pre = d->rules[d->rule[s]].max_ltd;
                r.a_post = d->rules[d->rule[s]].max_ltp;
            }
        } else {
            wsts[(size_t)p] = SynStatic{w[p], meta};
        }
    }

    // ---- current synapses: latch slots by target (CSC order), out-lists by source
    {
        std::vector<unsigned char> is_cur((size_t)S, 0);
        e->cur_tgt_ptr.assign((size_t)e->N + 1, 0);
        e->cur_out_ptr.assign((size_t)e->N + 1, 0);
        for (int j = 0; j < e->N; ++j)
            for (int p = cptr[j]; p < cptr[j + 1]; ++p)
                if (d->type[e->csc_orig[p]] == NBG_SYN_CURRENT) {
                    is_cur[p] = 1;
                    e->cur_tgt_ptr[j + 1]++;
                    e->cur_out_ptr[src_of[p] + 1]++;
                }
        for (int i = 0; i < e->N; ++i) {
            e->cur_tgt_ptr[i + 1] += e->cur_tgt_ptr[i];
            e->cur_out_ptr[i + 1] += e->cur_out_ptr[i];
        }
        const int nc = e->cur_tgt_ptr[e->N];
        e->cur_latch.assign((size_t)nc, 0.0f);
        e->cur_out_tgt.assign((size_t)nc, 0);
        e->cur_out_delay.assign((size_t)nc, 0);
        e->cur_out_slot.assign((size_t)nc, 0);
        std::vector<int> fill(e->cur_out_ptr.begin(), e->cur_out_ptr.end() - 1);
        int slot = 0;
        for (int j = 0; j < e->N; ++j)
            for (int p = cptr[j]; p < cptr[j + 1]; ++p)
                if (is_cur[p]) {
                    const int q = fill[src_of[p]]++;
                    e->cur_out_tgt[q] = j;
                    e->cur_out_delay[q] = d->delay[e->csc_orig[p]];
                    e->cur_out_slot[q] = slot++;
                }
    }

    // ---- CSR by source over (mask bit, delay); generator sources and
    // current synapses excluded
    auto spike_syn = [&](int p) { return d->type[e->csc_orig[p]] != NBG_SYN_CURRENT; };
    std::vector<int> optr((size_t)e->N + 1, 0);
    std::vector<int> gptr((size_t)e->N + 1, 0);
    for (int j = 0; j < e->N; ++j)
        for (int p = cptr[j]; p < cptr[j + 1]; ++p) {
            if (!spike_syn(p)) continue;
            if (e->layers[pop[src_of[p]]].generator) gptr[j + 1]++;
            else optr[src_of[p] + 1]++;
        }
    for (int i = 0; i < e->N; ++i) {
        optr[i + 1] += optr[i];
        gptr[i + 1] += gptr[i];
    }
    std::vector<unsigned int> obit((size_t)optr[e->N]);
    std::vector<unsigned short> odelay((size_t)optr[e->N]);
    std::vector<int> gpos((size_t)gptr[e->N]), gsrc((size_t)gptr[e->N]);
    std::vector<unsigned short> gdelay((size_t)gptr[e->N]);
    {
        std::vector<int> fill(optr.begin(), optr.end() - 1);
        int gq = 0;
        for (int j = 0; j < e->N; ++j)
            for (int p = cptr[j]; p < cptr[j + 1]; ++p) {
                if (!spike_syn(p)) continue;
                const unsigned short dl = (unsigned short)d->delay[e->csc_orig[p]];
                if (e->layers[pop[src_of[p]]].generator) {
                    gpos[gq] = p - cptr[j]; // ascending within j: CSC order
                    gsrc[gq] = src_of[p];
                    gdelay[gq] = dl;
                    ++gq;
                    continue;
                }
                const int q = fill[src_of[p]]++;
                obit[q] = (unsigned int)woff[j] * 32u + (unsigned int)(p - cptr[j]);
                odelay[q] = dl;
            }
    }
    if ((uint64_t)e->Wt * 32ull > 0xFFFFFFFFull) return bail(fail(NBG_ERR_UNSUPPORTED, "too many synapses"));
    // one 32-bit word per out-synapse when the mask bit and the delay above
    // dmin fit in it together (one load per out-synapse instead of two)
    std::vector<unsigned int> opk;
    {
        auto bits_for = [](uint64_t maxval) {
            int b = 0;
            while (b < 64 && (maxval >> b) != 0) ++b;
            return b;
        };
        const int dbits = bits_for((uint64_t)(e->dmax - std::min(e->dmin, e->dmax)));
        const int bbits = bits_for((uint64_t)e->Wt * 32ull - 1ull);
        if (!obit.empty() && dbits + bbits <= 32) {
            e->out_dbits = dbits;
            e->out_dmin = e->dmin;
            opk.resize(obit.size());
            for (size_t q = 0; q < obit.size(); ++q)
                opk[q] = (obit[q] << dbits) | (unsigned int)(odelay[q] - e->dmin);
        }
    }

    {   // update-kernel instance: the models the update threads meet (generator
        // layers have their own threads) and whether anything learns
        unsigned models = 0u;
        for (const LayerDev &L : e->layers)
            if (!L.generator) models |= 1u << L.model;
        const unsigned lif_poisson = (1u << NBG_MODEL_LIF_VJ) | (1u << NBG_MODEL_POISSON);
        if (models == (1u << NBG_MODEL_IZH_RK4) && e->plastic)
            e->update_kernel = k_update<Spec<1u << NBG_MODEL_IZH_RK4, 1>>;
        else if (models == (1u << NBG_MODEL_LIF_VJ) && !e->plastic)
            e->update_kernel = k_update<Spec<1u << NBG_MODEL_LIF_VJ, 0>>;
        else if ((models & ~lif_poisson) == 0u && !e->plastic)
            e->update_kernel = k_update<Spec<lif_poisson, 0>>;
        else
            e->update_kernel = k_update<GenericSpec>;
    }
    int B = opt.block_steps > 0 ? std::min(opt.block_steps, e->dmin) : e->dmin;
    e->B = std::max(1, std::min(B, kMaxBlockSteps));

    // ---- device allocation
    if (cudaSetDevice(e->device) != cudaSuccess)
        return bail(fail(NBG_ERR_CUDA, "cudaSetDevice(%d) failed: no usable CUDA device", opt.device));
    nbg_status st = NBG_OK;
    auto chk = [&](cudaError_t ce, const char *what) {
        if (ce != cudaSuccess && st == NBG_OK)
            st = fail(ce == cudaErrorMemoryAllocation ? NBG_ERR_OOM : NBG_ERR_CUDA, "%s: %s", what,
                      cudaGetErrorString(ce));
    };
    chk(cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking), "stream");
    chk(cudaEventCreate(&e->ev0), "event");
    chk(cudaEventCreate(&e->ev1), "event");
    chk(cudaEventCreate(&e->evr0), "event");
    chk(cudaEventCreate(&e->evr1), "event");
    chk(cudaDeviceGetAttribute(&e->sm_count, cudaDevAttrMultiProcessorCount, e->device), "SM count");
    // the decay-table head in dynamic shared memory comes on top of the
    // kernel's static staging arrays: above the 48 KiB a launch gets by default
    chk(cudaFuncSetAttribute(reinterpret_cast<const void *>(e->update_kernel),
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(kSharedDecayEntries * sizeof(float2))),
        "update kernel shared memory");
    if (const char *rb = std::getenv("NBG_RASTER_BITMAP_WORDS")) {
        const long long v = std::atoll(rb);
        if (v > 0) e->raster_bitmap_words = (size_t)v;
    }
    if (const char *rf = std::getenv("NBG_RASTER_ORDER_FAIL")) e->raster_order_fail = std::atoi(rf) != 0;

    chk(e->pop.upload(pop), "pop");
    const size_t N = (size_t)e->N;
    chk(e->v.alloc(N), "v");
    chk(e->u.alloc(N), "u");
    chk(e->gexc.alloc(N), "gexc");
    chk(e->ginh.alloc(N), "ginh");
    chk(e->iext.alloc(N), "iext");
    chk(e->last.alloc(N), "last");
    chk(e->csc_ptr_d.upload(cptr), "csc_ptr");
    chk(e->woff.upload(woff), "woff");
    if (e->plastic) chk(e->rec.upload(recs), "synapse records");
    else chk(e->wst.upload(wsts), "synapse records");
    chk(e->init_w_d.upload(w), "initial weights");
    chk(e->mask.alloc((size_t)e->D * e->Wt), "mask ring");
    e->Ws = (e->Wt + 31) / 32 + 1;
    chk(e->wsum.alloc((size_t)e->D * e->Ws), "mask summary ring");
    chk(e->out_ptr.upload(optr), "out_ptr");
    if (!opk.empty()) {
        chk(e->out_pk.upload(opk), "out lists");
    } else {
        chk(e->out_bit.upload(obit), "out_bit");
        chk(e->out_delay.upload(odelay), "out_delay");
    }
    chk(e->gen_ptr.upload(gptr), "gen_ptr");
    chk(e->gen_pos.upload(gpos), "gen_pos");
    chk(e->gen_src.upload(gsrc), "gen_src");
    chk(e->gen_delay.upload(gdelay), "gen_delay");
    // thread map: generator neurons leave the one-thread-per-neuron grid
    {
        std::vector<int> upd, gen;
        for (int i = 0; i < e->N; ++i) (e->layers[pop[i]].generator ? gen : upd).push_back(i);
        e->N_upd = (int)upd.size();
        e->N_gen = (int)gen.size();
        bool prefix = true; // updated neurons 0..N_upd-1: no map needed
        for (int i = 0; i < e->N_upd && prefix; ++i) prefix = upd[(size_t)i] == i;
        if (!prefix) chk(e->upd_ids_d.upload(upd), "thread map");
        if (!gen.empty()) chk(e->gen_ids_d.upload(gen), "generator ids");
    }
    chk(e->err.alloc(1), "err");
    chk(e->run_t0.alloc(1), "run_t0");
    chk(e->cursor.alloc(1), "cursor");
    chk(e->ev_cursor.alloc(1), "ev_cursor");
    chk(e->n_events.alloc(1), "n_events");
    if (e->ev_cap > 0) {
        chk(e->ev_t.alloc((size_t)e->ev_cap), "event log");
        chk(e->ev_pos.alloc((size_t)e->ev_cap), "event log");
        chk(e->ev_w.alloc((size_t)e->ev_cap), "event log");
    }

    if (st != NBG_OK) return bail(st);
    st = upload_layers(e);
    if (st == NBG_OK) st = ensure_decay_table(e, 4096);
    if (st == NBG_OK) st = reset_state(e);
    if (st != NBG_OK) return bail(st);
    e->spike_capacity = opt.spike_capacity;
    *out = e;
    return NBG_OK;
}

nbg_status nbg_destroy(nbg_engine *e) {
    if (!e) return NBG_OK;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    if (e->graph) cudaGraphExecDestroy(e->graph);
    if (e->ev0) cudaEventDestroy(e->ev0);
    if (e->evr0) cudaEventDestroy(e->evr0);
    if (e->evr1) cudaEventDestroy(e->evr1);
    if (e->ev1) cudaEventDestroy(e->ev1);
    for (auto ev : e->tev)
        if (ev) cudaEventDestroy(ev);
    if (e->stream) cudaStreamDestroy(e->stream);
    if (e->pin_ids) cudaFreeHost(e->pin_ids);
    if (e->pin_t) cudaFreeHost(e->pin_t);
    delete e;
    return NBG_OK;
}

nbg_status nbg_reset(nbg_engine *e) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    return reset_state(e);
}

nbg_status nbg_reset_neurons(nbg_engine *e, int first, int count) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (first < 0 || count < 0 || (int64_t)first + count > e->N)
        return fail(NBG_ERR_INVALID, "neuron range [%d, %d) outside [0, %d)", first, first + count, e->N);
    if (count == 0) return NBG_OK;
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    const size_t f = (size_t)first, c = (size_t)count;
    NBG_CUDA(cudaMemcpy(e->v.p + f, e->init_v.data() + f, c * sizeof(float), cudaMemcpyHostToDevice));
    NBG_CUDA(cudaMemcpy(e->u.p + f, e->init_u.data() + f, c * sizeof(float), cudaMemcpyHostToDevice));
    NBG_CUDA(cudaMemcpy(e->iext.p + f, e->init_iext.data() + f, c * sizeof(float), cudaMemcpyHostToDevice));
    NBG_CUDA(cudaMemset(e->gexc.p + f, 0, c * sizeof(float)));
    NBG_CUDA(cudaMemset(e->ginh.p + f, 0, c * sizeof(float)));
    const std::vector<int> last0(c, 10000);
    NBG_CUDA(cudaMemcpy(e->last.p + f, last0.data(), c * sizeof(int), cudaMemcpyHostToDevice));
    // pending arrivals: the range's mask words in every ring slot (summary
    // bits left set only make the next drain read a zero word)
    const int w0 = e->woff_host[f], w1 = e->woff_host[f + c];
    if (w1 > w0)
        NBG_CUDA(cudaMemset2D(e->mask.p + w0, (size_t)e->Wt * sizeof(unsigned int), 0,
                              (size_t)(w1 - w0) * sizeof(unsigned int), (size_t)e->D));
    return NBG_OK;
}

nbg_status nbg_run(nbg_engine *e, int steps) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (steps <= 0) return fail(NBG_ERR_INVALID, "Simulation.run steps must be positive");
    NBG_CUDA(cudaSetDevice(e->device));
    const int count = e->ran ? steps : steps + 1;
    if ((int64_t)e->next_t + count > 0x7FFFFFF0ll) return fail(NBG_ERR_INVALID, "simulation time overflow");
    nbg_status st = ensure_decay_table(e, (int64_t)e->next_t + count + 1);
    if (st != NBG_OK) return st;
    // raster capacity for this call
    int64_t cap = e->spike_capacity > 0 ? e->spike_capacity
                                        : std::min<int64_t>((int64_t)e->N * count, (int64_t)1 << 26);
    cap = std::min<int64_t>(std::max<int64_t>(cap, 1), 0x7FFFFFFF); // 32-bit device cursor
    if ((int64_t)e->out_ids.n < cap) {
        NBG_CUDA(e->out_ids.alloc((size_t)cap));
        NBG_CUDA(e->out_t.alloc((size_t)cap));
    }
    const int ntr = (int)e->trace_ids.size();
    if (ntr > 0 && (int64_t)e->trace.n < (int64_t)count * ntr) NBG_CUDA(e->trace.alloc((size_t)count * ntr));
    const int t0 = e->next_t;
    // external spikes of this call: per-step lists on the device
    std::vector<std::pair<int, int>> ext_due;
    if (!e->ext_pending.empty()) {
        std::vector<std::pair<int, int>> later;
        for (const auto &x : e->ext_pending) {
            if (x.first < t0 + count) {
                ext_due.push_back(x);
                e->ext_keys.erase(((uint64_t)(uint32_t)x.first << 32) | (uint32_t)x.second);
            } else {
                later.push_back(x);
            }
        }
        e->ext_pending.swap(later);
        std::sort(ext_due.begin(), ext_due.end());
    }
    if (!ext_due.empty() || e->ext_ptr_d.p) {
        if ((int64_t)e->ext_ptr_d.n < count + 1) NBG_CUDA(e->ext_ptr_d.alloc((size_t)count + 1));
        if (e->ext_ids_d.n < std::max<size_t>(ext_due.size(), 1))
            NBG_CUDA(e->ext_ids_d.alloc(std::max<size_t>(ext_due.size(), 1)));
        e->ext_ptr_h.assign((size_t)count + 1, 0);
        e->ext_ids_h.resize(ext_due.size());
        for (size_t k = 0; k < ext_due.size(); ++k) {
            e->ext_ptr_h[(size_t)(ext_due[k].first - t0) + 1]++;
            e->ext_ids_h[k] = ext_due[k].second;
        }
        for (int k = 0; k < count; ++k) e->ext_ptr_h[(size_t)k + 1] += e->ext_ptr_h[(size_t)k];
        NBG_CUDA(cudaMemcpyAsync(e->ext_ptr_d.p, e->ext_ptr_h.data(), ((size_t)count + 1) * sizeof(int),
                                 cudaMemcpyHostToDevice, e->stream));
        if (!ext_due.empty())
            NBG_CUDA(cudaMemcpyAsync(e->ext_ids_d.p, e->ext_ids_h.data(), ext_due.size() * sizeof(int),
                                     cudaMemcpyHostToDevice, e->stream));
    }
    NBG_CUDA(cudaMemcpyAsync(e->run_t0.p, &t0, sizeof(int), cudaMemcpyHostToDevice, e->stream));
    NBG_CUDA(cudaMemsetAsync(e->cursor.p, 0, sizeof(unsigned int), e->stream));
    NBG_CUDA(cudaMemsetAsync(e->err.p, 0, sizeof(int), e->stream));
    const NetDev nd = e->dev();

    e->last_upd_ms = 0.0;
    e->last_prop_ms = 0.0;
    NBG_CUDA(cudaEventRecord(e->ev0, e->stream));
    const int B = e->B;
    int64_t launches = 0;
    // pending current events inside this call split it into segments
    std::vector<nbg_engine::CurrentEvent> due;
    {
        std::vector<nbg_engine::CurrentEvent> later;
        for (const auto &c : e->currents) {
            if (c.t < t0) continue; // already past: dropped
            (c.t < t0 + count ? due : later).push_back(c);
        }
        e->currents.swap(later);
    }
    // latched currents due in this call, in time order: after all latches of a
    // step, each touched target's total (float sum over its slots in order)
    if (!e->latches.empty()) {
        std::vector<nbg_engine::LatchEvent> now, later;
        for (const auto &x : e->latches) (x.t < t0 + count ? now : later).push_back(x);
        e->latches.swap(later);
        std::sort(now.begin(), now.end(), [](const nbg_engine::LatchEvent &a, const nbg_engine::LatchEvent &b) {
            return a.t != b.t ? a.t < b.t : a.seq < b.seq;
        });
        std::vector<int> touched;
        for (size_t k = 0; k < now.size();) {
            const int t = now[k].t;
            touched.clear();
            for (; k < now.size() && now[k].t == t; ++k) {
                e->cur_latch[(size_t)now[k].slot] = now[k].value;
                const int j = (int)(std::upper_bound(e->cur_tgt_ptr.begin(), e->cur_tgt_ptr.end(), now[k].slot) -
                                    e->cur_tgt_ptr.begin()) - 1;
                touched.push_back(j);
            }
            std::sort(touched.begin(), touched.end());
            touched.erase(std::unique(touched.begin(), touched.end()), touched.end());
            for (int j : touched) {
                float total = 0.0f;
                for (int q = e->cur_tgt_ptr[j]; q < e->cur_tgt_ptr[j + 1]; ++q) total += e->cur_latch[(size_t)q];
                due.push_back({t, j, total});
            }
        }
        std::stable_sort(due.begin(), due.end(), [](const nbg_engine::CurrentEvent &a,
                                                    const nbg_engine::CurrentEvent &b) { return a.t < b.t; });
    }
    const int t_end = t0 + count;
    if (e->use_graph && due.empty()) {
        // the whole call as one graph: nfull blocks of B steps and a tail block
        const int nfull = count / B, tail = count % B;
        const int nblocks = nfull + (tail ? 1 : 0);
        nbg_status ps = ensure_timing_events(e, nblocks);
        if (ps != NBG_OK) return ps;
        if (!e->graph || e->graph_blocks != nfull || e->graph_tail != tail || e->graph_B != B ||
            e->graph_threads != e->threads || std::memcmp(&e->graph_nd, &nd, sizeof(NetDev)) != 0) {
            if (e->graph) {
                cudaGraphExecDestroy(e->graph);
                e->graph = nullptr;
            }
            cudaGraph_t g;
            NBG_CUDA(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
            for (int k = 0; k < nfull; ++k) launch_block(e, nd, B, k * B, k, true);
            if (tail) launch_block(e, nd, tail, nfull * B, nfull, true);
            NBG_CUDA(cudaStreamEndCapture(e->stream, &g));
            cudaError_t ie = cudaGraphInstantiate(&e->graph, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) return fail(NBG_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ie));
            e->graph_blocks = nfull;
            e->graph_tail = tail;
            e->graph_B = B;
            e->graph_threads = e->threads;
            e->graph_nd = nd;
        }
        NBG_CUDA(cudaGraphLaunch(e->graph, e->stream));
        nbg_status hs = harvest_timing(e, nblocks);
        if (hs != NBG_OK) return hs;
        launches += nblocks;
    } else {
        // direct launches, split at timed current injections
        nbg_status ps = ensure_timing_events(e, kLaunchChunk);
        if (ps != NBG_OK) return ps;
        int t = t0;
        size_t ci = 0;
        while (t < t_end) {
            while (ci < due.size() && due[ci].t == t) {
                NBG_CUDA(cudaMemcpyAsync(e->iext.p + due[ci].id, &due[ci].value, sizeof(float),
                                         cudaMemcpyHostToDevice, e->stream));
                NBG_CUDA(cudaStreamSynchronize(e->stream)); // the host value is a vector element
                ++ci;
            }
            const int seg_end = ci < due.size() ? due[ci].t : t_end;
            const int seg = seg_end - t;
            const int nblocks = (seg + B - 1) / B;
            int slot = 0;
            for (int k = 0; k < nblocks; ++k) {
                const int bk = std::min(B, seg - k * B);
                launch_block(e, nd, bk, t + k * B - t0, slot++);
                ++launches;
                if (slot == kLaunchChunk) {
                    nbg_status hs = harvest_timing(e, slot);
                    if (hs != NBG_OK) return hs;
                    slot = 0;
                }
            }
            nbg_status hs = harvest_timing(e, slot);
            if (hs != NBG_OK) return hs;
            t = seg_end;
        }
    }
    NBG_CUDA(cudaGetLastError());
    NBG_CUDA(cudaEventRecord(e->ev1, e->stream));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e->ev0, e->ev1);
    e->last_ms = ms;
    e->last_launches = launches;

    int errv = 0;
    NBG_CUDA(cudaMemcpy(&errv, e->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    e->next_t += count;
    e->ran = true;
    if (errv & kErrEventLog) return fail(NBG_ERR_OVERFLOW, "delivered-event log capacity exceeded");
    if (errv & kErrOverflow)
        return fail(NBG_ERR_OVERFLOW, "spike raster capacity (%lld) exceeded in this run call", (long long)cap);
    // raster: the device's unordered (step, id) entries, ordered on the
    // device, downloaded through pinned staging buffers and merged with the
    // external spikes of output neurons
    unsigned ndev = 0;
    NBG_CUDA(cudaMemcpy(&ndev, e->cursor.p, sizeof(ndev), cudaMemcpyDeviceToHost));
    // The step loop has run and the engine's time has moved on, so a failed
    // device ordering must not drop the call's spikes: the unordered entries
    // are then downloaded and ordered on the host instead.
    const int *ord_ids = nullptr, *ord_t = nullptr;
    bool host_order = false;
    {
        unsigned nord = 0;
        if (order_raster(e, ndev, t0, count, &nord) == NBG_OK) { // ordering may have grown ord_ids / ord_t
            ord_ids = e->ord_ids.p;
            ord_t = e->ord_t.p;
        } else {
            cudaGetLastError(); // an allocation failure is not sticky: clear it
            NBG_CUDA(cudaStreamSynchronize(e->stream));
            ord_ids = e->out_ids.p;
            ord_t = e->out_t.p;
            host_order = true;
            e->last_order_launches = -1;
        }
    }
    const auto h0 = std::chrono::steady_clock::now();
    if ((size_t)ndev > e->pin_cap) { // grown by half again when short
        if (e->pin_ids) cudaFreeHost(e->pin_ids);
        if (e->pin_t) cudaFreeHost(e->pin_t);
        e->pin_ids = e->pin_t = nullptr;
        e->pin_cap = 0;
        const size_t cap = (size_t)ndev + (size_t)ndev / 2;
        NBG_CUDA(cudaMallocHost(&e->pin_ids, cap * sizeof(int)));
        NBG_CUDA(cudaMallocHost(&e->pin_t, cap * sizeof(int)));
        e->pin_cap = cap;
    }
    if (ndev > 0) {
        NBG_CUDA(cudaMemcpy(e->pin_ids, ord_ids, ndev * sizeof(int), cudaMemcpyDeviceToHost));
        NBG_CUDA(cudaMemcpy(e->pin_t, ord_t, ndev * sizeof(int), cudaMemcpyDeviceToHost));
    }
    if (host_order && ndev > 1) { // (step, id) order on the host
        std::vector<uint64_t> key((size_t)ndev);
        for (size_t k = 0; k < ndev; ++k)
            key[k] = ((uint64_t)(uint32_t)e->pin_t[k] << 32) | (uint32_t)e->pin_ids[k];
        std::sort(key.begin(), key.end());
        for (size_t k = 0; k < ndev; ++k) {
            e->pin_t[k] = (int)(key[k] >> 32);
            e->pin_ids[k] = (int)(uint32_t)key[k];
        }
    }
    const auto h1 = std::chrono::steady_clock::now();
    {
        std::vector<std::pair<int, int>> ext_rec; // external spikes of recorded neurons, (step, id) order
        for (const auto &x : ext_due)
            if (e->layers[e->pop_host[x.second]].record) ext_rec.push_back(x);
        append_raster(e, e->pin_t, e->pin_ids, (size_t)ndev, ext_rec);
    }
    const auto h2 = std::chrono::steady_clock::now();
    e->last_download_ms = std::chrono::duration<double, std::milli>(h1 - h0).count();
    e->last_append_ms = std::chrono::duration<double, std::milli>(h2 - h1).count();
    if (ntr > 0) {
        const size_t rb = e->trace_rows.size();
        e->trace_rows.resize(rb + (size_t)count * ntr);
        NBG_CUDA(cudaMemcpy(e->trace_rows.data() + rb, e->trace.p, (size_t)count * ntr * sizeof(float),
                            cudaMemcpyDeviceToHost));
        e->trace_nrows += count;
    }
    if (e->ev_cap > 0) {
        unsigned long long nev = 0;
        NBG_CUDA(cudaMemcpy(&nev, e->ev_cursor.p, sizeof(nev), cudaMemcpyDeviceToHost));
        std::vector<int> et((size_t)nev), ep((size_t)nev);
        std::vector<float> ew((size_t)nev);
        if (nev) {
            NBG_CUDA(cudaMemcpy(et.data(), e->ev_t.p, nev * sizeof(int), cudaMemcpyDeviceToHost));
            NBG_CUDA(cudaMemcpy(ep.data(), e->ev_pos.p, nev * sizeof(int), cudaMemcpyDeviceToHost));
            NBG_CUDA(cudaMemcpy(ew.data(), e->ev_w.p, nev * sizeof(float), cudaMemcpyDeviceToHost));
        }
        for (size_t k = 0; k < nev; ++k) {
            e->log_t.push_back(et[k]);
            e->log_conn.push_back(e->csc_orig[ep[k]]);
            e->log_w.push_back(ew[k]);
        }
        NBG_CUDA(cudaMemset(e->ev_cursor.p, 0, sizeof(unsigned long long)));
    }
    return NBG_OK;
}

nbg_status nbg_next_time(const nbg_engine *e, int *t) {
    if (!e || !t) return fail(NBG_ERR_INVALID, "null argument");
    *t = e->next_t;
    return NBG_OK;
}
nbg_status nbg_num_neurons(const nbg_engine *e, int *n) {
    if (!e || !n) return fail(NBG_ERR_INVALID, "null argument");
    *n = e->N;
    return NBG_OK;
}
nbg_status nbg_num_synapses(const nbg_engine *e, int64_t *s) {
    if (!e || !s) return fail(NBG_ERR_INVALID, "null argument");
    *s = e->S;
    return NBG_OK;
}
nbg_status nbg_block_steps(const nbg_engine *e, int *b) {
    if (!e || !b) return fail(NBG_ERR_INVALID, "null argument");
    *b = e->B;
    return NBG_OK;
}

nbg_status nbg_set_launch(nbg_engine *e, int threads_per_block, int block_steps) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (threads_per_block <= 0 || threads_per_block % 32 || threads_per_block > 256)
        return fail(NBG_ERR_INVALID, "threads_per_block must be a multiple of 32 and <= 256");
    if (block_steps < 0) return fail(NBG_ERR_INVALID, "block_steps must be >= 0");
    const int B = block_steps > 0 ? std::min(block_steps, e->dmin) : e->dmin;
    e->threads = threads_per_block;
    e->B = std::max(1, std::min(B, kMaxBlockSteps));
    if (e->graph) {
        cudaGraphExecDestroy(e->graph);
        e->graph = nullptr;
    }
    return NBG_OK;
}

nbg_status nbg_get_state(nbg_engine *e, int field, float *out) {
    if (!e || !out) return fail(NBG_ERR_INVALID, "null argument");
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    const size_t bytes = (size_t)e->N * sizeof(float);
    switch (field) {
    case NBG_FIELD_V: NBG_CUDA(cudaMemcpy(out, e->v.p, bytes, cudaMemcpyDeviceToHost)); break;
    case NBG_FIELD_U: NBG_CUDA(cudaMemcpy(out, e->u.p, bytes, cudaMemcpyDeviceToHost)); break;
    case NBG_FIELD_G_EXC: NBG_CUDA(cudaMemcpy(out, e->gexc.p, bytes, cudaMemcpyDeviceToHost)); break;
    case NBG_FIELD_G_INH: NBG_CUDA(cudaMemcpy(out, e->ginh.p, bytes, cudaMemcpyDeviceToHost)); break;
    case NBG_FIELD_I_EXT: NBG_CUDA(cudaMemcpy(out, e->iext.p, bytes, cudaMemcpyDeviceToHost)); break;
    case NBG_FIELD_LAST_SPIKE: {
        std::vector<int> tmp((size_t)e->N);
        NBG_CUDA(cudaMemcpy(tmp.data(), e->last.p, (size_t)e->N * sizeof(int), cudaMemcpyDeviceToHost));
        for (int i = 0; i < e->N; ++i) out[i] = (float)tmp[i];
        break;
    }
    default: return fail(NBG_ERR_INVALID, "unknown state field %d", field);
    }
    return NBG_OK;
}

nbg_status nbg_set_state(nbg_engine *e, int field, const float *in) {
    if (!e || !in) return fail(NBG_ERR_INVALID, "null argument");
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    const size_t bytes = (size_t)e->N * sizeof(float);
    switch (field) {
    case NBG_FIELD_V: NBG_CUDA(cudaMemcpy(e->v.p, in, bytes, cudaMemcpyHostToDevice)); break;
    case NBG_FIELD_U: NBG_CUDA(cudaMemcpy(e->u.p, in, bytes, cudaMemcpyHostToDevice)); break;
    case NBG_FIELD_I_EXT: NBG_CUDA(cudaMemcpy(e->iext.p, in, bytes, cudaMemcpyHostToDevice)); break;
    default: return fail(NBG_ERR_INVALID, "state field %d is not writable", field);
    }
    return NBG_OK;
}

nbg_status nbg_num_spikes(nbg_engine *e, int64_t *n) {
    if (!e || !n) return fail(NBG_ERR_INVALID, "null argument");
    *n = (int64_t)e->spk_id.size();
    return NBG_OK;
}

nbg_status nbg_get_spikes(nbg_engine *e, int32_t *times, int32_t *ids, int64_t capacity) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    const int64_t n = (int64_t)e->spk_id.size();
    if (capacity < n) return fail(NBG_ERR_OVERFLOW, "need capacity %lld", (long long)n);
    if (n && times) std::memcpy(times, e->spk_t.data(), n * sizeof(int32_t));
    if (n && ids) std::memcpy(ids, e->spk_id.data(), n * sizeof(int32_t));
    return NBG_OK;
}

nbg_status nbg_get_spikes_from(nbg_engine *e, int64_t offset, int64_t count, int32_t *times, int32_t *ids) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    const int64_t n = (int64_t)e->spk_id.size();
    if (offset < 0 || count < 0 || offset + count > n)
        return fail(NBG_ERR_INVALID, "spike range [%lld, %lld) outside the %lld recorded spikes", (long long)offset,
                    (long long)(offset + count), (long long)n);
    if (count && times) std::memcpy(times, e->spk_t.data() + offset, count * sizeof(int32_t));
    if (count && ids) std::memcpy(ids, e->spk_id.data() + offset, count * sizeof(int32_t));
    return NBG_OK;
}

nbg_status nbg_set_layer_record(nbg_engine *e, int layer, int record) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (layer < 0 || layer >= (int)e->layers.size()) return fail(NBG_ERR_INVALID, "layer %d out of range", layer);
    if ((e->layers[layer].record != 0) == (record != 0)) return NBG_OK;
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    e->layers[layer].record = record != 0 ? 1 : 0;
    NBG_CUDA(cudaMemcpy(e->d_layers.p + layer, &e->layers[layer], sizeof(LayerDev), cudaMemcpyHostToDevice));
    return NBG_OK;
}

nbg_status nbg_get_decay_table(nbg_engine *e, int rule, int which, int64_t capacity, float *out, int64_t *len) {
    if (!e || !len) return fail(NBG_ERR_INVALID, "null argument");
    if (rule < 0 || rule >= e->n_rules || which < 0 || which > 1)
        return fail(NBG_ERR_INVALID, "no decay table (rule %d, trace %d)", rule, which);
    nbg_status st = ensure_decay_table(e, 1);
    if (st != NBG_OK) return st;
    *len = e->dtab_len;
    if (out && capacity > 0) {
        NBG_CUDA(cudaSetDevice(e->device));
        const int64_t n = std::min<int64_t>(capacity, e->dtab_len);
        std::vector<float2> row((size_t)n);
        NBG_CUDA(cudaMemcpy(row.data(), e->dtab.p + (size_t)rule * e->dtab_len, n * sizeof(float2),
                            cudaMemcpyDeviceToHost));
        for (int64_t k = 0; k < n; ++k) out[k] = which ? row[(size_t)k].y : row[(size_t)k].x;
    }
    return NBG_OK;
}

nbg_status nbg_clear_spikes(nbg_engine *e) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    e->spk_t.clear();
    e->spk_id.clear();
    return NBG_OK;
}

nbg_status nbg_num_events(nbg_engine *e, int64_t *n) {
    if (!e || !n) return fail(NBG_ERR_INVALID, "null argument");
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    unsigned long long v = 0;
    NBG_CUDA(cudaMemcpy(&v, e->n_events.p, sizeof(v), cudaMemcpyDeviceToHost));
    *n = (int64_t)v;
    return NBG_OK;
}

nbg_status nbg_get_weights(nbg_engine *e, float *w, float *apre, float *apost, int32_t *last) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    const size_t S = (size_t)e->S;
    if (S == 0) return NBG_OK;
    if (e->plastic) {
        std::vector<SynRec> r(S);
        NBG_CUDA(cudaMemcpy(r.data(), e->rec.p, S * sizeof(SynRec), cudaMemcpyDeviceToHost));
        for (size_t p = 0; p < S; ++p) {
            const int64_t o = e->csc_orig[p];
            if (w) w[o] = r[p].w;
            if (apre) apre[o] = r[p].apre;
            if (apost) apost[o] = r[p].apost;
            if (last) last[o] = r[p].last;
        }
        return NBG_OK;
    }
    std::vector<SynStatic> r(S); // no plastic synapse: traces are identically zero
    NBG_CUDA(cudaMemcpy(r.data(), e->wst.p, S * sizeof(SynStatic), cudaMemcpyDeviceToHost));
    for (size_t p = 0; p < S; ++p) {
        const int64_t o = e->csc_orig[p];
        if (w) w[o] = r[p].w;
        if (apre) apre[o] = 0.0f;
        if (apost) apost[o] = 0.0f;
        if (last) last[o] = 0;
    }
    return NBG_OK;
}

nbg_status nbg_set_weight(nbg_engine *e, int64_t conn, float w) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (conn < 0 || conn >= e->S) return fail(NBG_ERR_INVALID, "connection index %lld out of range", (long long)conn);
    if (!std::isfinite(w)) return fail(NBG_ERR_INVALID, "weight must be finite");
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    const int64_t p = e->orig_pos[conn];
    float *dst = e->plastic ? &e->rec.p[p].w : &e->wst.p[p].w;
    NBG_CUDA(cudaMemcpy(dst, &w, sizeof(float), cudaMemcpyHostToDevice));
    NBG_CUDA(cudaMemcpy(e->init_w_d.p + p, &w, sizeof(float), cudaMemcpyHostToDevice));
    e->init_w[p] = w;
    return NBG_OK;
}

nbg_status nbg_set_weights(nbg_engine *e, const float *w) {
    if (!e || (!w && e->S > 0)) return fail(NBG_ERR_INVALID, "null argument");
    for (int64_t s = 0; s < e->S; ++s)
        if (!std::isfinite(w[s])) return fail(NBG_ERR_INVALID, "weight %lld is not finite", (long long)s);
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    for (int64_t s = 0; s < e->S; ++s) e->init_w[e->orig_pos[s]] = w[s];
    if (e->S > 0) {
        NBG_CUDA(cudaMemcpy(e->init_w_d.p, e->init_w.data(), e->S * sizeof(float), cudaMemcpyHostToDevice));
        NBG_CUDA(reset_synapses(e, false)); // weights only: the STDP traces stay
    }
    return NBG_OK;
}

nbg_status nbg_set_current_at(nbg_engine *e, int t, int id, float value) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (id < 0 || id >= e->N) return fail(NBG_ERR_INVALID, "neuron id %d out of range", id);
    if (t < e->next_t) return fail(NBG_ERR_INVALID, "time %d is in the past (next step %d)", t, e->next_t);
    if (e->layers[e->pop_host[id]].generator)
        return fail(NBG_ERR_UNSUPPORTED, "neuron %d belongs to a source-free PoissonRate layer (evaluated inline)", id);
    if (!std::isfinite(value)) return fail(NBG_ERR_INVALID, "current must be finite");
    nbg_engine::CurrentEvent c{t, id, value};
    auto it = std::upper_bound(e->currents.begin(), e->currents.end(), c,
                               [](const nbg_engine::CurrentEvent &a, const nbg_engine::CurrentEvent &b) {
                                   return a.t < b.t;
                               });
    e->currents.insert(it, c);
    return NBG_OK;
}

nbg_status nbg_add_external_spikes(nbg_engine *e, int64_t n, const int32_t *times, const int32_t *ids) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (n < 0 || (n > 0 && (!times || !ids))) return fail(NBG_ERR_INVALID, "bad external spike arrays");
    std::vector<uint64_t> keys((size_t)n);
    for (int64_t k = 0; k < n; ++k) {
        const int t = times[k], id = ids[k];
        if (id < 0 || id >= e->N) return fail(NBG_ERR_INVALID, "external spike %lld: neuron id %d out of range",
                                              (long long)k, id);
        if (t < e->next_t)
            return fail(NBG_ERR_INVALID, "external spike %lld: time %d is in the past (next step %d)", (long long)k,
                        t, e->next_t);
        if (e->layers[e->pop_host[id]].model != NBG_MODEL_INPUT_SPIKE)
            return fail(NBG_ERR_UNSUPPORTED, "external spike %lld: neuron %d is not an input-spike neuron",
                        (long long)k, id);
        keys[(size_t)k] = ((uint64_t)(uint32_t)t << 32) | (uint32_t)id;
    }
    std::unordered_set<uint64_t> seen;
    for (int64_t k = 0; k < n; ++k)
        if (e->ext_keys.count(keys[(size_t)k]) || !seen.insert(keys[(size_t)k]).second)
            return fail(NBG_ERR_UNSUPPORTED, "external spike %lld: neuron %d already spikes at step %d",
                        (long long)k, ids[k], times[k]);
    for (int64_t k = 0; k < n; ++k) {
        e->ext_keys.insert(keys[(size_t)k]);
        e->ext_pending.emplace_back(times[k], ids[k]);
    }
    return NBG_OK;
}

nbg_status nbg_add_external_currents(nbg_engine *e, int64_t n, const int32_t *times, const int32_t *ids,
                                     const float *currents) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (n < 0 || (n > 0 && (!times || !ids || !currents))) return fail(NBG_ERR_INVALID, "bad external current arrays");
    for (int64_t k = 0; k < n; ++k) {
        if (ids[k] < 0 || ids[k] >= e->N)
            return fail(NBG_ERR_INVALID, "external current %lld: neuron id %d out of range", (long long)k, ids[k]);
        if (times[k] < e->next_t)
            return fail(NBG_ERR_INVALID, "external current %lld: time %d is in the past (next step %d)",
                        (long long)k, times[k], e->next_t);
        if (e->layers[e->pop_host[ids[k]]].model != NBG_MODEL_INPUT_CURRENT)
            return fail(NBG_ERR_UNSUPPORTED, "external current %lld: neuron %d is not an input-current neuron",
                        (long long)k, ids[k]);
        if (!std::isfinite(currents[k]))
            return fail(NBG_ERR_INVALID, "external current %lld: value must be finite", (long long)k);
        if ((int64_t)times[k] + 65535 > 0x7FFFFFF0ll) return fail(NBG_ERR_INVALID, "external current time overflow");
    }
    for (int64_t k = 0; k < n; ++k) {
        const int src = ids[k];
        for (int q = e->cur_out_ptr[src]; q < e->cur_out_ptr[src + 1]; ++q) {
            const int j = e->cur_out_tgt[q];
            if (e->layers[e->pop_host[j]].generator) continue; // unreachable: a current input is an input
            e->latches.push_back({times[k] + e->cur_out_delay[q], e->cur_out_slot[q], currents[k], e->latch_seq++});
        }
    }
    return NBG_OK;
}

nbg_status nbg_set_trace(nbg_engine *e, int n, const int32_t *ids) {
    if (!e || (n > 0 && !ids) || n < 0) return fail(NBG_ERR_INVALID, "bad trace arguments");
    NBG_CUDA(cudaSetDevice(e->device));
    NBG_CUDA(cudaStreamSynchronize(e->stream));
    std::vector<int> slot((size_t)e->N, -1);
    for (int k = 0; k < n; ++k) {
        if (ids[k] < 0 || ids[k] >= e->N) return fail(NBG_ERR_INVALID, "trace id %d out of range", ids[k]);
        if (slot[ids[k]] >= 0) return fail(NBG_ERR_INVALID, "trace id %d listed twice", ids[k]);
        slot[ids[k]] = k;
    }
    NBG_CUDA(e->trace_slot.upload(slot));
    e->trace_ids.assign(ids, ids + n);
    e->trace_rows.clear();
    e->trace_nrows = 0;
    return NBG_OK;
}

nbg_status nbg_num_trace_rows(nbg_engine *e, int64_t *rows) {
    if (!e || !rows) return fail(NBG_ERR_INVALID, "null argument");
    *rows = e->trace_nrows;
    return NBG_OK;
}

nbg_status nbg_get_traces(nbg_engine *e, float *out) {
    if (!e || !out) return fail(NBG_ERR_INVALID, "null argument");
    if (!e->trace_rows.empty()) std::memcpy(out, e->trace_rows.data(), e->trace_rows.size() * sizeof(float));
    return NBG_OK;
}

nbg_status nbg_num_logged_events(nbg_engine *e, int64_t *n) {
    if (!e || !n) return fail(NBG_ERR_INVALID, "null argument");
    *n = (int64_t)e->log_t.size();
    return NBG_OK;
}

nbg_status nbg_get_logged_events(nbg_engine *e, int32_t *t, int64_t *conn, float *w) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    const size_t n = e->log_t.size();
    if (n && t) std::memcpy(t, e->log_t.data(), n * sizeof(int32_t));
    if (n && conn) std::memcpy(conn, e->log_conn.data(), n * sizeof(int64_t));
    if (n && w) std::memcpy(w, e->log_w.data(), n * sizeof(float));
    return NBG_OK;
}

nbg_status nbg_profile(nbg_engine *e, double *total_ms, double *update_ms, double *propagate_ms,
                       int64_t *launches) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (total_ms) *total_ms = e->last_ms;
    if (update_ms) *update_ms = e->last_upd_ms;
    if (propagate_ms) *propagate_ms = e->last_prop_ms;
    if (launches) *launches = e->last_launches;
    return NBG_OK;
}

nbg_status nbg_raster_profile(nbg_engine *e, double *order_ms, double *download_ms, double *append_ms,
                              int64_t *order_launches) {
    if (!e) return fail(NBG_ERR_INVALID, "null engine");
    if (order_ms) *order_ms = e->last_order_ms;
    if (download_ms) *download_ms = e->last_download_ms;
    if (append_ms) *append_ms = e->last_append_ms;
    if (order_launches) *order_launches = e->last_order_launches;
    return NBG_OK;
}

} // extern "C"
