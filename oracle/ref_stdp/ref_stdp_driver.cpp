/* Reference pair-STDP driver -- TEST INFRASTRUCTURE ONLY.
 *
 * Linked with the reference's own STDP.cpp, STDP_State.cpp, SynapseState.cpp,
 * LearningRule.cpp, WithPostSynaptic.cpp, Interconnections.cpp and Neuron.cpp
 * (compiled from the reference tree by oracle/ref_stdp/Makefile into
 * oracle/_ref/libnbg_ref_stdp.so).  It sets up one post-synaptic neuron with
 * n plastic input connections the way the reference's own test fixture does
 * (tests/model_codegen/pair_stdp_gpu_trajectory.cpp:31-52: the rule from its
 * parameter map, InitState, the connections' LearningRuleIndex_withPost and
 * the neuron's PostSynapticLearning tables), then replays an event schedule:
 * at every tick, the pre-synaptic arrivals of that tick in connection order
 * (STDP::ApplyPreSynaticSpike), then the neuron's spike if it fires
 * (STDP::ApplyPostSynaticSpike), the order of PropogatedSpikeGroup events
 * before the neuron update within one time step.  The weights after every
 * tick and the final trace state come back to the caller. */
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "boost/any.hpp"
#include "../source_file_realtime_v1_async/LearningRule/inc/Rule/STDP.h"
#include "../source_file_realtime_v1_async/LearningRule/inc/SynapseState.h"
#include "../source_file_realtime_v1_async/Neuron/inc/Neuron.h"
#include "../source_file_realtime_v1_async/Simulation/inc/Simulation.h"
#include "../source_file_realtime_v1_async/connections/inc/Interconnections.h"

/* Openmp/src defines the OpenMP queue count with the simulation; Neuron's
 * destructor reads it (one queue here). */
int NumberOfOpenMPQueues = 1;

extern "C" int nbgref_stdp_run(int n_conn, const float *w0, const float *wmax, float max_ltp, float ltp_tau,
                               float max_ltd, float ltd_tau, float basetimestep, int n_ticks,
                               const unsigned char *pre, const unsigned char *post, float *w_traj, float *apre,
                               float *apost, int *last_update) {
    if (n_conn <= 0 || n_ticks <= 0) return 1;
    std::map<std::string, boost::any> params;
    params["Max_LTP"] = max_ltp;
    params["LTP_tau"] = ltp_tau;
    params["Max_LTD"] = max_ltd;
    params["LTD_tau"] = ltd_tau;
    std::unique_ptr<STDP> rule(new STDP(params));
    rule->LearningRuleID = 0;
    rule->InitState(n_conn, 1, basetimestep);

    std::vector<Interconnections> conn((size_t)n_conn);
    Neuron target;
    target.NumberOfRule = 1;
    target.PostSynapticLearning_Number = new int[1]{n_conn};
    target.PostSynapticLearning = new Interconnections **[1]{};
    target.PostSynapticLearning[0] = new Interconnections *[n_conn];
    target.IndexOfInputLearningIndex[0] = new int *[1]{};
    target.IndexOfInputLearningIndex[0][0] = new int[n_conn];
    for (int k = 0; k < n_conn; ++k) {
        conn[k].weight = w0[k];
        conn[k].maximum_weight = wmax[k];
        conn[k].TargetNeuron = &target;
        conn[k].LearningRuleIndex_withPost = k;
        target.PostSynapticLearning[0][k] = &conn[k];
        target.IndexOfInputLearningIndex[0][0][k] = k;
    }
    Simulation sim;
    sim.basetimesteps = basetimestep;
    for (int t = 0; t < n_ticks; ++t) {
        for (int k = 0; k < n_conn; ++k)
            if (pre[(size_t)t * n_conn + k]) rule->ApplyPreSynaticSpike(&conn[k], t, &sim);
        if (post[t]) rule->ApplyPostSynaticSpike(&target, t, &sim);
        for (int k = 0; k < n_conn; ++k) w_traj[(size_t)t * n_conn + k] = conn[k].weight;
    }
    const SynapseState *st = rule->State;
    for (int k = 0; k < n_conn; ++k) {
        apre[k] = st->StateValue[k * st->NumberOfState + 0];
        apost[k] = st->StateValue[k * st->NumberOfState + 1];
        last_update[k] = st->LastUpdate[k];
    }
    return 0;
}
