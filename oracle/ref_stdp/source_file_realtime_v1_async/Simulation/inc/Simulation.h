/* Harness stand-in (test infrastructure only) for the reference's
 * Simulation/inc/Simulation.h.  The pair-STDP rule reads one member of the
 * simulation it is given -- the base time step, Sim->basetimesteps
 * (LearningRule/src/Rule/STDP.cpp:23,46) -- and the full class pulls in the
 * event queue, drivers, dense runtime and CUDA headers.  This header gives
 * the same member with the same type (Simulation.h:90 in the reference)
 * and nothing else. */
#pragma once

class Simulation {
  public:
    float basetimesteps;
};
