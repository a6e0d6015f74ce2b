// Autotuner of the fused gate sweeps (tune.cpp).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "sim.h"

namespace kbwg {

struct TuneResult {
    uint32_t tile_k = 0;      // tile size chosen (2^tile_k amplitudes); 0 = one kernel per gate
    uint32_t depth = 0;       // fusion depth chosen
    uint32_t candidates = 0;  // settings timed
    double ms = 0.0;          // device time of one application with the chosen settings
    double default_ms = 0.0;  // the same with the default settings (0: the default was not a candidate)
    bool cached = false;      // taken from the process-wide cache, nothing timed
};

// Time the circuit under every (tile size, fusion depth) pair the handle
// supports, set the fastest on the handle, restore the state.  Returns a
// KBWG_* code; err holds the reason of a failure.
int32_t autotune(Sim &s, const std::vector<GateDesc> &gates, uint32_t reps, TuneResult &out, std::string &err);

}  // namespace kbwg
