// Monte Carlo pivot and jump moves over a batch of systems
// (MultipleMonteCarloSampler, src/monte_carlo_sampler.cpp:1-308).
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "engine.h"

namespace ug {

// Per-system move tables on the device (concatenated over systems).
struct McDev {
    int n_sys;
    const unsigned* seed;    // per system: the thermostat seed (the reference's sys.random_seed)
    // pivot moves: per system [piv_off[s], piv_off[s+1]) locations
    const int* piv_off;
    const int* piv_atom;     // loc * 5: previous C, N, CA, C, next N (global atom indices)
    const int* piv_range;    // loc * 2: [first, end) of the atoms moved with the C-terminal side
    const int* piv_layer;    // loc: proposal layer (index into the system's table)
    const int* tab_off;      // per system: offset of its proposal tables (layers x n_bin x n_bin)
    const int* n_bin;        // per system
    const float* prop_pot;   // normalised -log proposal probability
    const float* prop_cdf;   // cumulative proposal probability
    // jump moves: per system [jmp_off[s], jmp_off[s+1]) chains
    const int* jmp_off;
    const int* jmp_range;    // chain * 2: [first atom, end)
    const float* jmp_trans;  // chain: translation width
    const float* jmp_rot;    // chain: rotation width (radians)
    const float* prob_mod;   // per system: the jump move's log-probability ratio
    float* delta_lprob;      // per system output: log-probability ratio of the proposal
    float* u_accept;         // per system output: the uniform the acceptance test uses
};

// The move samplers of every system of an engine's batch, read from
// /input/pivot_moves and /input/jump_moves of each configuration.
class McSampler {
public:
    McSampler(Engine& e, const std::vector<std::string>& paths);
    bool any_pivot = false, any_jump = false;
    std::vector<char> has_pivot, has_jump;  // per system
    // Per sampler (pivot, then jump) and system: success and attempt counts
    // since the last reset.
    std::vector<unsigned long long> success[2], attempt[2];
    // One step of each sampler for every system that has it
    // (monte_carlo_step, src/monte_carlo_sampler.cpp:248-276): energies, a
    // proposal from the sampler's random stream keyed by (system seed,
    // round), energies again, Metropolis test at the system's temperature,
    // rejected proposals undone.  accepted[2 * s + k] (may be null): 1, 0,
    // or -1 when system s has no sampler k.
    void step(uint64_t round, int* accepted);

private:
    Engine& e_;
    McDev d_{};
    float* saved_ = nullptr;
};

}  // namespace ug
