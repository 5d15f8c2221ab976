// Replica exchange on the device (the reference's ReplicaExchange,
// src/main.cpp:147-317): the energies, the swaps, the Metropolis decisions
// (FP64), the draws from the replica-exchange Threefry stream and the undo of
// rejected swaps are all kernels on the engine stream, so an exchange needs
// no host round trip and is captured into the round graph.
#pragma once
#include <cstdint>
#include <vector>

#include "engine.h"

namespace ug {

// The plan of an engine's batch: alternating swap sets of system pairs.
struct RemdDev {
    int n_sys = 0;
    int n_sets = 0;
    int criterion = 0;               // 0 or 1 (src/main.cpp:276-313)
    uint32_t seed = 0;               // key word 0 of the exchange stream (stream id 1)
    const int2* pairs = nullptr;     // all sets' pairs, set after set
    const int* set_off = nullptr;    // n_sets + 1
    unsigned long long* attempt = nullptr;  // exchanges made so far: selects the set (attempt % n_sets)
    // the round the draws are keyed by: round0 + (attempt + 1) * interval, or
    // round_val when round_fixed (a single exchange called with its round)
    unsigned long long round0 = 0, round_val = 0;
    int interval = 0, round_fixed = 0;
    int* cur = nullptr;              // the current set: first pair, pair count
    int* flag = nullptr;             // per pair slot of the current set: 1 = swap in the next swap kernel
    double* lb_old = nullptr;        // per system: -E / T before the swaps
    int* replica = nullptr;          // per system: index of the replica it holds
    unsigned* n_attempt = nullptr;   // per pair of all sets
    unsigned* n_success = nullptr;   // per pair of all sets
    int* accepted = nullptr;         // per pair slot of the current set: 1 accepted, 0 rejected
};

class Remd {
public:
    // sets: the swap sets, each a list of (s1, s2) pairs of systems with equal
    // atom counts, no system twice in a set; interval: rounds between
    // exchanges (0: exchanges only when called); round0: the round counter at
    // the first round after this call.
    Remd(Engine& e, const std::vector<std::vector<std::pair<int, int>>>& sets, uint32_t seed, int criterion,
         int interval, unsigned long long round0);
    // enqueue one exchange on the engine stream (energies, swaps, decisions,
    // undo); round_fixed >= 0 keys the draws by that round instead of the
    // plan's schedule
    void enqueue(long long round_fixed = -1);
    int interval() const { return d_.interval; }
    int max_pairs() const { return max_pairs_; }
    // host copies: replica index per system; per pair attempts, successes;
    // exchanges made; the last exchange's accept flags (current set order)
    void read(std::vector<int>& replica, std::vector<unsigned>& n_att, std::vector<unsigned>& n_succ,
              unsigned long long& attempts, std::vector<int>& last_accepted, int& last_set);
    // device state that an overflow rollback restores (replica indices,
    // counters): copy to / from the snapshot area
    void snapshot(bool restore);

private:
    Engine& e_;
    RemdDev d_;
    int max_pairs_ = 0, n_pair_total_ = 0;
    int* snap_ = nullptr;  // replica (n_sys) + n_attempt + n_success (pairs) + attempt (2 ints)
};

}  // namespace ug
