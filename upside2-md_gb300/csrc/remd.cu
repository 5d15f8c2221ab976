// Replica exchange on the device (src/main.cpp:243-316).
//
// One exchange, criterion 0: energies at the current coordinates; every pair
// of the current swap set exchanges its coordinates; energies again; each
// swap whose change of log Boltzmann factors, (new1 + new2) - (old1 + old2)
// with lb = -E / T, is negative and fails the test exp(diff) >= u is undone.
// Criterion 1: one energy evaluation, and each pair with diff = lb2 - lb1 >= 0
// or exp(diff) >= u swaps.  A uniform is drawn only for a negative diff, in
// pair order, from the exchange stream: Threefry-4x32-20 with key (seed, 1,
// 0, 0) and counter (round lo, round hi, 0, k) for the k-th draw, the first
// word as r123::u01<float> (src/random.h:19-52).  The sets alternate
// (attempt % n_sets).  Momenta stay with their systems; coordinates and the
// replica index move.  Energies are the engine's FP64 sums and the acceptance
// arithmetic is FP64.
#include <algorithm>
#include <stdexcept>

#include "dev_math.cuh"
#include "launch.cuh"
#include "remd.h"

namespace ug {

namespace {

__device__ __forceinline__ unsigned long long remd_round(const RemdDev& r) {
    return r.round_fixed ? r.round_val : r.round0 + (*r.attempt + 1ull) * (unsigned long long)r.interval;
}

// the k-th uniform of the exchange stream at `round`
__device__ __forceinline__ float remd_uniform(const RemdDev& r, unsigned long long round, unsigned k) {
    uint32_t key[4] = {r.seed, 1u, 0u, 0u};
    uint32_t ctr[4] = {uint32_t(round & 0xffffffffu), uint32_t(round >> 32), 0u, k};
    uint32_t bits[4];
    threefry4x32(ctr, key, bits);
    return u01f(bits[0]);
}

// Decisions of the current set by one warp, pairs in order, 32 at a time: a
// lane draws only when its diff is negative, the draw index being the number
// of earlier pairs that drew.  swap_if_accept: criterion 1 (flag = accept);
// else criterion 0 (flag = reject, the swap to undo).
__device__ void remd_decide(const RemdDev& r, const double* __restrict__ lb_new, bool criterion1) {
    const int lane = threadIdx.x;
    const int lo = r.cur[0], n = r.cur[1];
    const unsigned long long round = remd_round(r);
    unsigned drawn = 0;
    for (int k0 = 0; k0 < n; k0 += 32) {
        const int k = k0 + lane;
        double diff = 0.0;
        int2 p = make_int2(0, 0);
        if (k < n) {
            p = r.pairs[lo + k];
            if (criterion1) diff = r.lb_old[p.y] - r.lb_old[p.x];
            else diff = (lb_new[p.x] + lb_new[p.y]) - (r.lb_old[p.x] + r.lb_old[p.y]);
        }
        const bool draw = k < n && diff < 0.0;
        const unsigned mask = __ballot_sync(0xffffffffu, draw);
        if (k < n) {
            bool accept = true;
            if (draw) {
                const unsigned idx = drawn + __popc(mask & ((1u << lane) - 1u));
                const double u = double(remd_uniform(r, round, idx));
                accept = criterion1 ? exp(diff) >= u : !(exp(diff) < u);
            }
            r.flag[k] = criterion1 ? (accept ? 1 : 0) : (accept ? 0 : 1);
            r.accepted[k] = accept ? 1 : 0;
            r.n_attempt[lo + k] += 1u;
            if (accept) r.n_success[lo + k] += 1u;
        }
        drawn += __popc(mask);
    }
    __syncwarp();
    if (lane == 0) *r.attempt += 1ull;
}

// After the first energy evaluation: pick the set, record -E/T, and either
// mark every pair for the trial swap (criterion 0) or decide (criterion 1).
__global__ void remd_begin_kernel(RemdDev r, const double* __restrict__ energy, const float* __restrict__ temp) {
    grid_dep_entry();
    const int lane = threadIdx.x;
    const int set = int(*r.attempt % (unsigned long long)r.n_sets);
    const int lo = r.set_off[set], n = r.set_off[set + 1] - lo;
    for (int s = lane; s < r.n_sys; s += 32) r.lb_old[s] = -energy[s] / double(temp[s]);
    if (lane == 0) {
        r.cur[0] = lo;
        r.cur[1] = n;
    }
    __syncwarp();
    if (r.criterion == 1) {
        remd_decide(r, nullptr, true);
    } else {
        for (int k = lane; k < n; k += 32) r.flag[k] = 1;
    }
}

// After the second energy evaluation (criterion 0): decide, flag the rejected
// swaps for undoing.
__global__ void remd_finish_kernel(RemdDev r, const double* __restrict__ energy, const float* __restrict__ temp,
                                   double* __restrict__ lb_new) {
    grid_dep_entry();
    const int lane = threadIdx.x;
    for (int s = lane; s < r.n_sys; s += 32) lb_new[s] = -energy[s] / double(temp[s]);
    __syncwarp();
    remd_decide(r, lb_new, false);
}

// Block k swaps the coordinates (and replica indices) of the k-th pair of the
// current set when its flag is set.
__global__ void remd_swap_kernel(RemdDev r, const int* __restrict__ atom_off, float* __restrict__ pos) {
    grid_dep_entry();
    const int k = blockIdx.x;
    if (k >= r.cur[1] || !r.flag[k]) return;  // block-uniform
    const int2 p = r.pairs[r.cur[0] + k];
    float* a = pos + 3 * size_t(atom_off[p.x]);
    float* b = pos + 3 * size_t(atom_off[p.y]);
    const int n = 3 * (atom_off[p.x + 1] - atom_off[p.x]);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float t = a[i];
        a[i] = b[i];
        b[i] = t;
    }
    if (threadIdx.x == 0) {
        const int t = r.replica[p.x];
        r.replica[p.x] = r.replica[p.y];
        r.replica[p.y] = t;
    }
}

}  // namespace

Remd::Remd(Engine& e, const std::vector<std::vector<std::pair<int, int>>>& sets, uint32_t seed, int criterion,
           int interval, unsigned long long round0)
    : e_(e) {
    if (sets.empty()) throw Error("replica exchange needs at least one swap set");
    if (criterion != 0 && criterion != 1) throw Error("replica exchange criterion must be 0 or 1");
    if (interval < 0) throw Error("replica exchange interval must be >= 0");
    std::vector<int2> pairs;
    std::vector<int> off{0};
    for (auto& set : sets) {
        std::vector<char> seen(size_t(e.n_sys), 0);
        for (auto& p : set) {
            if (p.first < 0 || p.second < 0 || p.first >= e.n_sys || p.second >= e.n_sys || p.first == p.second)
                throw Error("invalid replica pair");
            if (seen[size_t(p.first)] || seen[size_t(p.second)])
                throw Error("Overlapping indices in swap set.  No replica index can appear more than once in a swap set.");
            seen[size_t(p.first)] = seen[size_t(p.second)] = 1;
            if (e.n_atom[size_t(p.first)] != e.n_atom[size_t(p.second)])
                throw Error("Replica exchange requires all systems have the same number of atoms");
            pairs.push_back(make_int2(p.first, p.second));
        }
        off.push_back(int(pairs.size()));
        max_pairs_ = std::max(max_pairs_, int(set.size()));
    }
    n_pair_total_ = int(pairs.size());
    d_.n_sys = e.n_sys;
    d_.n_sets = int(sets.size());
    d_.criterion = criterion;
    d_.seed = seed;
    d_.interval = interval;
    d_.round0 = round0;
    d_.pairs = pairs.empty() ? nullptr : e.upload(pairs);
    d_.set_off = e.upload(off);
    d_.attempt = e.alloc<unsigned long long>(1);
    d_.cur = e.alloc<int>(2);
    d_.flag = e.alloc<int>(size_t(std::max(1, max_pairs_)));
    d_.accepted = e.alloc<int>(size_t(std::max(1, max_pairs_)));
    d_.lb_old = e.alloc<double>(2 * size_t(e.n_sys));
    std::vector<int> rep(size_t(e.n_sys));
    for (int s = 0; s < e.n_sys; ++s) rep[size_t(s)] = s;
    d_.replica = e.upload(rep);
    d_.n_attempt = e.alloc<unsigned>(size_t(std::max(1, n_pair_total_)));
    d_.n_success = e.alloc<unsigned>(size_t(std::max(1, n_pair_total_)));
    snap_ = e.alloc<int>(size_t(e.n_sys) + 2 * size_t(std::max(1, n_pair_total_)) + 2);
    UG_CK(cudaMemsetAsync(d_.attempt, 0, sizeof(unsigned long long), e.st));
    UG_CK(cudaMemsetAsync(d_.n_attempt, 0, sizeof(unsigned) * size_t(std::max(1, n_pair_total_)), e.st));
    UG_CK(cudaMemsetAsync(d_.n_success, 0, sizeof(unsigned) * size_t(std::max(1, n_pair_total_)), e.st));
    UG_CK(cudaMemsetAsync(d_.cur, 0, 2 * sizeof(int), e.st));
    UG_CK(cudaMemsetAsync(d_.accepted, 0, sizeof(int) * size_t(std::max(1, max_pairs_)), e.st));
    UG_CK(cudaStreamSynchronize(e.st));
}

void Remd::enqueue(long long round_fixed) {
    RemdDev r = d_;
    r.round_fixed = round_fixed >= 0 ? 1 : 0;
    r.round_val = round_fixed >= 0 ? (unsigned long long)round_fixed : 0ull;
    cudaStream_t st = e_.st;
    const int blocks = std::max(1, max_pairs_);
    e_.compute(true);
    ug::launch(remd_begin_kernel, 1, 32, 0, st, r, e_.d_energy, e_.d_temp);
    ug::launch(remd_swap_kernel, blocks, 256, 0, st, r, e_.atom_off_d, e_.d_pos);
    if (d_.criterion == 0) {
        e_.compute(true);
        ug::launch(remd_finish_kernel, 1, 32, 0, st, r, e_.d_energy, e_.d_temp, d_.lb_old + e_.n_sys);
        ug::launch(remd_swap_kernel, blocks, 256, 0, st, r, e_.atom_off_d, e_.d_pos);
    }
    UG_CK(cudaGetLastError());
}

void Remd::read(std::vector<int>& replica, std::vector<unsigned>& n_att, std::vector<unsigned>& n_succ,
                unsigned long long& attempts, std::vector<int>& last_accepted, int& last_set) {
    replica.resize(size_t(d_.n_sys));
    n_att.resize(size_t(n_pair_total_));
    n_succ.resize(size_t(n_pair_total_));
    int cur[2] = {0, 0};
    UG_CK(cudaMemcpyAsync(replica.data(), d_.replica, sizeof(int) * replica.size(), cudaMemcpyDeviceToHost, e_.st));
    if (n_pair_total_) {
        UG_CK(cudaMemcpyAsync(n_att.data(), d_.n_attempt, sizeof(unsigned) * n_att.size(), cudaMemcpyDeviceToHost, e_.st));
        UG_CK(cudaMemcpyAsync(n_succ.data(), d_.n_success, sizeof(unsigned) * n_succ.size(), cudaMemcpyDeviceToHost,
                              e_.st));
    }
    UG_CK(cudaMemcpyAsync(&attempts, d_.attempt, sizeof(unsigned long long), cudaMemcpyDeviceToHost, e_.st));
    UG_CK(cudaMemcpyAsync(cur, d_.cur, sizeof(cur), cudaMemcpyDeviceToHost, e_.st));
    last_accepted.assign(size_t(std::max(1, max_pairs_)), 0);
    UG_CK(cudaMemcpyAsync(last_accepted.data(), d_.accepted, sizeof(int) * last_accepted.size(), cudaMemcpyDeviceToHost,
                          e_.st));
    UG_CK(cudaStreamSynchronize(e_.st));
    last_accepted.resize(size_t(cur[1]));
    last_set = attempts ? int((attempts - 1) % (unsigned long long)d_.n_sets) : -1;
}

void Remd::snapshot(bool restore) {
    const size_t np = size_t(std::max(1, n_pair_total_)), ns = size_t(d_.n_sys);
    struct Part {
        void* dev;
        size_t bytes, off;
    } parts[4] = {{d_.replica, 4 * ns, 0},
                  {d_.n_attempt, 4 * np, 4 * ns},
                  {d_.n_success, 4 * np, 4 * ns + 4 * np},
                  {d_.attempt, 8, 4 * ns + 8 * np}};
    char* base = reinterpret_cast<char*>(snap_);
    for (auto& p : parts) {
        if (restore) UG_CK(cudaMemcpyAsync(p.dev, base + p.off, p.bytes, cudaMemcpyDeviceToDevice, e_.st));
        else UG_CK(cudaMemcpyAsync(base + p.off, p.dev, p.bytes, cudaMemcpyDeviceToDevice, e_.st));
    }
}

}  // namespace ug
