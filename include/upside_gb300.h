/* Batched GB300 Upside engine: many systems (replicas, or proteins of uneven
 * length) advanced together by one set of sm_103a kernels and one captured
 * CUDA graph.  These entry points have no counterpart in the reference C
 * library; they expose the GPU form of the reference driver's per-system loop
 * (src/main.cpp:915-999) and replica exchange (src/main.cpp:147-317).
 *
 * All arrays are host arrays, copied at the call; positions and momenta of
 * the whole batch are concatenated in the order the systems were given.
 * Functions return 0 on success and non-zero on error (ug_last_error()).
 */
#ifndef UPSIDE_GB300_BATCH_H
#define UPSIDE_GB300_BATCH_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct UgBatch UgBatch;

const char* ug_last_error(void);

/* Select the CUDA device used by engines created afterwards on this thread. */
int ug_set_device(int device);

/* Build one engine over n_sys `.up` files (identical node graphs). */
UgBatch* ug_create(int n_sys, const char* const* paths, const int* n_atom);
void ug_free(UgBatch* b);
int ug_atom_total(UgBatch* b);

int ug_set_pos(UgBatch* b, const float* pos);
int ug_get_pos(UgBatch* b, float* pos);
int ug_set_mom(UgBatch* b, const float* mom);
int ug_get_mom(UgBatch* b, float* mom);

/* Potential + derivative for every system; energy[n_sys] (FP64 sums), deriv
 * (atom_total,3) may be NULL. */
int ug_evaluate(UgBatch* b, double* energy, float* deriv);

/* Thermostat state: per-system temperature and seed, common timescale; the
 * per-system invocation counter (the thermostat's RNG counter) is set by
 * ug_set_round. */
int ug_set_thermostat(UgBatch* b, const float* temperature, const uint32_t* seed);
int ug_set_round(UgBatch* b, const uint64_t* round);

/* Integrator of the rounds: multistep = 0 the three-stage cycle (inner_step
 * must be 3); multistep = 1 the reference's multistep integrator
 * (src/deriv_engine.cpp:333-351): per round the forces of the slow nodes
 * (config attribute integrator_level 1) kick the momenta once by inner_step
 * dt, then inner_step stages of the fast nodes' forces (level 0) move them.
 * The thermostat's time step is inner_step dt per round. */
int ug_set_integrator(UgBatch* b, int multistep, int inner_step);
/* dE/dx of the nodes of one integrator level (0 fast, 1 slow) at the current
 * positions: the forces each part of a multistep round uses; deriv is
 * (atom_total, 3).  The two levels sum to ug_evaluate's derivative. */
int ug_level_forces(UgBatch* b, int level, float* deriv);

/* Advance n_round rounds of {thermostat; 3 x (force, p -= dt F, x += dt p)}
 * (or the multistep round, ug_set_integrator).
 * use_graph != 0 replays a captured CUDA graph of graph_rounds rounds. */
int ug_run(UgBatch* b, int n_round, float dt, float timescale, int use_graph, int graph_rounds);

/* Node introspection over the whole batch (rows of all systems concatenated). */
int ug_node_dims(UgBatch* b, const char* node, int* n_elem, int* width);
int ug_node_output(UgBatch* b, const char* node, float* out, int n);
int ug_node_sens(UgBatch* b, const char* node, float* out, int n);
int ug_node_edges(UgBatch* b, const char* node, int32_t* pairs, int cap);
int ug_value_by_name(UgBatch* b, const char* node, const char* what, float* out, int n);
/* per-node potential of each system after ug_evaluate: out[n_sys] */
int ug_node_potential(UgBatch* b, const char* node, double* out);

/* Parameters of a node, shared by every system of the batch (set_param /
 * get_param of the reference, src/engine_c_library.cpp:68-92), and
 * dE/d(param) after ug_evaluate summed over all systems of the batch (the
 * adjoint kernels behind get_param_deriv, src/engine_c_library.cpp:94-110);
 * a batch of frames of one protein gives the frame sum in one call. */
int ug_set_param(UgBatch* b, const char* node, const float* param, int n);
int ug_get_param(UgBatch* b, const char* node, float* param, int n);
int ug_param_deriv(UgBatch* b, const char* node, float* deriv, int n);

/* One replica exchange over the batch, criterion 0 (ReplicaExchange::
 * attempt_swaps, src/main.cpp:243-316): energies of all systems, coordinates
 * of the given pairs (pairs[2*k], pairs[2*k+1]) swapped, energies again, and
 * each swap whose log-Boltzmann change fails the Metropolis test undone.  All
 * on the device: FP64 acceptance, uniforms from the replica-exchange Threefry
 * stream (key (seed, 1), counter (round, 0, draw)).  accepted[k] receives
 * 0/1.  Synchronises. */
int ug_replica_exchange(UgBatch* b, int n_pairs, const int* pairs, uint32_t seed, uint64_t round, int* accepted);
/* Periodic replica exchange inside the integration rounds (the reference's
 * --replica-interval with alternating --swap-set lists, src/main.cpp:996-997):
 * after every interval-th round (counted from this call) one exchange with the
 * next swap set in turn (exchange k uses set k % n_sets and round key
 * (k + 1) * interval), criterion 0 or 1 (src/main.cpp:276-313).  set_sizes[k]
 * pairs of set k follow one another in pairs.  ug_run and ug_bench then run
 * the exchanges on the device, in the captured graphs (a graph replay is one
 * interval and its exchange).  n_sets = 0 removes the plan. */
int ug_set_replica_exchange(UgBatch* b, int n_sets, const int* set_sizes, const int* pairs, uint32_t seed,
                            int interval, int criterion);
/* State of the periodic plan: replica index held by each system (n_sys),
 * per pair of all sets its attempts and successes (cap_pairs entries at
 * most), exchanges made, and the last exchange's accept flags (in the order
 * of its set) and set index. */
int ug_replica_state(UgBatch* b, int* replica, unsigned* n_attempt, unsigned* n_success, int cap_pairs,
                     unsigned long long* n_exchanges, int* last_accepted, int* last_set);
/* Periodic box for every system of the batch (no counterpart in the
 * reference, which has open boundaries): edge lengths lx, ly, lz in angstrom,
 * 0 for an open direction.  Pair searches, pair terms (rotamer, hbond,
 * coverage and environment graphs, backbone pairs) use the minimum image;
 * bonded terms and coordinates are untouched (coordinates are never
 * wrapped).  Rejects a box edge under twice a graph's cutoff plus candidate
 * buffer. */
int ug_set_box(UgBatch* b, float lx, float ly, float lz);
/* One exchange of the periodic plan now (the next set in turn, drawn with the
 * round key of that exchange), outside the round schedule.  Synchronises. */
int ug_exchange_now(UgBatch* b);
/* Rounds per timed replay of ug_bench: 1, or the exchange interval. */
int ug_timed_rounds(UgBatch* b);

/* Monte Carlo moves over the batch (the reference's MultipleMonteCarloSampler,
 * src/monte_carlo_sampler.cpp:248-308): for every system with
 * /input/pivot_moves, then every system with /input/jump_moves, one move
 * drawn from the sampler's random stream keyed by the system's thermostat
 * seed and `round`, accepted by the Metropolis test on the energy change at
 * the system's temperature (rejected moves are undone).  accepted[2*s + k]
 * (may be NULL): 1 accepted, 0 rejected, -1 system s has no sampler k
 * (k = 0 pivot, 1 jump). */
int ug_monte_carlo(UgBatch* b, uint64_t round, int* accepted);

/* status bits: 1 pair list overflow (grown automatically), 2 BP hit max_iter,
 * 4 residue-pair storage overflow */
int ug_status(UgBatch* b, int clear);
/* kernel launches per force evaluation and device bytes held */
int ug_info(UgBatch* b, int* launches_per_eval, int64_t* device_bytes);

/* Timed integration rounds for benchmarking: n_round replays of a captured
 * one-round CUDA graph, each bracketed by CUDA events on the engine stream;
 * with flush_l2 a 256 MiB buffer is rewritten before every round (outside
 * the events) so no round starts with a warm L2.  ms[n_round] receives the
 * device time of each round.  With e2e != 0 each timed region also holds the
 * host->device copy of positions and momenta from pinned host memory and the
 * device->host copy of them back (the state a caller round-trips per round). */
int ug_bench(UgBatch* b, int n_round, float dt, float timescale, int flush_l2, int e2e, float* ms);
/* The rotamer BP solve kernel over the last ug_bench: stats[0] its summed
 * device time in ms (CUDA events recorded around each launch inside the
 * replayed graph, on the engine stream), stats[1] its number of launches,
 * stats[2] its summed algorithmic bytes (P, messages, beliefs and indices
 * each sweep touches; the count is kept by the kernel itself). */
int ug_bench_kernel(UgBatch* b, double* stats);

/* Autotuner (no counterpart in the reference): from the batch's current
 * state, times n_round integration rounds for each candidate setting and
 * keeps the fastest; the state is restored after every trial and at the end.
 * Tuned: the candidate-cache buffer of the pair lists (1, 2, 3, 4, 6 times the
 * reference's 1 + 0.2 cutoff; results do not depend on it), then the BP
 * solve's blocks per system, lanes per node and threads per block, then the
 * number of streams the node graph is spread over (1, 2, 4, 8, 16).  report
 * receives '\n'-separated "setting\tms_per_round" lines and a final
 * "chosen\tsetting" line.  Returns the number of candidates tried (or -1). */
int ug_autotune(UgBatch* b, int n_round, float dt, float timescale, char* report, int cap);
/* Set the tuned quantities directly: cache buffer scale (>= 1), BP launch
 * variant (0..8: blocks per system x lanes per node x threads = 2x8x1024,
 * 2x4x1024, 2x16x1024, 1x8x1024, 4x8x512, 4x4x512, 8x4x256, 8x8x256,
 * 16x4x128) and the number of streams the node graph is spread over (1..16). */
int ug_set_tuning(UgBatch* b, float cache_buffer_scale, int bp_variant, int node_streams);

/* Per-node device time of n_eval eager force evaluations (CUDA events on the
 * engine stream): names '\n'-separated "<node>:fwd" / "<node>:bwd", ms[k] the
 * mean time of entry k.  Returns the number of entries (or -1). */
int ug_profile(UgBatch* b, int n_eval, char* names, int names_cap, float* ms, int cap);

/* Pair list of one point set held in device memory: every (i, j), i < j, with
 * |x_i - x_j| < cutoff, the interaction-graph pair search of the engine
 * (replaces PairlistComputation's cache pass, src/interaction_graph.h:122-157,
 * for callers without an engine).  pos: n x 3 floats on the device; pairs:
 * device int32 (i, j) x cap, 8-byte aligned (each pair is stored as one 8-byte
 * word; an unaligned pointer is rejected); *n_pairs (device int32) receives the
 * total number of pairs, which may exceed cap (pairs past cap are not written)
 * and saturates at INT32_MAX when the true total does not fit.  cutoff must be
 * finite and > 0.  Pair order: i / 4, then j, then i % 4.  stream: a
 * cudaStream_t or NULL.  Allocates its scratch (2 ceil(n/4) + 1 ints) with
 * cudaMalloc and synchronises the stream before returning. */
int ug_pair_list(const float* pos, int n, float cutoff, int32_t* pairs, int cap, int32_t* n_pairs, void* stream);

/* ug_pair_list without any device allocation (no counterpart in the
 * reference).  For callers that cannot allocate device memory when they need
 * the list: services whose device memory is reserved up front, code that must
 * not synchronise the device the way cudaMalloc/cudaFree can, hosts without an
 * allocator of their own.  The scratch is a fixed device array built into the
 * library, so n is limited to 262144 points; larger n is rejected with an
 * error naming the limit.  The first call on each device looks up that array's
 * address (make it before any stream capture); later calls only enqueue work
 * on `stream` and return without synchronising.  Nothing has to be zeroed
 * beforehand.  Calls that can run at the same time on one device (two streams,
 * two host threads) share the array and race: order them on one stream.
 * The looked-up address is kept for the life of the process, so the device's
 * primary context must stay alive as long as the library is used (no
 * cudaDeviceReset between calls).
 * Output, order, alignment and arguments as ug_pair_list. */
int ug_pair_list_noalloc(const float* pos, int n, float cutoff, int32_t* pairs, int cap, int32_t* n_pairs,
                         void* stream);

/* Learned BP warm start (no counterpart in the reference; it replaces the
 * uniform initial state of the BP solve, src/rotamer.cpp:1110-1135).  A
 * per-residue MLP, 64 features -> 128 -> 128 -> 8 rotamer logits with ReLU,
 * predicts each residue's converged rotamer marginal; the solve starts from
 * the prediction and still iterates to the configured tolerance.  Per system
 * the engine tracks the sweeps needed from the learned and from the uniform
 * start (every 64th solve tries the other one) and uses the learned start
 * only while it saves at least 8 sweeps, about what the network's kernels
 * cost in device time; systems on the uniform start skip the network's
 * feature kernel.  Weights are FP32 row-major (W1 64x128,
 * b1 128, W2 128x128, b2 128, W3 128x8, b3 8), stored as bf16; pass all six
 * or none (none: keep the loaded weights, only switch).  enable selects the
 * start: 0 uniform (the reference's), 1 learned, 2 the previous solve's
 * marginals, 3 the previous solve's final messages and marginals (modes 2
 * and 3 make a solve depend on the previous evaluation of the same system,
 * to within the BP tolerance; the reference re-initialises every call).
 * Training data: ug_value_by_name on the rotamer node with "warm_features"
 * (n_node x 64), "bp_marginal" (n_node x 8), "bp_nrot", "bp_n_node". */
int ug_set_warm_start(UgBatch* b, const float* w1, const float* b1, const float* w2, const float* b2, const float* w3,
                      const float* b3, int enable);

/* Kernels of the warm-start network, on caller-owned device memory, enqueued
 * on `stream` (no counterpart in the reference).  bf16 operands are uint16
 * bit patterns; accumulation is FP32.
 *   gemm:   C[M x N] (row stride ldc) = (accumulate ? C : 0) + A[M x K] . B[K x N]
 *           with A(i,k) = A[i*a_r + k*a_c], B(k,n) = B[k*b_r + n*b_c]
 *   bias_act: H = bf16(act(Z + bias)) and/or Hf = act(Z + bias), act = ReLU if relu
 *   to_bf16: Y = bf16(X); with relu_of (bf16) given, X and Y are zeroed where it is not positive
 *   softmax_xent: softmax over the first nrot[i] of 8 logits, soft-target
 *           cross-entropy; dZ = scale (p - T), *loss += scale * loss (rows with nrot < 2: 0)
 *   colsum: out[N] = column sums of X[M x N]
 *   adam:   Adam step `step` (1-based) on w with gradient g, moments m, v; wb = bf16(w) */
int ug_mlp_gemm(const uint16_t* A, int64_t a_r, int64_t a_c, const uint16_t* B, int64_t b_r, int64_t b_c, float* C,
                int ldc, int M, int N, int K, int accumulate, void* stream);
int ug_mlp_bias_act(const float* Z, const float* bias, uint16_t* H, float* Hf, int M, int N, int relu, void* stream);
int ug_mlp_to_bf16(float* X, const uint16_t* relu_of, uint16_t* Y, int64_t n, void* stream);
int ug_mlp_softmax_xent(const float* Z, const float* T, const int32_t* nrot, float* dZ, float* loss, int M, float scale,
                        void* stream);
int ug_mlp_colsum(const float* X, float* out, int M, int N, void* stream);
int ug_mlp_adam(float* w, const float* g, float* m, float* v, uint16_t* wb, int n, float lr, float b1, float b2,
                float eps, int step, void* stream);

#ifdef __cplusplus
}
#endif
#endif
