// C ABI of the GB300 engine: the reference's engine C library entry points
// (drop-in, src/engine_c_library.h:6-33) and the batch API (upside_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"
#include "mc.h"
#include "remd.h"
#include "warm.h"
#include "../../include/engine_c_library.h"
#include "../../include/upside_gb300.h"

using ug::Engine;

namespace {
thread_local std::string g_err;

// -------------------------------------------------- clamped spline helpers ---
// uniform cubic B-spline weights
void bsp4h(float y, float b[4]) {
    float y2 = y * y, y3 = y2 * y, o = 1.f - y;
    b[0] = o * o * o / 6.f;
    b[1] = (3.f * y3 - 6.f * y2 + 4.f) / 6.f;
    b[2] = (-3.f * y3 + 3.f * y2 + 3.f * y + 1.f) / 6.f;
    b[3] = y3 / 6.f;
}
void clamped_h(const float* c, float x, int n, float& v, float& d) {
    if (x <= 1.f) { v = c[0] / 6.f + c[1] * (2.f / 3.f) + c[2] / 6.f; d = 0.f; return; }
    if (x >= float(n - 2)) { v = c[n - 3] / 6.f + c[n - 2] * (2.f / 3.f) + c[n - 1] / 6.f; d = 0.f; return; }
    int xb = int(x);
    float y = x - float(xb), b[4], o = 1.f - y;
    bsp4h(y, b);
    float db[4] = {-0.5f * o * o, 1.5f * y * y - 2.f * y, -1.5f * y * y + y + 0.5f, 0.5f * y * y};
    v = d = 0.f;
    for (int k = 0; k < 4; ++k) { v += c[xb - 1 + k] * b[k]; d += c[xb - 1 + k] * db[k]; }
}
}  // namespace

// opaque handle type of the drop-in ABI
struct DerivEngine {
    std::unique_ptr<Engine> e;
    int n_atom;
};
struct UgBatch {
    std::unique_ptr<Engine> e;
    std::vector<std::string> paths;       // the systems' configurations
    std::unique_ptr<ug::McSampler> mc;    // their Monte Carlo moves, read at first use
    // the plan of ug_replica_exchange (kept while its pairs and seed repeat)
    std::unique_ptr<ug::Remd> oneshot;
    std::vector<int> oneshot_key;
    // measured kernel over the last ug_bench: device ms, launches, algorithmic bytes
    double kt_ms = 0.0, kt_bytes = 0.0;
    long long kt_launches = 0;
};

#define GUARD_BEGIN try {
#define GUARD_END(ret)                                   \
    }                                                    \
    catch (const std::exception& ex) {                   \
        g_err = ex.what();                               \
        fprintf(stderr, "\n\nERROR: %s\n", ex.what());   \
        return ret;                                      \
    }

extern "C" {

// ============================================================ drop-in ABI ===
DerivEngine* construct_deriv_engine(int n_atom, const char* potential_file, bool quiet) {
    (void)quiet;
    GUARD_BEGIN
    auto* d = new DerivEngine;
    d->n_atom = n_atom;
    d->e.reset(new Engine({std::string(potential_file)}, {n_atom}));
    return d;
    GUARD_END(nullptr)
}

void free_deriv_engine(DerivEngine* engine) { delete engine; }

int evaluate_energy(float* energy, DerivEngine* engine, const float* pos) {
    GUARD_BEGIN
    engine->e->set_pos(pos);
    engine->e->compute_checked(true);
    double en = 0;
    engine->e->energies(&en);
    *energy = float(en);
    return 0;
    GUARD_END(1)
}

int evaluate_deriv(float* deriv, DerivEngine* engine, const float* pos) {
    GUARD_BEGIN
    engine->e->set_pos(pos);
    engine->e->compute_checked(true);
    engine->e->get_deriv(deriv);
    return 0;
    GUARD_END(1)
}

int set_param(int n_param, const float* param, DerivEngine* engine, const char* node_name) {
    GUARD_BEGIN
    engine->e->node(node_name).set_param(*engine->e, std::vector<float>(param, param + n_param));
    return 0;
    GUARD_END(1)
}

int get_param(int n_param, float* param, DerivEngine* engine, const char* node_name) {
    GUARD_BEGIN
    auto v = engine->e->node(node_name).get_param(*engine->e);
    if (v.size() != size_t(n_param))
        throw ug::Error("Wrong number of parameters, expected " + std::to_string(v.size()) + " but got " +
                        std::to_string(n_param));
    std::copy(v.begin(), v.end(), param);
    return 0;
    GUARD_END(1)
}

int get_param_deriv(int n_param, float* deriv, DerivEngine* engine, const char* node_name) {
    GUARD_BEGIN
    auto v = engine->e->node(node_name).param_deriv(*engine->e);
    if (v.size() != size_t(n_param))
        throw ug::Error("Wrong number of parameters, expected " + std::to_string(v.size()) + " but got " +
                        std::to_string(n_param));
    std::copy(v.begin(), v.end(), deriv);
    return 0;
    GUARD_END(1)
}

static int node_copy(Engine& e, const char* name, float* out, int n, bool sens) {
    auto& nd = e.node(name);
    if (nd.potential) {
        if (n != 1) throw ug::Error("wrong size for potential node");
        double v = 0;
        UG_CK(cudaMemcpy(&v, e.d_pot + size_t(nd.pot_slot) * e.n_sys, sizeof(double), cudaMemcpyDeviceToHost));
        *out = float(v);
        return 0;
    }
    if (n != nd.total * nd.width) throw ug::Error("wrong size for CoordNode");
    e.sync();
    UG_CK(cudaMemcpy(out, sens ? nd.sens : nd.out, sizeof(float) * size_t(n), cudaMemcpyDeviceToHost));
    return 0;
}

int get_sens(int n_output, float* output, DerivEngine* engine, const char* node_name) {
    GUARD_BEGIN
    return node_copy(*engine->e, node_name, output, n_output, true);
    GUARD_END(1)
}

int get_output(int n_output, float* output, DerivEngine* engine, const char* node_name) {
    GUARD_BEGIN
    return node_copy(*engine->e, node_name, output, n_output, false);
    GUARD_END(1)
}

int get_output_dims(int* n_elem, int* elem_width, DerivEngine* engine, const char* node_name) {
    GUARD_BEGIN
    auto& nd = engine->e->node(node_name);
    *n_elem = nd.potential ? 1 : nd.total;
    *elem_width = nd.potential ? 1 : nd.width;
    return 0;
    GUARD_END(1)
}

int get_value_by_name(int n_output, float* output, DerivEngine* engine, const char* node_name, const char* log_name) {
    GUARD_BEGIN
    auto v = engine->e->node(node_name).value_by_name(*engine->e, log_name);
    if (n_output != int(v.size()))
        throw ug::Error("expected size (" + std::to_string(n_output) + " elements) inconsistent with actual size (" +
                        std::to_string(v.size()) + ")");
    std::copy(v.begin(), v.end(), output);
    return 0;
    GUARD_END(1)
}

// Clamped spline helpers: B-spline coefficients whose clamped spline
// interpolates `values` at the interior knots, with zero end slopes
// (clamped_spline_solve, src/engine_c_library.cpp:197-206).
int clamped_spline_solve(int N, float* bspline_coeff, const float* values) {
    int n = N - 2;
    if (n < 2) return 1;
    std::vector<double> a(size_t(n), 1. / 6.), b(size_t(n), 2. / 3.), c(size_t(n), 1. / 6.), d(values, values + n);
    c[0] *= 2.;
    a[size_t(n - 1)] *= 2.;
    for (int k = 1; k < n; ++k) {  // Thomas algorithm
        double m = a[size_t(k)] / b[size_t(k - 1)];
        b[size_t(k)] -= m * c[size_t(k - 1)];
        d[size_t(k)] -= m * d[size_t(k - 1)];
    }
    d[size_t(n - 1)] /= b[size_t(n - 1)];
    for (int k = n - 2; k >= 0; --k) d[size_t(k)] = (d[size_t(k)] - c[size_t(k)] * d[size_t(k + 1)]) / b[size_t(k)];
    for (int k = 0; k < n; ++k) bspline_coeff[k + 1] = float(d[size_t(k)]);
    bspline_coeff[0] = bspline_coeff[2];
    bspline_coeff[N - 1] = bspline_coeff[N - 3];
    return 0;
}

int clamped_spline_value(int N, float* result, const float* bspline_coeff, int nx, float* x) {
    for (int i = 0; i < nx; ++i) {
        float v, d;
        clamped_h(bspline_coeff, x[i], N, v, d);
        result[i] = v;
    }
    return 0;
}

int get_clamped_value_and_deriv(int N, float* result, const float* bspline_coeff, int nx, float* x) {
    for (int i = 0; i < nx; ++i) clamped_h(bspline_coeff, x[i], N, result[2 * i], result[2 * i + 1]);
    return 0;
}

int get_clamped_coeff_deriv(int N, float* result, const float* bspline_coeff, float x) {
    (void)bspline_coeff;
    for (int i = 0; i < N; ++i) result[i] = 0.f;
    if (x <= 1.f) { result[0] = 1.f / 6.f; result[1] = 2.f / 3.f; result[2] = 1.f / 6.f; return 0; }
    if (x >= float(N - 2)) { result[N - 3] = 1.f / 6.f; result[N - 2] = 2.f / 3.f; result[N - 1] = 1.f / 6.f; return 0; }
    int xb = int(x);
    float b[4];
    bsp4h(x - float(xb), b);
    for (int k = 0; k < 4; ++k) result[xb - 1 + k] = b[k];
    return 0;
}

// ============================================================== batch API ===
const char* ug_last_error(void) { return g_err.c_str(); }

int ug_set_device(int device) {
    GUARD_BEGIN
    UG_CK(cudaSetDevice(device));
    return 0;
    GUARD_END(1)
}

UgBatch* ug_create(int n_sys, const char* const* paths, const int* n_atom) {
    GUARD_BEGIN
    std::vector<std::string> p(paths, paths + n_sys);
    std::vector<int> na(n_atom, n_atom + n_sys);
    auto* b = new UgBatch;
    b->e.reset(new Engine(p, na));
    b->paths = p;
    return b;
    GUARD_END(nullptr)
}

void ug_free(UgBatch* b) { delete b; }
int ug_atom_total(UgBatch* b) { return b->e->atom_total; }

int ug_set_pos(UgBatch* b, const float* pos) {
    GUARD_BEGIN
    b->e->set_pos(pos);
    return 0;
    GUARD_END(1)
}
int ug_get_pos(UgBatch* b, float* pos) {
    GUARD_BEGIN
    b->e->get_pos(pos);
    return 0;
    GUARD_END(1)
}
int ug_set_mom(UgBatch* b, const float* mom) {
    GUARD_BEGIN
    UG_CK(cudaMemcpyAsync(b->e->d_mom, mom, sizeof(float) * 3 * size_t(b->e->atom_total), cudaMemcpyHostToDevice, b->e->st));
    b->e->sync();
    return 0;
    GUARD_END(1)
}
int ug_get_mom(UgBatch* b, float* mom) {
    GUARD_BEGIN
    UG_CK(cudaMemcpyAsync(mom, b->e->d_mom, sizeof(float) * 3 * size_t(b->e->atom_total), cudaMemcpyDeviceToHost, b->e->st));
    b->e->sync();
    return 0;
    GUARD_END(1)
}

int ug_evaluate(UgBatch* b, double* energy, float* deriv) {
    GUARD_BEGIN
    b->e->compute_checked(true);
    if (energy) b->e->energies(energy);
    if (deriv) b->e->get_deriv(deriv);
    return 0;
    GUARD_END(1)
}

int ug_set_thermostat(UgBatch* b, const float* temperature, const uint32_t* seed) {
    GUARD_BEGIN
    UG_CK(cudaMemcpyAsync(b->e->d_temp, temperature, sizeof(float) * size_t(b->e->n_sys), cudaMemcpyHostToDevice, b->e->st));
    UG_CK(cudaMemcpyAsync(b->e->d_seed, seed, sizeof(uint32_t) * size_t(b->e->n_sys), cudaMemcpyHostToDevice, b->e->st));
    b->e->sync();
    return 0;
    GUARD_END(1)
}

int ug_level_forces(UgBatch* b, int level, float* deriv) {
    GUARD_BEGIN
    if (level != 0 && level != 1) throw ug::Error("integrator level must be 0 or 1");
    b->e->compute_checked(false, level);
    b->e->get_deriv(deriv);
    return 0;
    GUARD_END(1)
}

int ug_monte_carlo(UgBatch* b, uint64_t round, int* accepted) {
    GUARD_BEGIN
    if (!b->mc) b->mc.reset(new ug::McSampler(*b->e, b->paths));
    b->mc->step(round, accepted);
    return 0;
    GUARD_END(1)
}

int ug_set_integrator(UgBatch* b, int multistep, int inner_step) {
    GUARD_BEGIN
    if (inner_step < 1) throw ug::Error("inner_step must be at least 1");
    if (!multistep && inner_step != 3) throw ug::Error("the three-stage integrator has inner_step 3");
    b->e->multistep = multistep != 0;
    b->e->inner_step = inner_step;
    return 0;
    GUARD_END(1)
}

int ug_set_round(UgBatch* b, const uint64_t* round) {
    GUARD_BEGIN
    UG_CK(cudaMemcpyAsync(b->e->d_round, round, sizeof(uint64_t) * size_t(b->e->n_sys), cudaMemcpyHostToDevice, b->e->st));
    b->e->sync();
    return 0;
    GUARD_END(1)
}

int ug_run(UgBatch* b, int n_round, float dt, float timescale, int use_graph, int graph_rounds) {
    GUARD_BEGIN
    b->e->run_rounds(n_round, dt, timescale, use_graph != 0, graph_rounds);
    return 0;
    GUARD_END(1)
}

int ug_node_dims(UgBatch* b, const char* node, int* n_elem, int* width) {
    GUARD_BEGIN
    auto& nd = b->e->node(node);
    *n_elem = nd.potential ? 1 : nd.total;
    *width = nd.potential ? 1 : nd.width;
    return 0;
    GUARD_END(1)
}
int ug_node_output(UgBatch* b, const char* node, float* out, int n) {
    GUARD_BEGIN
    return node_copy(*b->e, node, out, n, false);
    GUARD_END(1)
}
int ug_node_sens(UgBatch* b, const char* node, float* out, int n) {
    GUARD_BEGIN
    return node_copy(*b->e, node, out, n, true);
    GUARD_END(1)
}
int ug_node_edges(UgBatch* b, const char* node, int32_t* pairs, int cap) {
    GUARD_BEGIN
    auto* g = b->e->node(node).graph();
    if (!g) throw ug::Error("node has no pair list");
    b->e->sync();
    int ne = 0;
    UG_CK(cudaMemcpy(&ne, g->n_edge, 4, cudaMemcpyDeviceToHost));
    int k = std::min(ne, cap);
    if (k > 0) UG_CK(cudaMemcpy(pairs, g->edges, sizeof(int2) * size_t(k), cudaMemcpyDeviceToHost));
    return ne;
    GUARD_END(-1)
}
int ug_value_by_name(UgBatch* b, const char* node, const char* what, float* out, int n) {
    GUARD_BEGIN
    auto v = b->e->node(node).value_by_name(*b->e, what);
    if (n != int(v.size())) throw ug::Error("size mismatch: " + std::to_string(v.size()));
    std::copy(v.begin(), v.end(), out);
    return 0;
    GUARD_END(1)
}
int ug_set_param(UgBatch* b, const char* node, const float* param, int n) {
    GUARD_BEGIN
    b->e->node(node).set_param(*b->e, std::vector<float>(param, param + n));
    return 0;
    GUARD_END(1)
}
int ug_get_param(UgBatch* b, const char* node, float* param, int n) {
    GUARD_BEGIN
    auto v = b->e->node(node).get_param(*b->e);
    if (n != int(v.size())) throw ug::Error("parameter size mismatch: " + std::to_string(v.size()));
    std::copy(v.begin(), v.end(), param);
    return 0;
    GUARD_END(1)
}
int ug_param_deriv(UgBatch* b, const char* node, float* deriv, int n) {
    GUARD_BEGIN
    auto v = b->e->node(node).param_deriv(*b->e);
    if (n != int(v.size())) throw ug::Error("parameter size mismatch: " + std::to_string(v.size()));
    std::copy(v.begin(), v.end(), deriv);
    return 0;
    GUARD_END(1)
}

int ug_set_warm_start(UgBatch* b, const float* w1, const float* b1, const float* w2, const float* b2, const float* w3,
                      const float* b3, int enable) {
    GUARD_BEGIN
    const float* p[6] = {w1, b1, w2, b2, w3, b3};
    bool given = w1 && b1 && w2 && b2 && w3 && b3;
    if (!given && (w1 || b1 || w2 || b2 || w3 || b3)) throw ug::Error("ug_set_warm_start: give all six arrays or none");
    bool found = false;
    if (enable < 0 || enable > 3) throw ug::Error("ug_set_warm_start: mode must be 0, 1, 2 or 3");
    for (auto& n : b->e->nodes) found |= n->set_warm(*b->e, given ? p : nullptr, enable);
    if (!found) throw ug::Error("ug_set_warm_start: the node graph has no rotamer node");
    b->e->drop_graph();
    return 0;
    GUARD_END(1)
}

int ug_node_potential(UgBatch* b, const char* node, double* out) {
    GUARD_BEGIN
    auto& nd = b->e->node(node);
    if (!nd.potential) throw ug::Error("not a potential node");
    b->e->sync();
    UG_CK(cudaMemcpy(out, b->e->d_pot + size_t(nd.pot_slot) * b->e->n_sys, sizeof(double) * size_t(b->e->n_sys),
                     cudaMemcpyDeviceToHost));
    return 0;
    GUARD_END(1)
}

}  // extern "C"
namespace ug {
void threefry_host(const uint32_t c[4], const uint32_t k[4], uint32_t out[4]) {
    static const int R[8][2] = {{10, 26}, {11, 21}, {13, 27}, {23, 5}, {6, 20}, {17, 11}, {25, 10}, {18, 20}};
    uint32_t ks[5] = {k[0], k[1], k[2], k[3], 0x1BD11BDAu ^ k[0] ^ k[1] ^ k[2] ^ k[3]};
    uint32_t x[4];
    for (int i = 0; i < 4; ++i) x[i] = c[i] + ks[i];
    auto rotl = [](uint32_t v, int r) { return (v << r) | (v >> (32 - r)); };
    for (int r = 0; r < 20; ++r) {
        if (r % 2 == 0) {
            x[0] += x[1]; x[1] = rotl(x[1], R[r % 8][0]); x[1] ^= x[0];
            x[2] += x[3]; x[3] = rotl(x[3], R[r % 8][1]); x[3] ^= x[2];
        } else {
            x[0] += x[3]; x[3] = rotl(x[3], R[r % 8][0]); x[3] ^= x[0];
            x[2] += x[1]; x[1] = rotl(x[1], R[r % 8][1]); x[1] ^= x[2];
        }
        if (r % 4 == 3) {
            uint32_t s = uint32_t(r / 4 + 1);
            for (int i = 0; i < 4; ++i) x[i] += ks[(s + uint32_t(i)) % 5];
            x[3] += s;
        }
    }
    for (int i = 0; i < 4; ++i) out[i] = x[i];
}
void swap_coords(Engine& e, int s1, int s2, float* tmp) {
    if (e.n_atom[size_t(s1)] != e.n_atom[size_t(s2)]) throw ug::Error("replica exchange needs equal atom counts");
    size_t n = sizeof(float) * 3 * size_t(e.n_atom[size_t(s1)]);
    float* a = e.d_pos + 3 * size_t(e.atom_off[size_t(s1)]);
    float* b = e.d_pos + 3 * size_t(e.atom_off[size_t(s2)]);
    UG_CK(cudaMemcpyAsync(tmp, a, n, cudaMemcpyDeviceToDevice, e.st));
    UG_CK(cudaMemcpyAsync(a, b, n, cudaMemcpyDeviceToDevice, e.st));
    UG_CK(cudaMemcpyAsync(b, tmp, n, cudaMemcpyDeviceToDevice, e.st));
}
}  // namespace ug
using ug::swap_coords;
using ug::threefry_host;
extern "C" {

// One exchange over the given pairs (criterion 0), on the device: the
// replica-exchange kernels of remd.cu with the draws keyed by `round`.  The
// plan for these pairs is kept between calls with the same pairs.
int ug_replica_exchange(UgBatch* b, int n_pairs, const int* pairs, uint32_t seed, uint64_t round, int* accepted) {
    GUARD_BEGIN
    Engine& e = *b->e;
    std::vector<int> key(pairs, pairs + 2 * size_t(n_pairs));
    key.push_back(int(seed));
    if (!b->oneshot || b->oneshot_key != key) {
        std::vector<std::vector<std::pair<int, int>>> sets(1);
        for (int k = 0; k < n_pairs; ++k) sets[0].emplace_back(pairs[2 * k], pairs[2 * k + 1]);
        b->oneshot.reset(new ug::Remd(e, sets, seed, 0, 0, 0ull));
        b->oneshot_key = key;
    }
    b->oneshot->enqueue((long long)round);
    std::vector<int> rep, acc;
    std::vector<unsigned> na, ns;
    unsigned long long att = 0;
    int set = 0;
    b->oneshot->read(rep, na, ns, att, acc, set);
    if (accepted)
        for (int k = 0; k < n_pairs; ++k) accepted[k] = acc[size_t(k)];
    return 0;
    GUARD_END(1)
}

int ug_set_replica_exchange(UgBatch* b, int n_sets, const int* set_sizes, const int* pairs, uint32_t seed,
                            int interval, int criterion) {
    GUARD_BEGIN
    Engine& e = *b->e;
    if (n_sets <= 0) {
        e.drop_graph();
        e.remd.reset();
        return 0;
    }
    std::vector<std::vector<std::pair<int, int>>> sets(static_cast<size_t>(n_sets));
    size_t q = 0;
    for (int k = 0; k < n_sets; ++k) {
        if (set_sizes[k] < 0) throw ug::Error("negative swap set size");
        for (int i = 0; i < set_sizes[k]; ++i, ++q) sets[size_t(k)].emplace_back(pairs[2 * q], pairs[2 * q + 1]);
    }
    e.drop_graph();
    e.remd.reset(new ug::Remd(e, sets, seed, criterion, interval, 0ull));
    e.remd_done = 0;
    return 0;
    GUARD_END(1)
}

int ug_replica_state(UgBatch* b, int* replica, unsigned* n_attempt, unsigned* n_success, int cap_pairs,
                     unsigned long long* n_exchanges, int* last_accepted, int* last_set) {
    GUARD_BEGIN
    Engine& e = *b->e;
    if (!e.remd) throw ug::Error("no replica exchange plan");
    std::vector<int> rep, acc;
    std::vector<unsigned> na, ns;
    unsigned long long att = 0;
    int set = -1;
    e.remd->read(rep, na, ns, att, acc, set);
    if (replica) std::copy(rep.begin(), rep.end(), replica);
    if (int(na.size()) > cap_pairs) throw ug::Error("pair arrays too small");
    if (n_attempt) std::copy(na.begin(), na.end(), n_attempt);
    if (n_success) std::copy(ns.begin(), ns.end(), n_success);
    if (n_exchanges) *n_exchanges = att;
    if (last_accepted) std::copy(acc.begin(), acc.end(), last_accepted);
    if (last_set) *last_set = set;
    return 0;
    GUARD_END(1)
}

int ug_set_box(UgBatch* b, float lx, float ly, float lz) {
    GUARD_BEGIN
    b->e->set_box(lx, ly, lz);
    return 0;
    GUARD_END(1)
}

int ug_exchange_now(UgBatch* b) {
    GUARD_BEGIN
    if (!b->e->remd) throw ug::Error("no replica exchange plan");
    b->e->remd->enqueue();
    b->e->sync();
    return 0;
    GUARD_END(1)
}

int ug_timed_rounds(UgBatch* b) { return b->e->timed_rounds(); }

int ug_status(UgBatch* b, int clear) {
    GUARD_BEGIN
    return b->e->status(clear != 0);
    GUARD_END(-1)
}

int ug_info(UgBatch* b, int* launches, int64_t* bytes) {
    GUARD_BEGIN
    if (launches) *launches = b->e->launches_per_compute ? b->e->launches_per_compute : b->e->count_launches();
    if (bytes) *bytes = int64_t(b->e->device_bytes);
    return 0;
    GUARD_END(1)
}

int ug_bench(UgBatch* b, int n_round, float dt, float timescale, int flush_l2, int e2e, float* ms) {
    GUARD_BEGIN
    Engine& e = *b->e;
    // with periodic replica exchanges a timed replay is one interval and its
    // exchange, started on an interval boundary
    const int xi = e.remd ? e.remd->interval() : 0;
    if (xi > 0 && e.remd_done % (unsigned long long)xi)
        e.run_rounds(int(xi - e.remd_done % (unsigned long long)xi), dt, timescale, false, 1);
    if (!e.graph_exec || e.graph_rounds != e.timed_rounds() || !e.graph_timed) e.capture_timed(dt, timescale);
    b->kt_ms = b->kt_bytes = 0.0;
    b->kt_launches = 0;
    double bytes0 = e.kernel_bytes();
    const size_t flush_bytes = size_t(256) << 20;
    void* flush = nullptr;
    if (flush_l2) UG_CK(cudaMalloc(&flush, flush_bytes));
    size_t state = sizeof(float) * 3 * size_t(e.atom_total);
    float *hpos = nullptr, *hmom = nullptr;
    if (e2e) {
        UG_CK(cudaMallocHost(&hpos, state));
        UG_CK(cudaMallocHost(&hmom, state));
        UG_CK(cudaMemcpyAsync(hpos, e.d_pos, state, cudaMemcpyDeviceToHost, e.st));
        UG_CK(cudaMemcpyAsync(hmom, e.d_mom, state, cudaMemcpyDeviceToHost, e.st));
    }
    std::vector<cudaEvent_t> ev(2 * size_t(n_round));
    for (auto& x : ev) UG_CK(cudaEventCreate(&x));
    for (int r = 0; r < n_round; ++r) {
        if (flush) UG_CK(cudaMemsetAsync(flush, r & 0xff, flush_bytes, e.st));
        UG_CK(cudaEventRecord(ev[2 * size_t(r)], e.st));
        if (e2e) {
            UG_CK(cudaMemcpyAsync(e.d_pos, hpos, state, cudaMemcpyHostToDevice, e.st));
            UG_CK(cudaMemcpyAsync(e.d_mom, hmom, state, cudaMemcpyHostToDevice, e.st));
        }
        e.launch_graph();
        if (e2e) {
            UG_CK(cudaMemcpyAsync(hpos, e.d_pos, state, cudaMemcpyDeviceToHost, e.st));
            UG_CK(cudaMemcpyAsync(hmom, e.d_mom, state, cudaMemcpyDeviceToHost, e.st));
        }
        UG_CK(cudaEventRecord(ev[2 * size_t(r) + 1], e.st));
        if (e.graph_timed) {
            // the graph's event-record nodes are re-recorded by the next
            // replay: read this round's kernel brackets now
            UG_CK(cudaStreamSynchronize(e.st));
            for (int k = 0; k + 1 < e.kt_used; k += 2) {
                float t = 0.f;
                if (cudaEventElapsedTime(&t, e.kt_ev[size_t(k)], e.kt_ev[size_t(k) + 1]) != cudaSuccess) {
                    // no timing for this kernel (reported as zero launches);
                    // the round times above are unaffected
                    cudaGetLastError();
                    b->kt_launches = 0;
                    b->kt_ms = 0.0;
                    e.graph_timed = false;
                    break;
                }
                b->kt_ms += t;
                b->kt_launches += 1;
            }
        }
    }
    UG_CK(cudaStreamSynchronize(e.st));
    e.remd_done += (unsigned long long)n_round * (unsigned long long)e.timed_rounds();
    b->kt_bytes = e.kernel_bytes() - bytes0;
    for (int r = 0; r < n_round; ++r) UG_CK(cudaEventElapsedTime(&ms[r], ev[2 * size_t(r)], ev[2 * size_t(r) + 1]));
    for (auto& x : ev) cudaEventDestroy(x);
    if (flush) cudaFree(flush);
    if (hpos) cudaFreeHost(hpos);
    if (hmom) cudaFreeHost(hmom);
    int s = e.status(true);
    if (s & (ug::ST_EDGE_OVERFLOW | ug::ST_RES_EDGE_OVERFLOW)) {
        // storage grew mid-run: results of this run are invalid, report it
        for (auto& n : e.nodes) n->grow(e);
        throw ug::Error("pair-list storage overflowed during the timed rounds; rerun");
    }
    return 0;
    GUARD_END(1)
}

int ug_autotune(UgBatch* b, int n_round, float dt, float timescale, char* report, int cap) {
    GUARD_BEGIN
    auto r = b->e->autotune(n_round, dt, timescale);
    std::string s;
    for (auto& x : r) s += x.first + "\t" + std::to_string(x.second) + "\n";
    int c, l, t;
    ug::bp_variant_desc(b->e->tuned_bp_variant, &c, &l, &t);
    s += "chosen\tcache_buffer_scale=" + std::to_string(b->e->tuned_buffer_scale).substr(0, 4) +
         ",bp_blocks_per_system=" + std::to_string(c) + ",lanes_per_node=" + std::to_string(l) +
         ",threads=" + std::to_string(t) + ",node_streams=" + std::to_string(b->e->n_lanes) + "\n";
    if (int(s.size()) + 1 > cap) throw ug::Error("report buffer too small");
    memcpy(report, s.c_str(), s.size() + 1);
    return int(r.size());
    GUARD_END(-1)
}

int ug_set_tuning(UgBatch* b, float cache_buffer_scale, int bp_variant, int node_streams) {
    GUARD_BEGIN
    if (node_streams < 1 || node_streams > 16) throw ug::Error("node_streams must be 1..16");
    b->e->set_tuning(cache_buffer_scale, bp_variant);
    if (node_streams != b->e->n_lanes) {
        b->e->n_lanes = node_streams;
        b->e->setup_lanes();
    }
    return 0;
    GUARD_END(1)
}

int ug_bench_kernel(UgBatch* b, double* stats) {
    GUARD_BEGIN
    stats[0] = b->kt_ms;
    stats[1] = double(b->kt_launches);
    stats[2] = b->kt_bytes;
    return 0;
    GUARD_END(1)
}

int ug_profile(UgBatch* b, int n_eval, char* names, int names_cap, float* ms, int cap) {
    GUARD_BEGIN
    auto p = b->e->profile_nodes(n_eval);
    std::string s;
    for (size_t k = 0; k < p.size(); ++k) {
        s += p[k].first + "\n";
        if (int(k) < cap) ms[k] = p[k].second;
    }
    if (int(s.size()) + 1 > names_cap) throw ug::Error("names buffer too small");
    memcpy(names, s.c_str(), s.size() + 1);
    return int(p.size());
    GUARD_END(-1)
}

// ------------------------------------------- warm-start network kernels ---
#define UG_MLP(call)                                        \
    GUARD_BEGIN                                             \
    UG_CK(call);                                            \
    return 0;                                               \
    GUARD_END(1)

int ug_mlp_gemm(const uint16_t* A, int64_t a_r, int64_t a_c, const uint16_t* B, int64_t b_r, int64_t b_c, float* C,
                int ldc, int M, int N, int K, int accumulate, void* stream) {
    UG_MLP(ug::launch_gemm_bf16(A, a_r, a_c, B, b_r, b_c, C, ldc, M, N, K, accumulate,
                                static_cast<cudaStream_t>(stream)))
}
int ug_mlp_bias_act(const float* Z, const float* bias, uint16_t* H, float* Hf, int M, int N, int relu, void* stream) {
    UG_MLP(ug::launch_bias_act(Z, bias, H, Hf, M, N, relu, static_cast<cudaStream_t>(stream)))
}
int ug_mlp_to_bf16(float* X, const uint16_t* relu_of, uint16_t* Y, int64_t n, void* stream) {
    UG_MLP(ug::launch_to_bf16(X, relu_of, Y, n, static_cast<cudaStream_t>(stream)))
}
int ug_mlp_softmax_xent(const float* Z, const float* T, const int32_t* nrot, float* dZ, float* loss, int M, float scale,
                        void* stream) {
    UG_MLP(ug::launch_softmax_xent(Z, T, nrot, dZ, loss, M, scale, static_cast<cudaStream_t>(stream)))
}
int ug_mlp_colsum(const float* X, float* out, int M, int N, void* stream) {
    UG_MLP(ug::launch_colsum(X, out, M, N, static_cast<cudaStream_t>(stream)))
}
int ug_mlp_adam(float* w, const float* g, float* m, float* v, uint16_t* wb, int n, float lr, float b1, float b2,
                float eps, int step, void* stream) {
    UG_MLP(ug::launch_adam(w, g, m, v, wb, n, lr, b1, b2, eps, step, static_cast<cudaStream_t>(stream)))
}

int ug_pair_list(const float* pos, int n, float cutoff, int32_t* pairs, int cap, int32_t* n_pairs, void* stream) {
    GUARD_BEGIN
    if (n < 0 || cap < 0 || !(cutoff > 0.f) || !std::isfinite(cutoff))
        throw ug::Error("ug_pair_list: need n >= 0, cap >= 0, a finite cutoff > 0");
    if ((n > 0 && !pos) || (cap > 0 && !pairs) || !n_pairs) throw ug::Error("ug_pair_list: null device pointer");
    if (reinterpret_cast<uintptr_t>(pairs) % 8)
        throw ug::Error("ug_pair_list: pairs must be 8-byte aligned (pairs are stored as int32 pairs)");
    auto st = static_cast<cudaStream_t>(stream);
    size_t n_rows = (size_t(n) + 3) / 4;
    int* scratch = nullptr;
    UG_CK(cudaMalloc(&scratch, sizeof(int) * (2 * n_rows + 1)));
    cudaError_t e1 = ug::launch_point_pairs(pos, n, cutoff, pairs, cap, n_pairs, scratch, scratch + n_rows, st);
    cudaError_t e2 = cudaStreamSynchronize(st);
    cudaError_t e3 = cudaFree(scratch);
    UG_CK(e1);
    UG_CK(e2);
    UG_CK(e3);
    return 0;
    GUARD_END(1)
}

int ug_pair_list_noalloc(const float* pos, int n, float cutoff, int32_t* pairs, int cap, int32_t* n_pairs,
                         void* stream) {
    GUARD_BEGIN
    if (n < 0 || cap < 0 || !(cutoff > 0.f) || !std::isfinite(cutoff))
        throw ug::Error("ug_pair_list_noalloc: need n >= 0, cap >= 0, a finite cutoff > 0");
    if (reinterpret_cast<uintptr_t>(pairs) % 8)
        throw ug::Error("ug_pair_list_noalloc: pairs must be 8-byte aligned (pairs are stored as int32 pairs)");
    if (n > ug::point_pairs_noalloc_max())
        throw ug::Error("ug_pair_list_noalloc: n = " + std::to_string(n) + " points exceeds the fixed scratch limit of " +
                        std::to_string(ug::point_pairs_noalloc_max()) + " points (use ug_pair_list)");
    if ((n > 0 && !pos) || (cap > 0 && !pairs) || !n_pairs)
        throw ug::Error("ug_pair_list_noalloc: null device pointer");
    int* scratch = nullptr;
    UG_CK(ug::point_pairs_noalloc_scratch(&scratch));
    int n_rows = (n + 3) / 4;
    UG_CK(ug::launch_point_pairs(pos, n, cutoff, pairs, cap, n_pairs, scratch, scratch + n_rows,
                                 static_cast<cudaStream_t>(stream)));
    return 0;
    GUARD_END(1)
}

}  // extern "C"
