// GB300 Upside engine: host-side graph of force-field nodes over a batch of
// systems, device buffers, and the integrator.  Every node's compute runs as
// sm_103a kernels over all systems of the batch at once.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "graph.h"
#include "h5lite.h"

namespace ug {

struct Error : std::runtime_error {
    explicit Error(const std::string& s) : std::runtime_error(s) {}
};

void cuda_check(cudaError_t e, const char* what);
#define UG_CK(x) ::ug::cuda_check((x), #x)

class Engine;
class Remd;

// One `/input/potential/<node>` group of every system of the batch.
struct Groups {
    std::vector<h5lite::File*> files;
    std::string path;
    size_t size() const { return files.size(); }
    h5lite::File& f(size_t s) const { return *files[s]; }
    std::string p(const std::string& n) const { return path + "/" + n; }
};

struct GNode {
    std::string name;
    std::vector<int> args;
    bool potential = false;
    int width = 0, total = 0;
    std::vector<int> off;  // per-system element offsets (n_sys+1)
    float* out = nullptr;  // total*width
    float* sens = nullptr;
    int pot_slot = -1;
    // multistep integrator level: 1 slow, 0 fast, -1 both (coordinate nodes
    // feeding both); from the config attribute integrator_level
    int level = 0;
    virtual ~GNode() {}
    virtual void forward(Engine& e, bool energy) = 0;
    // Part of the forward work that needs only the arguments listed in
    // early_args (indices into args): the engine enqueues it once those are
    // ready, before forward(), which waits for all arguments.
    std::vector<int> early_args;
    virtual void forward_early(Engine&) {}
    virtual void backward(Engine&) {}
    virtual std::vector<float> get_param(Engine&) { return {}; }
    virtual void set_param(Engine&, const std::vector<float>&) { throw Error("set_param not supported for this node"); }
    virtual std::vector<float> param_deriv(Engine&) { return {}; }
    virtual std::vector<float> value_by_name(Engine&, const std::string& w) {
        throw Error("Value " + w + " not implemented");
    }
    virtual DGraph* graph() { return nullptr; }
    // state that one evaluation leaves for the next (the surface node's):
    // copied aside before a chunk of rounds and put back when the chunk is
    // run again after a storage overflow
    virtual void keep_state(Engine&, bool /*restore*/) {}
    // enlarge edge storage after an overflow; returns true if anything grew
    virtual bool grow(Engine&) { return false; }
    // measured kernel of this node: bracket its launches with events from
    // ev[*used..cap) (ev null: stop), and the running total of its
    // algorithmic bytes; nodes without one return false / 0
    virtual bool set_kernel_timer(cudaEvent_t*, int*, int) { return false; }
    // BP warm start (rotamer node): six FP32 weight arrays or null to keep the
    // current ones; mode 0 off, 1 learned, 2 previous marginals, 3 previous
    // messages and marginals; returns false
    // for nodes without one
    virtual bool set_warm(Engine&, const float* const*, int) { return false; }
    // tuning knobs: candidate-cache buffer scale (pair-list nodes) and the BP
    // solve's launch variant (rotamer node; false elsewhere)
    virtual void set_buffer_scale(float) {}
    virtual bool set_bp_variant(int) { return false; }
    virtual double kernel_bytes(Engine&) { return 0.0; }
    // The per-element arrays the reference's node logs at its default log
    // level, from the last evaluation made with Engine::log_detail set: name,
    // values of all systems concatenated, per-system offsets (n_sys + 1); an
    // int64 array when integer is set.
    struct Log {
        std::string name;
        std::vector<double> values;
        std::vector<int> off;
        bool integer = false;
    };
    virtual void detailed_logs(Engine&, std::vector<Log>&) {}
};

class Engine {
public:
    Engine(const std::vector<std::string>& paths, const std::vector<int>& n_atom);
    ~Engine();

    int n_sys = 0;
    std::vector<int> n_atom, atom_off;
    int atom_total = 0;
    cudaStream_t st = nullptr;

    std::vector<std::unique_ptr<GNode>> nodes;
    std::map<std::string, int> index;
    int n_pot_slots = 0;

    // device state
    float* d_pos = nullptr;   // atom_total*3
    float* d_mom = nullptr;   // atom_total*3
    double* d_pot = nullptr;  // n_pot_slots*n_sys
    double* d_energy = nullptr;  // n_sys
    int* d_status = nullptr;
    unsigned long long* d_round = nullptr;  // per-system thermostat invocation counters
    float* d_temp = nullptr;   // per-system temperature
    unsigned* d_seed = nullptr;  // per-system thermostat seed
    float* d_sens_arena = nullptr;
    size_t sens_arena_floats = 0;
    int* atom_sys_d = nullptr;
    int* atom_off_d = nullptr;

    // allocation helpers (engine owns every device buffer)
    template <class T> T* alloc(size_t n);
    template <class T> T* upload(const std::vector<T>& v);
    void free_all();

    GNode& node(const std::string& name);
    GNode& arg(const GNode& n, int i) { return *nodes[size_t(n.args.at(size_t(i)))]; }

    // enqueue one force evaluation (forward + adjoint) on the stream; with
    // level 0 or 1 only the nodes of that integrator level (and those of both)
    // run, so the position sensitivity holds that level's forces
    void compute(bool energy, int level = -2);
    // Multistep integrator (the reference's integration_cycle with
    // inner_step, src/deriv_engine.cpp:333-351): per round one slow-force
    // kick of inner_step dt, then inner_step fast stages.  Off: the plain
    // three-stage cycle.  inner_step also sets the thermostat time step.
    bool multistep = false;
    int inner_step = 3;
    // one integration round: thermostat, then 3 x {compute; p -= dt F; x += dt p}
    void round(float dt, float timescale, bool thermostat);
    // the thermostat alone (one invocation: counters advance); its time step
    // is 3 dt thermo_span (the reference's thermostat interval in rounds)
    void thermalize(float dt, float timescale);
    float thermo_span = 1.f;
    // move each system's centroid to the origin (xy_only: x and y only)
    void recenter(bool xy_only);
    // periodic box of every system (edge lengths, 0 = open): the pair lists
    // and pair terms use the minimum image; coordinates are never wrapped
    void set_box(float lx, float ly, float lz);
    float box[3] = {0.f, 0.f, 0.f};
    // host helpers
    void set_pos(const float* pos_all);     // atom_total*3
    void get_pos(float* pos_all);
    void get_deriv(float* d_all);
    void energies(double* e);               // n_sys, valid after compute(true)
    int status(bool clear);
    // evaluate with automatic growth of pair-list storage on overflow
    void compute_checked(bool energy, int level = -2);
    void sync();

    // CUDA graph of `rounds_per_graph` integration rounds
    void capture(float dt, float timescale, int rounds_per_graph);
    // forget the captured graph (its kernels hold parameters that changed)
    void drop_graph();

    // node DAG on n_lanes streams (see engine.cu); off: one stream
    bool parallel_nodes = true;
    int n_lanes = 4;
    std::vector<cudaStream_t> lanes;  // lanes[0] is st
    std::vector<int> node_lane;
    std::vector<std::vector<int>> consumers;
    std::vector<cudaEvent_t> ev_fwd, ev_bwd, ev_lane;
    void setup_lanes();
    float graph_dt = 0.f, graph_timescale = 0.f, graph_span = 1.f;  // of the captured graph
    bool graph_multistep = false;
    int graph_inner = 3;
    // integration rounds with overflow recovery (see engine.cu); with
    // thermo_interval > 1 the thermostat runs only in rounds whose number
    // (first_round + index) is a multiple of it, and no graph is used
    void run_rounds(int n_round, float dt, float timescale, bool use_graph, int graph_rounds,
                    int thermo_interval = 1, unsigned long long first_round = 0);
    float* snap_pos = nullptr;
    float* snap_mom = nullptr;
    unsigned long long* snap_round = nullptr;
    int kept_status = 0;  // status bits read (and cleared) by internal checks

    // Autotuner: times n_round integration rounds (one-round graph, CUDA
    // events) from the same saved state for each candidate setting and keeps
    // the fastest: first the candidate-cache buffer scale, then the BP launch
    // variant.  Returns (setting, ms per round) for every candidate tried.
    std::vector<std::pair<std::string, float>> autotune(int n_round, float dt, float timescale);
    // set the tuned quantities by hand
    void set_tuning(float buffer_scale, int bp_variant);
    float tuned_buffer_scale = 1.f;
    int tuned_bp_variant = 0;
    void launch_graph();
    cudaGraphExec_t graph_exec = nullptr;
    cudaGraph_t graph = nullptr;
    int graph_rounds = 0;
    // kernel timing of the measured kernel (the rotamer BP solve): with
    // timed != 0 the captured graph records kt_ev around each of its launches
    bool graph_timed = false;
    std::vector<cudaEvent_t> kt_ev;
    int kt_used = 0;
    void capture_timed(float dt, float timescale);
    double kernel_bytes();

    // Replica exchange on the device (remd.h): with a plan whose interval is
    // > 0, run_rounds exchanges after every interval-th round (counted from
    // the plan) and a captured graph holds whole intervals with their
    // exchange.  remd_done: rounds run since the plan was set.
    std::unique_ptr<Remd> remd;
    unsigned long long remd_done = 0;
    bool graph_remd = false;  // the captured graph contains exchanges
    // rounds of one timed graph: one, or one exchange interval
    int timed_rounds() const;

    size_t device_bytes = 0;
    int launches_per_compute = 0;
    // evaluations made while set also fill the nodes' log arrays
    // (GNode::detailed_logs); graphs captured while it is clear never do
    bool log_detail = false;
    // number of kernel nodes in one captured force evaluation
    int count_launches();
    // per-node device time (ms) of n eager evaluations, CUDA events on the stream
    std::vector<std::pair<std::string, float>> profile_nodes(int n);

private:
    std::vector<void*> allocations_;
    std::vector<std::unique_ptr<h5lite::File>> files_;
};

// Threefry-4x32-20 on the host (the replica-exchange random stream)
void threefry_host(const uint32_t c[4], const uint32_t k[4], uint32_t out[4]);
// exchange the coordinates of systems s1 and s2 (equal atom counts) through
// tmp (device, 3 n_atom floats), on the engine stream
void swap_coords(Engine& e, int s1, int s2, float* tmp);

}  // namespace ug
