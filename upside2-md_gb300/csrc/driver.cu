// upside_main: the `upside` command-line driver on the GB300 engine
// (the reference's src/main.cpp:426-1105, declared extern "C" in src/main.h).
//
// Every configuration file is one system.  Systems whose node graphs and force
// fields agree share one batched engine (one set of kernels and one captured
// CUDA graph for all of them); the others get an engine each.  All systems
// advance in lockstep through the reference's schedule of rounds:
//
//   round nr:  if nr % frame_interval == 0:  recentre, evaluate, log a frame
//              if nr % thermostat_interval == 0:  (anneal T) thermostat
//              integration cycle (3 force evaluations)
//   after round nr with (nr + 1) % replica_interval == 0:  replica exchange
//
// Rounds between two host events run as replays of the engine's captured
// graph.  Frames go to `/output` of the configuration file (or of the file
// given with --output / --output-base) through the h5lite writer: the
// reference's arrays and shapes (src/state_logger.h, src/main.cpp:807-899),
// written every 100 frames and at the end.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <csignal>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "engine.h"
#include "h5lite.h"
#include "mc.h"

using ug::Engine;
using ug::Error;

namespace {

volatile std::sig_atomic_t g_signal = 0;
void on_signal(int sig) { g_signal = sig; }

// installs a handler for the duration of the run and puts the caller's back
struct SignalGuard {
    int sig;
    void (*old)(int);
    explicit SignalGuard(int s) : sig(s) { old = std::signal(s, on_signal); }
    ~SignalGuard() { std::signal(sig, old); }
};

const char* const UNSET = "not_Defined_By_user";

// the reference's split_string (src/main.cpp:134-145): "" gives no fields
std::vector<std::string> split(const std::string& s, const std::string& sep) {
    std::vector<std::string> out;
    size_t i = 0;
    while (i < s.size()) {
        size_t j = s.find(sep, i);
        if (j == std::string::npos) j = s.size();
        out.push_back(s.substr(i, j - i));
        i = j + sep.size();
    }
    return out;
}

double strict_double(const std::string& s) {
    size_t n = 0;
    double x = 0;
    try {
        x = std::stod(s, &n);
    } catch (...) {
        throw Error("invalid float '" + s + "'");
    }
    if (n != s.size()) throw Error("invalid float '" + s + "'");
    return x;
}
long long strict_int(const std::string& s) {
    size_t n = 0;
    long long x = 0;
    try {
        x = std::stoll(s, &n);
    } catch (...) {
        throw Error("invalid integer '" + s + "'");
    }
    if (n != s.size()) throw Error("invalid integer '" + s + "'");
    return x;
}

struct ArgError : std::runtime_error {
    std::string arg;
    ArgError(const std::string& what, const std::string& a) : std::runtime_error(what), arg(a) {}
};

// Command line of the reference (src/main.cpp:428-529), same names, defaults
// and required arguments.
struct Args {
    double time_step = 0.009, duration = -1., time_limit = -1.;
    unsigned long long seed = 42;
    std::string temperature;
    std::vector<std::string> swap_sets;
    double anneal_factor = 1., anneal_duration = -1., anneal_start = -1., anneal_end = -1.;
    double frame_interval = -1., dense_frame_interval = -1., replica_interval = 0.;
    int exchange_criterion = 0;
    double mc_interval = 0., thermostat_interval = -1., thermostat_timescale = 5.;
    double curvature_interval = 0., curvature_change = 0.05;
    std::string integrator;
    int inner_step = 3;
    std::string input = UNSET, input_base = UNSET, output = UNSET, output_base = UNSET;
    bool disable_recenter = false, disable_z_recenter = false, reraise = false;
    std::string log_level;
    bool deriv_agreement = false, record_momentum = false, restart_momentum = false;
    std::string set_param;
    std::vector<std::string> configs;
    bool help = false, version = false;
};

const char* USAGE =
    "USAGE: upside --duration <float> --frame-interval <float> [options] <config .up files> ...\n"
    "  --time-step <float>            integration time step (0.009)\n"
    "  --duration <float>             simulation time (required)\n"
    "  --frame-interval <float>       simulation time between frames (required)\n"
    "  --temperature <list>           comma-separated temperatures, one or one per system (1.0)\n"
    "  --seed <int>                   random seed (42)\n"
    "  --thermostat-timescale <float> (5.0)     --thermostat-interval <float> (every round)\n"
    "  --replica-interval <float>     time between replica exchanges (0: none)\n"
    "  --swap-set <pairs>             e.g. 0-1,2-3; repeat for more sets\n"
    "  --exchange-criterion <0|1>     (0)\n"
    "  --anneal-factor/-duration/-start/-end <float>\n"
    "  --time-limit <seconds>         stop (and write out) after this much wall time\n"
    "  -i/--input, --input-base       files holding /input/pos (and /input/mom)\n"
    "  -o/--output, --output-base     write /output to these files instead of the configs\n"
    "  --record-momentum, --restart-using-momentum, --disable-recentering,\n"
    "  --disable-z-recentering, --log-level <basic|detailed|extensive>, --set-param <file>\n";

Args parse_args(int argc, const char* const* argv) {
    Args a;
    enum Kind { VAL, SW, MULTI };
    struct Opt {
        Kind kind;
        std::function<void(const std::string&)> set;
    };
    bool have_duration = false, have_frame = false;
    std::map<std::string, Opt> opts = {
        {"time-step", {VAL, [&](const std::string& v) { a.time_step = strict_double(v); }}},
        {"duration", {VAL, [&](const std::string& v) { a.duration = strict_double(v); have_duration = true; }}},
        {"time-limit", {VAL, [&](const std::string& v) { a.time_limit = strict_double(v); }}},
        {"seed", {VAL, [&](const std::string& v) {
                      long long s = strict_int(v);
                      if (s < 0) throw Error("invalid seed '" + v + "'");
                      a.seed = (unsigned long long)s;
                  }}},
        {"temperature", {VAL, [&](const std::string& v) { a.temperature = v; }}},
        {"swap-set", {MULTI, [&](const std::string& v) { a.swap_sets.push_back(v); }}},
        {"anneal-factor", {VAL, [&](const std::string& v) { a.anneal_factor = strict_double(v); }}},
        {"anneal-duration", {VAL, [&](const std::string& v) { a.anneal_duration = strict_double(v); }}},
        {"anneal-start", {VAL, [&](const std::string& v) { a.anneal_start = strict_double(v); }}},
        {"anneal-end", {VAL, [&](const std::string& v) { a.anneal_end = strict_double(v); }}},
        {"frame-interval", {VAL, [&](const std::string& v) { a.frame_interval = strict_double(v); have_frame = true; }}},
        {"dense-frame-interval", {VAL, [&](const std::string& v) { a.dense_frame_interval = strict_double(v); }}},
        {"replica-interval", {VAL, [&](const std::string& v) { a.replica_interval = strict_double(v); }}},
        {"exchange-criterion", {VAL, [&](const std::string& v) { a.exchange_criterion = int(strict_int(v)); }}},
        {"monte-carlo-interval", {VAL, [&](const std::string& v) { a.mc_interval = strict_double(v); }}},
        {"thermostat-interval", {VAL, [&](const std::string& v) { a.thermostat_interval = strict_double(v); }}},
        {"thermostat-timescale", {VAL, [&](const std::string& v) { a.thermostat_timescale = strict_double(v); }}},
        {"curvature-changer-interval", {VAL, [&](const std::string& v) { a.curvature_interval = strict_double(v); }}},
        {"relative-curvature-radius-change", {VAL, [&](const std::string& v) { a.curvature_change = strict_double(v); }}},
        {"integrator", {VAL, [&](const std::string& v) { a.integrator = v; }}},
        {"inner-step", {VAL, [&](const std::string& v) { a.inner_step = int(strict_int(v)); }}},
        {"input", {VAL, [&](const std::string& v) { a.input = v; }}},
        {"input-base", {VAL, [&](const std::string& v) { a.input_base = v; }}},
        {"output", {VAL, [&](const std::string& v) { a.output = v; }}},
        {"output-base", {VAL, [&](const std::string& v) { a.output_base = v; }}},
        {"disable-recentering", {SW, [&](const std::string&) { a.disable_recenter = true; }}},
        {"disable-z-recentering", {SW, [&](const std::string&) { a.disable_z_recenter = true; }}},
        {"re-raise-signal", {SW, [&](const std::string&) { a.reraise = true; }}},
        {"log-level", {VAL, [&](const std::string& v) { a.log_level = v; }}},
        {"potential-deriv-agreement", {SW, [&](const std::string&) { a.deriv_agreement = true; }}},
        {"record-momentum", {SW, [&](const std::string&) { a.record_momentum = true; }}},
        {"restart-using-momentum", {SW, [&](const std::string&) { a.restart_momentum = true; }}},
        {"set-param", {VAL, [&](const std::string& v) { a.set_param = v; }}},
    };
    bool positional_only = false;
    for (int i = 1; i < argc; ++i) {
        std::string s = argv[i] ? argv[i] : "";
        if (positional_only || s.size() < 2 || s[0] != '-') {
            a.configs.push_back(s);
            continue;
        }
        if (s == "--") {
            positional_only = true;
            continue;
        }
        if (s == "-h" || s == "--help") {
            a.help = true;
            continue;
        }
        if (s == "--version") {
            a.version = true;
            continue;
        }
        std::string name, value;
        bool inline_value = false;
        if (s[1] == '-') {
            name = s.substr(2);
            size_t eq = name.find('=');
            if (eq != std::string::npos) {
                value = name.substr(eq + 1);
                name = name.substr(0, eq);
                inline_value = true;
            }
        } else if (s == "-i") {
            name = "input";
        } else if (s == "-o") {
            name = "output";
        } else {
            throw ArgError("Couldn't find match for argument", s);
        }
        auto it = opts.find(name);
        if (it == opts.end()) throw ArgError("Couldn't find match for argument", s);
        if (it->second.kind == SW) {
            if (inline_value) throw ArgError("Switch does not take a value", s);
            it->second.set("");
            continue;
        }
        if (!inline_value) {
            if (i + 1 >= argc) throw ArgError("Missing a value for this argument!", s);
            value = argv[++i];
        }
        try {
            it->second.set(value);
        } catch (const Error& e) {
            throw ArgError(e.what(), s);
        }
    }
    if (a.help || a.version) return a;
    if (!have_duration) throw ArgError("Required argument missing", "duration");
    if (!have_frame) throw ArgError("Required argument missing", "frame-interval");
    if (a.configs.empty()) throw ArgError("Required argument missing", "config_files");
    return a;
}

// ------------------------------------------------------------- logging ---
// One `/output` array: frames of a fixed row shape, or one row logged once.
struct Series {
    std::string name;
    h5lite::Dtype dt;
    std::vector<uint64_t> row;
    bool once = false;
    std::vector<uint8_t> data;
    uint64_t n = 0;
};

// The reference's H5Logger (src/state_logger.h:59-161) over the h5lite writer.
struct Logger {
    std::string path;
    h5lite::Writer w;  // in place: the configuration's tree without /output
    std::vector<Series> series;
    std::string invocation;
    size_t buffered = 0;

    Series& add(const std::string& name, const h5lite::Dtype& dt, std::vector<uint64_t> row, bool once = false) {
        for (auto& s : series)
            if (s.name == name) throw Error("output array '" + name + "' logged twice");
        Series s;
        s.name = name;
        s.dt = dt;
        s.row = std::move(row);
        s.once = once;
        series.push_back(std::move(s));
        return series.back();
    }
    Series& get(const std::string& name) {
        for (auto& s : series)
            if (s.name == name) return s;
        throw Error("no output array '" + name + "'");
    }
    static size_t row_bytes(const Series& s) {
        size_t n = size_t(s.dt.size);
        for (auto d : s.row) n *= size_t(d);
        return n;
    }
    void push(const std::string& name, const void* row) {
        Series& s = get(name);
        const uint8_t* p = static_cast<const uint8_t*>(row);
        s.data.insert(s.data.end(), p, p + row_bytes(s));
        s.n++;
    }
    template <class T> void push_vec(const std::string& name, const std::vector<T>& v) {
        Series& s = get(name);
        if (v.size() * sizeof(T) != row_bytes(s)) throw Error("output row size mismatch for '" + name + "'");
        push(name, v.data());
    }
    // after each frame: write every 100 frames (src/state_logger.h:84-91)
    void frame_done() {
        if (++buffered % 100 == 0) write();
    }
    void write() {
        w.remove("/output");
        w.group("/output");
        for (auto& s : series) {
            std::vector<uint64_t> dims;
            if (!s.once) dims.push_back(s.n);
            dims.insert(dims.end(), s.row.begin(), s.row.end());
            w.dataset("/output/" + s.name, s.dt, dims, s.data);
        }
        std::vector<uint8_t> inv(invocation.begin(), invocation.end());
        inv.push_back(0);
        w.attr("/output", "invocation", h5lite::dtype_string(int(inv.size())), {}, inv);
        w.save(path);
    }
};

// ------------------------------------------------------------- systems ---
struct Sys {
    std::string config, input, output;
    int n_atom = 0;
    int eng = -1, local = -1;
    uint32_t seed = 0;
    float T0 = 1.f, T = 1.f;
    std::unique_ptr<Logger> log;
    int replica_index = 0;
};

struct SwapPair {
    int s1, s2;
    unsigned long long n_attempt = 0, n_success = 0;
};

std::string graph_signature(h5lite::File& f) {
    std::string sig;
    for (auto& nm : f.list("/input/potential")) {
        sig += nm + "(";
        for (auto& a : f.attr_strings("/input/potential/" + nm, "arguments")) sig += a + ",";
        sig += ")";
    }
    return sig;
}

// (n_atom, 3, 1) array of a configuration or input file
std::vector<float> read_vec3(h5lite::File& f, const std::string& path, int n_atom, const std::string& file) {
    auto d = f.dims(path);
    if (d.size() != 3 || d[1] != 3) throw Error("invalid dimensions for " + path + " in " + file);
    if (d[2] != 1) throw Error("must have n_system 1 from config");
    if (int(d[0]) != n_atom)
        throw Error(path + " of " + file + " has " + std::to_string(d[0]) + " atoms, expected " +
                    std::to_string(n_atom));
    return f.read<float>(path);
}

ug::GNode* find_node(Engine& e, const std::string& name) {
    auto it = e.index.find(name);
    return it == e.index.end() ? nullptr : e.nodes[size_t(it->second)].get();
}
bool has_hbond_energy(Engine& e) {
    for (auto& kv : e.index)
        if (kv.first.compare(0, 12, "hbond_energy") == 0) return true;
    return false;
}

int run(const Args& A, const std::string& invocation, int verbose) {
    // "mv": the multistep integrator with --inner-step fast stages per round
    // (src/main.cpp:552-555); otherwise the three-stage cycle
    if (!A.integrator.empty() && A.integrator != "v" && A.integrator != "mv")
        throw Error("Illegal value for --integrator: '" + A.integrator + "' (v or mv)");
    const bool multistep = A.integrator == "mv";
    const int inner_step = multistep ? A.inner_step : 3;
    if (inner_step < 1) throw Error("--inner-step must be at least 1");
    if (A.curvature_interval != 0.) throw Error("--curvature-changer-interval is not available in the GPU driver");
    if (A.deriv_agreement) throw Error("--potential-deriv-agreement is not available in the GPU driver");
    int log_level = 1;
    if (A.log_level.empty() || A.log_level == "detailed") log_level = 1;
    else if (A.log_level == "basic") log_level = 0;
    else if (A.log_level == "extensive") log_level = 2;
    else throw Error("Illegal value for --log-level");

    const float dt = float(A.time_step);
    const unsigned long long n_round = (unsigned long long)std::llround(A.duration / (inner_step * dt));
    const long long thermo_interval = (long long)std::max(1., std::round(A.thermostat_interval / (inner_step * dt)));
    const long long frame_interval = (long long)std::max(1., std::round(A.frame_interval / (inner_step * dt)));
    const uint32_t base_seed = uint32_t(A.seed % 4294967291ull);
    if (verbose) printf("random seed: %lu\n", (unsigned long)base_seed);
    int duration_width = int(std::ceil(std::log(1. + A.duration) / std::log(10.)));
    bool do_recenter = !A.disable_recenter;
    bool xy_only = do_recenter && A.disable_z_recenter;

    int n_sys = int(A.configs.size());
    std::vector<Sys> sys(static_cast<size_t>(n_sys));
    auto temps = split(A.temperature.empty() ? std::string("1.0") : A.temperature, ",");
    if (temps.size() != 1u && int(temps.size()) != n_sys)
        throw Error("Received " + std::to_string(temps.size()) + " temperatures but have " + std::to_string(n_sys) +
                    " systems");
    for (int s = 0; s < n_sys; ++s) {
        sys[s].config = A.configs[s];
        sys[s].T0 = sys[s].T = float(strict_double(temps.size() > 1 ? temps[s] : temps[0]));
        sys[s].seed = base_seed + uint32_t(s);
        sys[s].replica_index = s;
    }
    double anneal_duration = A.anneal_duration == -1. ? A.duration : A.anneal_duration;
    double anneal_start = A.anneal_start < 0. ? 0. : A.anneal_start;
    double anneal_end = A.anneal_end;
    if (anneal_end > anneal_start) anneal_duration = anneal_end - anneal_start;
    // src/main.cpp:606-618, including its behaviour with the default end time
    auto anneal_temp = [&](double T0, double time) {
        double fraction = std::max(0., (time - anneal_start) / anneal_duration);
        double T1 = T0 * A.anneal_factor;
        if (time <= anneal_start) return T0;
        if (time > anneal_end) return T1;
        double r = std::sqrt(T0) * (1. - fraction) + std::sqrt(T1) * fraction;
        return r * r;
    };

    bool user_output = false;
    if (A.output != UNSET) {
        auto outs = split(A.output, ",");
        if (outs.size() != 1u && int(outs.size()) != n_sys)
            throw Error("Received " + std::to_string(outs.size()) + " outputs but have " + std::to_string(n_sys) +
                        " systems");
        for (int s = 0; s < n_sys; ++s) sys[s].output = outs.size() > 1 ? outs[s] : outs[0];
        user_output = true;
    }
    if (A.output_base != UNSET) {
        for (int s = 0; s < n_sys; ++s) sys[s].output = A.output_base + "_" + std::to_string(s) + ".h5";
        user_output = true;
    }
    bool user_input = false;
    if (A.input != UNSET) {
        auto ins = split(A.input, ",");
        if (ins.size() != 1u && int(ins.size()) != n_sys)
            throw Error("Received " + std::to_string(ins.size()) + " inputs but have " + std::to_string(n_sys) +
                        " systems");
        for (int s = 0; s < n_sys; ++s) sys[s].input = ins.size() > 1 ? ins[s] : ins[0];
        user_input = true;
    }
    if (A.input_base != UNSET) {
        for (int s = 0; s < n_sys; ++s) sys[s].input = A.input_base + "_" + std::to_string(s) + ".h5";
        user_input = true;
    }
    int replica_interval = 0;
    if (A.replica_interval != 0.) replica_interval = int(std::max(1., A.replica_interval / (inner_step * dt)));
    // src/main.cpp:567-569
    const int mc_interval = A.mc_interval > 0. ? std::max(1, int(A.mc_interval / (inner_step * dt))) : 0;

    // ---- configurations, positions, momenta; systems grouped into batches
    std::vector<std::vector<float>> pos0(static_cast<size_t>(n_sys)), mom0(static_cast<size_t>(n_sys));
    std::map<std::string, std::vector<int>> groups;
    std::vector<std::string> group_order;
    for (int s = 0; s < n_sys; ++s) {
        std::unique_ptr<h5lite::File> cfg;
        try {
            cfg.reset(new h5lite::File(sys[s].config));
        } catch (const std::exception&) {
            throw Error("Unable to open configuration file at " + sys[s].config);
        }
        std::unique_ptr<h5lite::File> inp;
        if (user_input) {
            try {
                inp.reset(new h5lite::File(sys[s].input));
            } catch (const std::exception&) {
                throw Error("Unable to open input position file " + sys[s].input);
            }
        }
        h5lite::File& pf = user_input ? *inp : *cfg;
        const std::string& pname = user_input ? sys[s].input : sys[s].config;
        auto d = pf.dims("/input/pos");
        if (d.size() != 3 || d[1] != 3) throw Error("invalid dimensions for initial position");
        if (d[2] != 1) throw Error("must have n_system 1 from config");
        sys[s].n_atom = int(d[0]);
        pos0[s] = read_vec3(pf, "/input/pos", sys[s].n_atom, pname);
        if (A.restart_momentum) {
            if (!pf.exists("/input/mom"))
                throw Error("input h5 file doesn't have input.mom group, can't restart using the momentum!");
            mom0[s] = read_vec3(pf, "/input/mom", sys[s].n_atom, pname);
        }
        // z-recentering with a z-dependent potential, or recentering with a
        // radial one, is refused as in src/main.cpp:852-870
        for (auto& nm : cfg->list("/input/potential")) {
            auto pre = [&](const char* p) { return nm.compare(0, strlen(p), p) == 0; };
            if (do_recenter && !xy_only &&
                (pre("membrane_potential") || pre("z_flat_bottom") || pre("tension") || pre("AFM")))
                throw Error("You have z-centering and a z-dependent potential turned on.  This is not what you want.  "
                            "Consider --disable-z-recentering or --disable-recentering.");
            if (do_recenter && (pre("cavity_radial") || pre("spherical_well")))
                throw Error("You have re-centering and a radial potential turned on.  This is not what you want.  "
                            "Consider --disable-recentering.");
        }
        std::string sig = graph_signature(*cfg);
        if (!groups.count(sig)) group_order.push_back(sig);
        groups[sig].push_back(s);
        // logger: the output file, or in place the configuration's tree
        auto lg = std::make_unique<Logger>();
        lg->invocation = invocation;
        if (user_output) {
            lg->path = sys[s].output;
        } else {
            lg->path = sys[s].config;
            h5lite::copy_tree(*cfg, "/", lg->w, "/", {"/output"});
        }
        sys[s].log = std::move(lg);
    }

    std::vector<std::unique_ptr<Engine>> engines;
    std::vector<std::vector<int>> members;
    auto make_engine = [&](const std::vector<int>& ss) {
        std::vector<std::string> paths;
        std::vector<int> na;
        for (int s : ss) {
            paths.push_back(sys[s].config);
            na.push_back(sys[s].n_atom);
        }
        engines.emplace_back(new Engine(paths, na));
        members.push_back(ss);
        for (size_t k = 0; k < ss.size(); ++k) {
            sys[ss[k]].eng = int(engines.size()) - 1;
            sys[ss[k]].local = int(k);
        }
    };
    for (auto& sig : group_order) {
        auto& ss = groups[sig];
        try {
            make_engine(ss);
        } catch (const Error& e) {
            // same graph, different force-field tables: one engine per system
            if (ss.size() == 1 || !strstr(e.what(), "differs between systems of one batch")) throw;
            for (int s : ss) make_engine({s});
        }
    }

    // --set-param: every dataset of the file's root replaces that node's
    // parameters (src/main.cpp:537-547, 750-752)
    if (!A.set_param.empty()) {
        h5lite::File pf(A.set_param);
        for (auto& nm : pf.list("/")) {
            auto v = pf.read<float>("/" + nm);
            for (auto& e : engines) e->node(nm).set_param(*e, v);
        }
    }

    // ---- thermostat and initial state
    for (size_t k = 0; k < engines.size(); ++k) {
        Engine& e = *engines[k];
        std::vector<float> pos, mom, temp;
        std::vector<uint32_t> seed;
        for (int s : members[k]) {
            pos.insert(pos.end(), pos0[s].begin(), pos0[s].end());
            if (A.restart_momentum) mom.insert(mom.end(), mom0[s].begin(), mom0[s].end());
            temp.push_back(sys[s].T);
            seed.push_back(sys[s].seed);
        }
        if (!A.restart_momentum) mom.assign(pos.size(), 0.f);
        std::vector<unsigned long long> rounds(members[k].size(), 0ull);
        e.set_pos(pos.data());
        UG_CK(cudaMemcpyAsync(e.d_mom, mom.data(), sizeof(float) * mom.size(), cudaMemcpyHostToDevice, e.st));
        UG_CK(cudaMemcpyAsync(e.d_temp, temp.data(), sizeof(float) * temp.size(), cudaMemcpyHostToDevice, e.st));
        UG_CK(cudaMemcpyAsync(e.d_seed, seed.data(), sizeof(uint32_t) * seed.size(), cudaMemcpyHostToDevice, e.st));
        UG_CK(cudaMemcpyAsync(e.d_round, rounds.data(), sizeof(unsigned long long) * rounds.size(),
                              cudaMemcpyHostToDevice, e.st));
        e.thermo_span = float(thermo_interval);
        e.multistep = multistep;
        e.inner_step = inner_step;
        // a fresh start thermalises the zero momenta once (src/main.cpp:787-791)
        if (!A.restart_momentum) e.thermalize(dt, float(A.thermostat_timescale));
        e.sync();
    }
    auto upload_temps = [&]() {
        for (size_t k = 0; k < engines.size(); ++k) {
            std::vector<float> temp;
            for (int s : members[k]) temp.push_back(sys[s].T);
            UG_CK(cudaMemcpyAsync(engines[k]->d_temp, temp.data(), sizeof(float) * temp.size(),
                                  cudaMemcpyHostToDevice, engines[k]->st));
            engines[k]->sync();
        }
    };

    // ---- Monte Carlo moves (src/main.cpp:838-841): per engine, from each
    // system's /input/pivot_moves and /input/jump_moves
    std::vector<std::unique_ptr<ug::McSampler>> samplers;
    if (mc_interval)
        for (size_t k = 0; k < engines.size(); ++k) {
            std::vector<std::string> paths;
            for (int s : members[k]) paths.push_back(sys[size_t(s)].config);
            samplers.emplace_back(new ug::McSampler(*engines[k], paths));
        }

    // ---- replica exchange (src/main.cpp:147-317)
    std::vector<std::vector<SwapPair>> swap_sets;
    std::vector<std::vector<std::pair<int, int>>> participating(static_cast<size_t>(n_sys));  // (set, pair)
    int n_attempt_swaps = 0;
    if (replica_interval) {
        for (size_t si = 0; si < A.swap_sets.size(); ++si) {
            swap_sets.emplace_back();
            for (auto& ps : split(A.swap_sets[si], ",")) {
                auto p = split(ps, "-");
                if (p.size() != 2u)
                    throw Error("invalid swap pair, because it contains " + std::to_string(p.size()) +
                                "elements but should contain 2");
                SwapPair sp;
                sp.s1 = int(strict_int(p[0]));
                sp.s2 = int(strict_int(p[1]));
                if (sp.s1 >= n_sys || sp.s2 >= n_sys || sp.s1 < 0 || sp.s2 < 0) throw Error("invalid system");
                swap_sets.back().push_back(sp);
            }
        }
        for (size_t si = 0; si < swap_sets.size(); ++si) {
            std::set<int> seen;
            for (size_t pi = 0; pi < swap_sets[si].size(); ++pi) {
                auto& sw = swap_sets[si][pi];
                if (seen.count(sw.s1) || seen.count(sw.s2) || sw.s1 == sw.s2)
                    throw Error("Overlapping indices in swap set.  No replica index can appear more than once in a "
                                "swap set.");
                seen.insert(sw.s1);
                seen.insert(sw.s2);
                participating[sw.s1].push_back({int(si), int(pi)});
                participating[sw.s2].push_back({int(si), int(pi)});
            }
        }
        if (swap_sets.empty()) throw Error("replica exchange requested but no swap sets proposed");
        for (auto& s : sys)
            if (s.n_atom != sys[0].n_atom)
                throw Error("Replica exchange requires all systems have the same number of atoms");
    }

    // ---- loggers (src/main.cpp:794-835, 199-222, 884-890)
    for (int s = 0; s < n_sys; ++s) {
        Logger& L = *sys[s].log;
        uint64_t na = uint64_t(sys[s].n_atom);
        L.add("pos", h5lite::dtype_float(4), {1, na, 3});
        if (A.record_momentum) L.add("mom", h5lite::dtype_float(4), {1, na, 3});
        L.add("kinetic", h5lite::dtype_float(8), {1});
        L.add("potential", h5lite::dtype_float(8), {1});
        L.add("time", h5lite::dtype_float(8), {});
        if (replica_interval) {
            L.add("replica_index", h5lite::dtype_int(4, true), {1});
            std::vector<int32_t> partner;
            for (auto& pp : participating[s]) {
                auto& sw = swap_sets[pp.first][pp.second];
                partner.push_back(sw.s1 != s ? sw.s1 : sw.s2);
            }
            Series& P = L.add("replica_swap_partner", h5lite::dtype_int(4, true), {uint64_t(partner.size())}, true);
            P.data.assign(reinterpret_cast<uint8_t*>(partner.data()),
                          reinterpret_cast<uint8_t*>(partner.data()) + 4 * partner.size());
            L.add("replica_cumulative_swaps", h5lite::dtype_int(4, true), {uint64_t(participating[s].size()), 2});
        }
        L.add("temperature", h5lite::dtype_float(8), {1});
        if (mc_interval) {  // [successes, attempts] since the previous frame
            auto& smp = *samplers[size_t(sys[s].eng)];
            if (smp.has_pivot[size_t(sys[s].local)]) L.add("pivot_stats", h5lite::dtype_int(4, true), {2});
            if (smp.has_jump[size_t(sys[s].local)]) L.add("jump_stats", h5lite::dtype_int(4, true), {2});
        }
        ug::GNode* hbn = find_node(*engines[size_t(sys[s].eng)], "protein_hbond");
        if (log_level >= 1 && hbn) {
            int ne = hbn->off[size_t(sys[s].local) + 1] - hbn->off[size_t(sys[s].local)];
            L.add("hbond", h5lite::dtype_float(4), {uint64_t(ne)});
        }
    }

    auto evaluate_all = [&](std::vector<double>& pot) {
        pot.assign(static_cast<size_t>(n_sys), 0.);
        for (size_t k = 0; k < engines.size(); ++k) {
            engines[k]->compute_checked(true);
            std::vector<double> e(members[k].size());
            engines[k]->energies(e.data());
            for (size_t j = 0; j < members[k].size(); ++j) pot[size_t(members[k][j])] = e[j];
        }
    };

    if (verbose && multistep) {  // src/deriv_engine.cpp:214-236
        Engine& e = *engines[0];
        printf("\nUsing the multi-step integrator\nslow motion\n  time step: %g\n  potential terms:\n",
               double(dt) * inner_step);
        for (auto& n : e.nodes)
            if (n->potential && n->level == 1) printf("    %s\n", n->name.c_str());
        printf("\nfast motion\n  time step: %g\n  potential terms:\n", double(dt));
        for (auto& n : e.nodes)
            if (n->potential && n->level == 0) printf("    %s\n", n->name.c_str());
    }
    if (verbose) {
        printf("\n");
        for (int s = 0; s < n_sys; ++s) printf("%s\nn_atom %i\n\n", sys[s].config.c_str(), sys[s].n_atom);
        for (int s = 0; s < n_sys; ++s) printf("%i %.2f\n", s, sys[s].T);
        printf("\nInitial potential energy:");
        std::vector<double> pot;
        evaluate_all(pot);
        for (double p : pot) printf(" %.2f", p);
        printf("\n");
    }

    // one frame of every system (src/main.cpp:946-968)
    unsigned long long round_num = 0;
    auto log_frame = [&]() {
        if (do_recenter)
            for (auto& e : engines) e->recenter(xy_only);
        std::vector<double> pot;
        // at the detailed level the nodes also fill their per-element logs
        for (auto& e : engines) e->log_detail = log_level >= 1;
        evaluate_all(pot);
        for (auto& e : engines) e->log_detail = false;
        for (size_t k = 0; k < engines.size(); ++k) {
            Engine& e = *engines[k];
            std::vector<ug::GNode::Log> node_logs;
            if (log_level >= 1)
                for (auto& n : e.nodes) n->detailed_logs(e, node_logs);
            std::vector<float> pos(3 * size_t(e.atom_total)), mom(3 * size_t(e.atom_total));
            UG_CK(cudaMemcpyAsync(pos.data(), e.d_pos, 4 * pos.size(), cudaMemcpyDeviceToHost, e.st));
            UG_CK(cudaMemcpyAsync(mom.data(), e.d_mom, 4 * mom.size(), cudaMemcpyDeviceToHost, e.st));
            std::vector<float> hb;
            ug::GNode* hbn = find_node(e, "protein_hbond");
            bool count_hbonds = has_hbond_energy(e);
            if (hbn) {
                hb.resize(size_t(hbn->total) * size_t(hbn->width));
                UG_CK(cudaMemcpyAsync(hb.data(), hbn->out, 4 * hb.size(), cudaMemcpyDeviceToHost, e.st));
            }
            e.sync();
            for (size_t j = 0; j < members[k].size(); ++j) {
                int s = members[k][j];
                Sys& S = sys[size_t(s)];
                Logger& L = *S.log;
                size_t a0 = size_t(e.atom_off[j]), na = size_t(S.n_atom);
                L.push("pos", pos.data() + 3 * a0);
                if (A.record_momentum) L.push("mom", mom.data() + 3 * a0);
                // (1/2) <|p|^2>: FP32 squares, FP64 sum (src/main.cpp:814-818)
                double kin = 0.;
                for (size_t a = 0; a < na; ++a) {
                    const float* p = mom.data() + 3 * (a0 + a);
                    kin += double(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
                }
                kin *= 0.5 / double(na);
                L.push_vec("kinetic", std::vector<double>{kin});
                L.push_vec("potential", std::vector<double>{pot[size_t(s)]});
                // the reference forms the time in FP32: (3 dt) * round (src/main.cpp:823-824)
                L.push_vec("time", std::vector<double>{double(float(inner_step) * dt * float(round_num))});
                if (replica_interval) {
                    L.push_vec("replica_index", std::vector<int32_t>{int32_t(S.replica_index)});
                    std::vector<int32_t> cum;
                    for (auto& pp : participating[size_t(s)]) {
                        auto& sw = swap_sets[size_t(pp.first)][size_t(pp.second)];
                        cum.push_back(int32_t(sw.n_success));
                        cum.push_back(int32_t(sw.n_attempt));
                    }
                    L.push("replica_cumulative_swaps", cum.data());
                }
                L.push_vec("temperature", std::vector<double>{double(S.T)});
                if (mc_interval) {
                    auto& smp = *samplers[k];
                    for (int q = 0; q < 2; ++q) {
                        if (!(q == 0 ? smp.has_pivot : smp.has_jump)[j]) continue;
                        L.push_vec(q == 0 ? "pivot_stats" : "jump_stats",
                                   std::vector<int32_t>{int32_t(smp.success[q][j]), int32_t(smp.attempt[q][j])});
                        smp.success[q][j] = smp.attempt[q][j] = 0;
                    }
                }
                double n_hbond = -1.;
                if (hbn) {
                    int r0 = hbn->off[j], r1 = hbn->off[j + 1];
                    std::vector<float> col;
                    for (int r = r0; r < r1; ++r) col.push_back(hb[size_t(r) * size_t(hbn->width) + 6]);
                    if (log_level >= 1) L.push_vec("hbond", col);
                    if (count_hbonds) {
                        n_hbond = 0.;
                        for (float c : col) n_hbond += c;
                    }
                }
                // node-level arrays (rotamer_*, rama_map_potential,
                // sigmoid_coupling), registered at the first frame
                for (auto& lg : node_logs) {
                    int a = lg.off[j], z = lg.off[j + 1];
                    bool known = false;
                    for (auto& se : L.series) known = known || se.name == lg.name;
                    if (!known) {
                        if (L.buffered != 0) throw Error("node log '" + lg.name + "' appeared after the first frame");
                        L.add(lg.name, lg.integer ? h5lite::dtype_int(8, true) : h5lite::dtype_float(4),
                              {uint64_t(z - a)});
                    }
                    if (lg.integer) {
                        std::vector<int64_t> row;
                        for (int i = a; i < z; ++i) row.push_back(int64_t(lg.values[size_t(i)]));
                        L.push_vec(lg.name, row);
                    } else {
                        std::vector<float> row;
                        for (int i = a; i < z; ++i) row.push_back(float(lg.values[size_t(i)]));
                        L.push_vec(lg.name, row);
                    }
                }
                if (verbose) {
                    double com[3] = {0, 0, 0}, rg = 0.;
                    for (size_t a = 0; a < na; ++a)
                        for (int d = 0; d < 3; ++d) com[d] += pos[3 * (a0 + a) + d];
                    for (double& c : com) c /= double(na);
                    for (size_t a = 0; a < na; ++a)
                        for (int d = 0; d < 3; ++d) {
                            double x = pos[3 * (a0 + a) + d] - com[d];
                            rg += x * x;
                        }
                    rg = std::sqrt(rg / double(na));
                    printf("%*.0f / %*.0f elapsed %2i system %.2f temp %5.1f hbonds, Rg %5.1f A, potential % 8.2f\n",
                           duration_width, double(round_num) * double(inner_step) * double(dt), duration_width,
                           A.duration, s, S.T, n_hbond, rg, pot[size_t(s)]);
                }
                L.frame_done();
            }
        }
        if (verbose) fflush(stdout);
    };

    float* swap_tmp = nullptr;
    auto swap_systems = [&](int a, int b) {
        Sys &A1 = sys[size_t(a)], &B1 = sys[size_t(b)];
        if (!swap_tmp) UG_CK(cudaMalloc(&swap_tmp, sizeof(float) * 3 * size_t(A1.n_atom)));
        if (A1.eng == B1.eng) {
            ug::swap_coords(*engines[size_t(A1.eng)], A1.local, B1.local, swap_tmp);
            engines[size_t(A1.eng)]->sync();
        } else {
            Engine &ea = *engines[size_t(A1.eng)], &eb = *engines[size_t(B1.eng)];
            ea.sync();
            eb.sync();
            size_t n = sizeof(float) * 3 * size_t(A1.n_atom);
            float* pa = ea.d_pos + 3 * size_t(ea.atom_off[size_t(A1.local)]);
            float* pb = eb.d_pos + 3 * size_t(eb.atom_off[size_t(B1.local)]);
            UG_CK(cudaMemcpy(swap_tmp, pa, n, cudaMemcpyDeviceToDevice));
            UG_CK(cudaMemcpy(pa, pb, n, cudaMemcpyDeviceToDevice));
            UG_CK(cudaMemcpy(pb, swap_tmp, n, cudaMemcpyDeviceToDevice));
        }
        std::swap(A1.replica_index, B1.replica_index);
    };
    // src/main.cpp:243-316; energies and acceptance in FP64, uniform draws from
    // the replica-exchange Threefry stream (seed, stream 1) at (round, 0, 0, k)
    auto attempt_swaps = [&](unsigned long long round) {
        int select = n_attempt_swaps % int(swap_sets.size());
        auto& set = swap_sets[size_t(select)];
        uint32_t key[4] = {base_seed, 1u, 0u, 0u};
        uint32_t ctr[4] = {uint32_t(round & 0xffffffffu), uint32_t(round >> 32), 0u, 0u};
        auto uniform = [&]() {
            uint32_t bits[4];
            ug::threefry_host(ctr, key, bits);
            ctr[3]++;
            return double(float(bits[0]) * (1.f / 4294967296.f) + (0.5f / 4294967296.f));
        };
        auto lboltz = [&](std::vector<double>& out) {
            std::vector<double> pot;
            evaluate_all(pot);
            out.resize(pot.size());
            for (size_t s = 0; s < pot.size(); ++s) out[s] = -pot[s] / double(sys[s].T);
        };
        if (A.exchange_criterion == 0) {
            std::vector<double> before, after;
            lboltz(before);
            for (auto& sp : set) swap_systems(sp.s1, sp.s2);
            lboltz(after);
            for (auto& sp : set) {
                sp.n_attempt++;
                double diff = (after[size_t(sp.s1)] + after[size_t(sp.s2)]) -
                              (before[size_t(sp.s1)] + before[size_t(sp.s2)]);
                if (diff < 0. && std::exp(diff) < uniform()) swap_systems(sp.s1, sp.s2);
                else sp.n_success++;
            }
        } else if (A.exchange_criterion == 1) {
            std::vector<double> lb;
            lboltz(lb);
            for (auto& sp : set) {
                sp.n_attempt++;
                double diff = lb[size_t(sp.s2)] - lb[size_t(sp.s1)];
                if (diff >= 0. || std::exp(diff) >= uniform()) {
                    swap_systems(sp.s1, sp.s2);
                    sp.n_success++;
                }
            }
        }
        n_attempt_swaps++;
    };

    // ---- main loop (src/main.cpp:913-997), all systems in lockstep
    SignalGuard sigint(SIGINT), sigterm(SIGTERM);
    g_signal = 0;
    bool passed_time_limit = false;
    const int graph_rounds = 16;
    const float timescale = float(A.thermostat_timescale);
    auto t0 = std::chrono::steady_clock::now();
    auto elapsed = [&]() { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); };
    bool annealing = A.anneal_factor != 1.;
    while (round_num < n_round && !g_signal) {
        unsigned long long last_start = round_num;
        bool do_break = false;
        while (!do_break && round_num < n_round) {
            if (g_signal) break;
            if (A.time_limit > 0. && elapsed() > A.time_limit) {
                passed_time_limit = true;
                break;
            }
            unsigned long long nr = round_num;
            // Monte Carlo moves, not at round 0 (src/main.cpp:941-944)
            if (nr && mc_interval && nr % (unsigned long long)mc_interval == 0)
                for (auto& smp : samplers) smp->step(nr, nullptr);
            if (nr % (unsigned long long)frame_interval == 0) log_frame();
            // the rounds up to the next host event
            unsigned long long end = std::min<unsigned long long>(n_round, (nr / frame_interval + 1) * frame_interval);
            unsigned long long brk = ~0ull;  // round after which replica exchange interrupts
            if (replica_interval) {
                unsigned long long r = nr;
                while (!(r > last_start && (r + 1) % (unsigned long long)replica_interval == 0)) ++r;
                brk = r;
                end = std::min(end, brk + 1);
            }
            if (mc_interval) end = std::min(end, (nr / mc_interval + 1) * (unsigned long long)mc_interval);
            if (annealing) {
                if (nr % (unsigned long long)thermo_interval == 0) {
                    for (auto& S : sys) S.T = float(anneal_temp(S.T0, double(inner_step) * double(dt) * double(nr + 1)));
                    upload_temps();
                }
                end = std::min(end, (nr / thermo_interval + 1) * thermo_interval);
            }
            int k = int(end - nr);
            for (auto& e : engines) e->run_rounds(k, dt, timescale, true, graph_rounds, int(thermo_interval), nr);
            round_num = end;
            if (brk != ~0ull && round_num == brk + 1) do_break = true;
        }
        if (g_signal || passed_time_limit) break;
        if (replica_interval && round_num % (unsigned long long)replica_interval == 0) attempt_swaps(round_num);
    }
    double secs = elapsed();
    if (swap_tmp) cudaFree(swap_tmp);
    if (g_signal) fprintf(stderr, "Received early termination signal\n");
    if (passed_time_limit) fprintf(stderr, "Passed time limit\n");
    for (auto& S : sys) S.log->write();

    if (verbose) {
        double rounds = double(std::max(1ull, round_num));
        printf("\n\nfinished in %.1f seconds (%.2f us/systems/step, %.1e simulation_time_unit/hour)\n", secs,
               secs * 1e6 / double(n_sys) / rounds / inner_step, rounds * inner_step * dt / secs * 3600.);
        printf("\navg_kinetic_energy/1.5kT");
        for (auto& S : sys) {
            Series& K = S.log->get("kinetic");
            const double* kin = reinterpret_cast<const double*>(K.data.data());
            double sum = 0.;
            long n = 0;
            for (uint64_t f = 0; f < K.n; ++f)
                if (f > K.n / 2) {
                    sum += kin[f];
                    ++n;
                }
            printf(" % .3f", sum / double(n) / (1.5 * S.T));
        }
        printf("\n");
    }
    int sig = int(g_signal);
    if (A.reraise && sig) std::raise(sig);
    return 0;
}

}  // namespace

extern "C" int upside_main(int argc, const char* const* argv, int verbose) {
    Args A;
    try {
        A = parse_args(argc, argv);
    } catch (const ArgError& e) {
        fprintf(stderr, "\n\nERROR: %s for argument %s\n", e.what(), e.arg.c_str());
        return 1;
    } catch (const std::exception& e) {
        fprintf(stderr, "\n\nERROR: %s\n", e.what());
        return 1;
    }
    if (A.help) {
        printf("%s", USAGE);
        fflush(stdout);
        return 0;
    }
    if (A.version) {
        printf("upside (GB300 driver) 2.0alpha\n");
        fflush(stdout);
        return 0;
    }
    std::string invocation(argc > 0 && argv[0] ? argv[0] : "upside");
    for (int i = 1; i < argc; ++i) invocation += std::string(" ") + (argv[i] ? argv[i] : "");
    if (verbose) printf("invocation: %s\n", invocation.c_str());
    int rc = 1;
    try {
        rc = run(A, invocation, verbose);
    } catch (const std::exception& e) {
        fprintf(stderr, "\n\nERROR: %s\n", e.what());
    }
    fflush(stdout);
    return rc;
}
