// CPU restatement of the Upside ff_2.1 force evaluation and integrator.
//
// TEST INFRASTRUCTURE (the oracle): used only by tests/, the smoke check and
// bench.py's CPU baseline.  It is never linked into the product library.
// It restates, node by node, the reference algorithm (src/*.cpp of
// sosnicklab/upside2-md; citations beside each node) in plain scalar C++,
// templated on the scalar type so a float instantiation tracks the reference
// and a double instantiation serves as the FP64 error yardstick.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// precision: 0 = float, 1 = double.  Returns NULL on error (message via ocpu_last_error).
void* ocpu_create(const char* up_path, int n_atom, int precision);
void ocpu_free(void* h);
const char* ocpu_last_error(void);

// Full evaluation (potential + derivative), like evaluate_energy/evaluate_deriv
// (src/engine_c_library.cpp:30-65).  pos and deriv are (n_atom,3) row-major.
int ocpu_evaluate(void* h, const float* pos, double* energy, float* deriv);

// Node introspection after ocpu_evaluate (same contract as get_output/get_sens).
int ocpu_output_dims(void* h, const char* node, int* n_elem, int* width);
int ocpu_get_output(void* h, const char* node, float* out, int n);
int ocpu_get_sens(void* h, const char* node, float* out, int n);
int ocpu_value_by_name(void* h, const char* node, const char* what, float* out, int n);
int ocpu_param_size(void* h, const char* node);
int ocpu_get_param_deriv(void* h, const char* node, float* out, int n);
int ocpu_set_param(void* h, const char* node, const float* p, int n);

// Pair list of an interaction-graph node after ocpu_evaluate: (i1,i2) index
// pairs in the reference's edge order.  Returns the number of edges (or -1);
// writes at most cap pairs.  For the rotamer node the bead graph is returned.
int ocpu_edges(void* h, const char* node, int32_t* pairs, int cap);

// Dynamics: n_round rounds of {OU thermostat, 3-stage integration_cycle}
// (src/main.cpp:974-984, src/deriv_engine.cpp:317-331, src/thermostat.cpp:9-18)
// starting from (pos, mom); round_start is the thermostat invocation counter.
int ocpu_run(void* h, float* pos, float* mom, int n_round, float dt, float temperature, float timescale,
             uint32_t seed, uint64_t round_start);

// Threefry-4x32-20 normal draws used by the thermostat (for RNG parity tests):
// fills out[3*n_atom] for one invocation.
void ocpu_thermostat_normals(uint32_t seed, uint64_t invocation, int n_atom, float* out);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
extern "C" {
#endif
// raw Threefry-4x32-20 block (known-answer tests)
void ocpu_threefry4x32(const uint32_t* ctr, const uint32_t* key, uint32_t* out);
#ifdef __cplusplus
}
#endif
