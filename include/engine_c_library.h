/* Drop-in C ABI of the GB300 Upside engine (libupside.so).
 *
 * The declarations mirror the reference's engine C library one for one
 * (src/engine_c_library.h:6-33 of sosnicklab/upside2-md), so existing callers
 * - py/upside_engine.py (ctypes, :46-91) and the training scripts - work
 * unchanged.  Every call is synchronous at the API edge; buffers are
 * caller-owned and copied; errors are returned as non-zero codes with a
 * message on stderr, never as exceptions.
 */
#ifndef UPSIDE_GB300_ENGINE_C_LIBRARY_H
#define UPSIDE_GB300_ENGINE_C_LIBRARY_H

#ifdef __cplusplus
extern "C" {
#else
#include <stdbool.h>
#endif

struct DerivEngine;

/* Replaces construct_deriv_engine (src/engine_c_library.cpp:9-21): reads the
 * node graph under /input/potential of the `.up` file and uploads it to the
 * GPU.  NULL on error. */
struct DerivEngine* construct_deriv_engine(int n_atom, const char* potential_file, bool quiet);
/* Replaces free_deriv_engine (src/engine_c_library.cpp:24-26). */
void free_deriv_engine(struct DerivEngine* engine);

/* Replaces evaluate_energy / evaluate_deriv (src/engine_c_library.cpp:30-65):
 * pos is (n_atom,3) row-major FP32; a full potential + derivative evaluation
 * runs; the energy (1 float) or dE/dx (n_atom,3) is returned.  0 on success. */
int evaluate_energy(float* energy, struct DerivEngine* engine, const float* pos);
int evaluate_deriv(float* deriv, struct DerivEngine* engine, const float* pos);

/* Replace set_param / get_param / get_param_deriv (src/engine_c_library.cpp:68-110).
 * get_param_deriv uses the state of the last evaluation. */
int set_param(int n_param, const float* param, struct DerivEngine* engine, const char* node_name);
int get_param_deriv(int n_param, float* deriv, struct DerivEngine* engine, const char* node_name);
int get_param(int n_param, float* param, struct DerivEngine* engine, const char* node_name);

/* Replace get_output_dims / get_output / get_sens (src/engine_c_library.cpp:113-178):
 * coordinate nodes give (n_elem, elem_width) row-major values; potential
 * nodes give one value (their potential, also for get_sens). */
int get_output_dims(int* n_elem, int* elem_width, struct DerivEngine* engine, const char* node_name);
int get_output(int n_output, float* output, struct DerivEngine* engine, const char* node_name);
int get_sens(int n_output, float* output, struct DerivEngine* engine, const char* node_name);

/* Replaces get_value_by_name (src/engine_c_library.cpp:181-195). */
int get_value_by_name(int n_output, float* output, struct DerivEngine* engine, const char* node_name,
                      const char* log_name);

/* Stateless clamped-spline helpers (src/engine_c_library.cpp:197-277). */
int clamped_spline_solve(int N, float* bspline_coeff, const float* values);
int clamped_spline_value(int N, float* result, const float* bspline_coeff, int nx, float* x);
int get_clamped_value_and_deriv(int N, float* result, const float* bspline_coeff, int nx, float* x);
int get_clamped_coeff_deriv(int N, float* result, const float* bspline_coeff, float x);

#ifdef __cplusplus
}
#endif
#endif
