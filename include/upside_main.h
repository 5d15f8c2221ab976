/* The upside command-line driver, exported by libupside.so for in-process
 * callers (py/upside_engine.py:94-118 of the reference calls it through
 * ctypes as in_process_upside).  Same declaration as the reference's
 * src/main.h:1-3 and the same command line as src/main.cpp:428-529: systems
 * are the configuration files given, output goes to /output of each file (or
 * to --output / --output-base files), return value 0 on success, 1 on a bad
 * argument or a failed run (message on stderr).  The GPU driver runs on the
 * current CUDA device; options of the reference that it does not support
 * (--curvature-changer-interval, --potential-deriv-agreement) are refused
 * with an error. */
#ifndef UPSIDE_GB300_MAIN_H
#define UPSIDE_GB300_MAIN_H
#ifdef __cplusplus
extern "C" {
#endif

int upside_main(int argc, const char* const* argv, int verbose);

#ifdef __cplusplus
}
#endif
#endif
