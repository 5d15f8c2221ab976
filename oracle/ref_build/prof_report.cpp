// Test infrastructure: the reference engine's own per-node timer report
// (TimeKeeper::print_report, src/timing.h:8-31, src/timing.cpp:11-55), for a
// library built with COLLECT_PROFILE (the "prof" target of this Makefile),
// where every node's compute and derivative pass runs under a Timer.
#include "timing.h"

extern "C" void ref_time_report(int n_steps) { global_time_keeper.print_report(n_steps); }
