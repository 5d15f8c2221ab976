// Test infrastructure (the reference oracle build only): src/environment.cpp
// compiled unchanged plus edge-list accessors for its coverage graphs
// (environment_coverage, hb_environment_coverage); replaces environment.o in
// libupside_ref.so.
#include "environment.cpp"

#include "edge_dump.h"

extern "C" int ref_edges_environment_coverage(DerivEngine* engine, const char* node, int32_t* pairs, int cap) {
    return ref_dump_graph<EnvironmentCoverage>(engine, node, pairs, cap);
}
extern "C" int ref_edges_hb_environment_coverage(DerivEngine* engine, const char* node, int32_t* pairs, int cap) {
    return ref_dump_graph<HbondEnvironmentCoverage>(engine, node, pairs, cap);
}
