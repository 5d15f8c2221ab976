// Test infrastructure (the reference oracle build only): src/hbond.cpp
// compiled unchanged plus edge-list accessors for its interaction-graph nodes
// (protein_hbond, hbond_coverage); replaces hbond.o in libupside_ref.so.
#include "hbond.cpp"

#include "edge_dump.h"

extern "C" int ref_edges_protein_hbond(DerivEngine* engine, const char* node, int32_t* pairs, int cap) {
    return ref_dump_graph<ProteinHBond>(engine, node, pairs, cap);
}
extern "C" int ref_edges_hbond_coverage(DerivEngine* engine, const char* node, int32_t* pairs, int cap) {
    return ref_dump_graph<HBondCoverage>(engine, node, pairs, cap);
}
