// Test infrastructure (the reference oracle build only).  The reference's
// src/rotamer.cpp compiled unchanged, plus one accessor that copies the edge
// list of the rotamer node's bead interaction graph (InteractionGraph::
// edge_indices1/2, n_edge after compute_edges, src/interaction_graph.h:51-258)
// so the tests can compare the engine's pair lists with the reference's own,
// pair for pair and in order.  This object replaces rotamer.o in
// libupside_ref.so; nothing else changes.
#include "rotamer.cpp"

#include "edge_dump.h"

extern "C" int ref_edges_rotamer(DerivEngine* engine, const char* node, int32_t* pairs, int cap) {
    return ref_dump_graph<RotamerSidechain<preferred_bead_type>>(engine, node, pairs, cap);
}
