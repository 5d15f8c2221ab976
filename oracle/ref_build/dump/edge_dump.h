// Test infrastructure: copy the current edge list of a reference node's
// interaction graph (member `igraph`) as (index1, index2) pairs in the
// reference's order.  Returns the number of edges (pairs past cap are not
// written), -1 if the node is missing or of another type.
#pragma once
#include <cstdint>
#include <string>

template <class NodeT>
int ref_dump_graph(DerivEngine* engine, const char* node, int32_t* pairs, int cap) {
    try {
        auto* n = dynamic_cast<NodeT*>(engine->get(std::string(node)).computation.get());
        if (!n) return -1;
        const auto& g = n->igraph;
        for (int e = 0; e < g.n_edge && e < cap; ++e) {
            pairs[2 * e] = g.edge_indices1[e];
            pairs[2 * e + 1] = g.edge_indices2[e];
        }
        return g.n_edge;
    } catch (...) {
        return -1;
    }
}
