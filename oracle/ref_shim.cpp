// Host-side stand-in for ThrustSortEdgesInBatch (tc/graph/thrust_helper.cu:16-42) so the
// reference's unmodified tc/graph/graph.cpp links and runs without a GPU. Same contract:
// edges with a -1 endpoint are skipped, the rest are sorted lexicographically by
// (src, dst) and packed to the front of the vector; the tail keeps stale entries, which
// Graph::ConvertToCSR never reads. TEST INFRASTRUCTURE ONLY.
#include <algorithm>
#include <vector>

#include "model.h"

void ThrustSortEdgesInBatch(std::vector<edge_t> &edge_list, int /*nodes*/) {
    std::vector<edge_t> kept;
    kept.reserve(edge_list.size());
    for (const edge_t &e : edge_list)
        if (e.src != -1 && e.dst != -1) kept.push_back(e);
    std::sort(kept.begin(), kept.end(), [](const edge_t &a, const edge_t &b) { return a < b; });
    std::copy(kept.begin(), kept.end(), edge_list.begin());
}

void ThrustSortEdges(std::vector<edge_t> &edge_list) {
    std::sort(edge_list.begin(), edge_list.end(),
              [](const edge_t &a, const edge_t &b) { return a < b; });
}
