// Driver around the reference's own host code, compiled from the reference sources by
// oracle/build_ref.sh into oracle/_ref/. TEST INFRASTRUCTURE ONLY: it produces the golden
// vectors that pin the oracle (tests/golden/make_golden.py).
//
//   ref_driver tc <edges.bin> <csr_out.bin>
//       Graph::ReadBinaryEdges -> TCPreprocessing -> ConvertToCSR (tc/graph/graph.cpp),
//       then the reference's two-hop Preprocessing (tc/bs_tc/bs_tc.cu:153-211) and the
//       HashmapKernel rule (bs_tc.cu:213-229: add cnt when w is an out-neighbour of u,
//       restated on the host because the kernel itself needs a GPU). Writes
//       int32 nodes, int32 edges, int32 offsets[nodes+1], int32 adjs[edges] and prints
//       "REF_TC <nodes> <edges> <count>".
//   ref_driver si_single <len> <skew> <selectivity> <density> <num_a> <outdir>
//   ref_driver si_multi <len> <skew> <selectivity> <distribution> <lambda> <num_a> <num_b> <outdir>
//       set_intersection/data_generator/data.cpp Data::Generator + Writer.
#include <malloc.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "data.h"
#include "graph.h"

void Preprocessing(int *adjs, int *offsets, uint nodes, std::vector<uint> &ray_origins_vals);

static bool binary_check(const int *data, int l, int r, int val) {
    while (l <= r) {
        int mid = (l + r) >> 1;
        if (data[mid] == val) return true;
        if (data[mid] < val) l = mid + 1;
        else r = mid - 1;
    }
    return false;
}

int main(int argc, char **argv) {
    // Graph::ReadBinaryEdges relies on malloc returning zeroed memory (graph.cpp:47-48);
    // serving every allocation from fresh mmap'd pages makes that hold for small inputs too.
    mallopt(M_MMAP_THRESHOLD, 0);
    if (argc < 2) {
        std::fprintf(stderr, "usage: ref_driver tc|si_single|si_multi ...\n");
        return 1;
    }
    std::string mode = argv[1];
    if (mode == "tc" && argc == 4) {
        std::string path = argv[2];
        Graph g;
        g.ReadBinaryEdges(path);
        g.TCPreprocessing();
        g.ConvertToCSR();
        int nodes = g.graph_info_.nodes, edges = g.graph_info_.edges;
        std::ofstream out(argv[3], std::ios::binary);
        out.write((const char *)&nodes, 4);
        out.write((const char *)&edges, 4);
        out.write((const char *)g.offsets_.data(), 4 * (size_t)(nodes + 1));
        out.write((const char *)g.adjs_.data(), 4 * (size_t)edges);
        out.close();
        std::vector<uint> triples;
        unsigned long long count = 0;
        if (nodes > 0) {
            Preprocessing(g.adjs_.data(), g.offsets_.data(), (uint)nodes, triples);
            for (size_t t = 0; t + 2 < triples.size(); t += 3) {
                uint u = triples[t], w = triples[t + 1], c = triples[t + 2];
                int len = g.offsets_[u + 1] - g.offsets_[u];
                if (len == 0) continue;
                if (binary_check(g.adjs_.data() + g.offsets_[u], 0, len - 1, (int)w)) count += c;
            }
        }
        std::printf("REF_TC %d %d %llu\n", nodes, edges, count);
        return 0;
    }
    if (mode == "si_single" && argc == 8) {
        Data d((uint)std::atoi(argv[6]), 1);
        d.Generator((uint32_t)std::atoi(argv[2]), std::atof(argv[3]), std::atof(argv[4]),
                    std::atof(argv[5]));
        d.Writer(argv[7]);
        return 0;
    }
    if (mode == "si_multi" && argc == 10) {
        Data d((uint)std::atoi(argv[7]), (uint)std::atoi(argv[8]));
        d.Generator((uint32_t)std::atoi(argv[2]), std::atof(argv[3]), std::atof(argv[4]),
                    static_cast<Distribution>(std::atoi(argv[5])), std::atof(argv[6]));
        d.Writer(argv[9]);
        return 0;
    }
    std::fprintf(stderr, "bad arguments\n");
    return 1;
}
