// bs_tc <graph.edge> <device_id> — drop-in for tc/bs_tc/main.cu: read the binary edge list,
// preprocess as the reference does, count on the GPU and print
// "BSTC: counting time = %f ms, counting result = %llu".
#include <cstdio>
#include <cstdlib>
#include <string>

#include "rtg_reference.h"

int main(int argc, char *argv[]) {
    if (argc != 3) {
        std::printf("Usage: ./bs_rt graph device_id\n");
        std::exit(1);
    }
    std::string graph_file = argv[1];
    int device_id = std::atoi(argv[2]);
    Graph graph(device_id);
    graph.ReadBinaryEdges(graph_file);
    graph.TCPreprocessing();
    graph.ConvertToCSR();
    CountOnGPU(graph.adjs_.data(), graph.offsets_.data(), graph.graph_info_.nodes,
               graph.graph_info_.edges, device_id);
    return 0;
}
