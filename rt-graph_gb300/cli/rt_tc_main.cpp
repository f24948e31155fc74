// rt_tc <graph.edge> <device_id> — drop-in for tc/rt_tc/main.cpp with the same result lines;
// the ray-tracing count is replaced by the GB300 batched intersection kernel.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "rtg_reference.h"

int main(int argc, char *argv[]) {
    if (argc != 3) {
        std::printf("Usage: ./rt_tc graph_file device_id\n");
        std::exit(1);
    }
    std::string graph_file = argv[1];
    int device_id = std::atoi(argv[2]);

    Graph graph(device_id);
    graph.ReadBinaryEdges(graph_file);
    graph.TCPreprocessing();
    graph.ConvertToCSR();
    std::printf("After preprocessing: nodes = %u, edges = %u\n", graph.graph_info_.nodes,
                graph.graph_info_.edges);

    RTTC tc(device_id);
    tc.BuildBVHAndComputeRay(graph.adjs_.data(), graph.offsets_.data(), graph.graph_info_);
    tc.CountTriangles();

    std::cout << "==========>>> Result <<<==========\n";
    std::cout << "GAS Memory Size = " << 1.0 * tc.bvh_memory_size_ / 1024 / 1024 / 1024 << " GB\n";
    std::cout << "BVH Building Time = " << tc.bvh_building_time_ << " ms\n";
    std::cout << "Counting Time = " << tc.counting_time_ << " ms\n";
    std::cout << "Triangle Counting = " << tc.total_triangles_ << std::endl;
    return 0;
}
