// Triangle-counting side of the reference interface over librtg: Graph (read, preprocess,
// CSR), CountOnGPU and RTTC. Preprocessing runs on the GPU with the reference's exact rules
// (RTG_ORIENT_DEGREE_RAW_REF), so adjs_/offsets_ equal what tc/graph/graph.cpp produces.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>

#include "rtg_reference.h"

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

void check(rtg_status s, rtg_ctx *ctx, const char *what) {
    if (s == RTG_OK) return;
    std::printf("RTG error: %s: %s (%d) %s\n", what, rtg_status_str(s), (int)s,
                ctx ? rtg_last_error(ctx) : "");
    std::exit(2);
}

rtg_ctx *open_ctx(int device) {
    rtg_ctx *ctx = nullptr;
    check(rtg_init(device, &ctx), nullptr, "rtg_init");
    return ctx;
}

}  // namespace

// --------------------------------------------------------------------------- Graph

Graph::Graph(int device_id) : device_(device_id) {}
Graph::Graph() {}

Graph::~Graph() {
    if (g_) rtg_graph_destroy(g_);
    if (ctx_) rtg_destroy(ctx_);
}

void Graph::ReadBinaryEdges(std::string &input_file_path) {
    std::ifstream probe(input_file_path, std::ios::binary | std::ios::ate);
    if (!probe) {
        std::cerr << "Error: file not found" << std::endl;
        std::exit(-1);
    }
    const size_t file_size = (size_t)probe.tellg();
    probe.close();
    std::cout << "The size of graph file: " << file_size << " bytes\n";
    uint64_t m = 0;
    check(rtg_edges_read(input_file_path.c_str(), RTG_FMT_EDGE_BIN, &m, nullptr, nullptr), nullptr,
          "read edges");
    src_.resize(m ? m : 1);
    dst_.resize(m ? m : 1);
    check(rtg_edges_read(input_file_path.c_str(), RTG_FMT_EDGE_BIN, &m, src_.data(), dst_.data()),
          nullptr, "read edges");
    src_.resize(m);
    dst_.resize(m);
    // nodes = number of distinct ids (the dense rank space of graph.cpp:40-62)
    uint32_t max_id = 0;
    for (uint64_t i = 0; i < m; ++i) max_id = std::max(max_id, std::max(src_[i], dst_[i]));
    std::vector<uint8_t> used(m ? (size_t)max_id + 1 : 0, 0);
    for (uint64_t i = 0; i < m; ++i) used[src_[i]] = used[dst_[i]] = 1;
    uint64_t nodes = 0;
    for (uint8_t u : used) nodes += u;
    graph_info_.nodes = (int)nodes;
    graph_info_.edges = (int)m;
    std::cout << "Graph Info: nodes = " << graph_info_.nodes << ", edges = " << graph_info_.edges
              << std::endl;
}

void Graph::TCPreprocessing() {
    const double t0 = now_ms();
    if (!ctx_) ctx_ = open_ctx(device_);
    if (g_) rtg_graph_destroy(g_);
    check(rtg_graph_from_host_edges(ctx_, src_.data(), dst_.data(), src_.size(), &g_), ctx_,
          "upload edges");
    check(rtg_csr_build(ctx_, g_, RTG_ORIENT_DEGREE_RAW_REF), ctx_, "TC preprocessing");
    rtg_graph_info info;
    check(rtg_graph_info_get(g_, &info), ctx_, "graph info");
    graph_info_.nodes = (int)info.n;
    graph_info_.edges = (int)info.m;
    std::cout << "TC Preprocessing Time = " << now_ms() - t0 << " ms\n";
}

void Graph::ConvertToCSR() {
    const double t0 = now_ms();
    if (!g_) TCPreprocessing();
    rtg_graph_info info;
    check(rtg_graph_info_get(g_, &info), ctx_, "graph info");
    std::vector<uint64_t> off(info.n + 1);
    std::vector<uint32_t> adj(info.m ? info.m : 1);
    check(rtg_csr_to_host(ctx_, g_, 0, off.data(), adj.data()), ctx_, "CSR copy");
    offsets_.assign(off.begin(), off.end());
    adjs_.assign(adj.begin(), adj.begin() + info.m);
    std::cout << "CSR converting time = " << now_ms() - t0 << " ms\n";
}

void Graph::Txt2Bin(const std::string &txt_file, const std::string &bin_file) {
    std::ifstream infile(txt_file);
    if (!infile) {
        std::cerr << "Error opening file: " << txt_file << std::endl;
        std::exit(1);
    }
    std::ofstream outfile(bin_file, std::ios::binary | std::ios::out);
    if (!outfile) {
        std::cerr << "Error opening file: " << bin_file << std::endl;
        std::exit(1);
    }
    std::string line;
    while (std::getline(infile, line)) {
        std::stringstream ss(line);
        int a, b;
        if (ss >> a >> b) {
            outfile.write(reinterpret_cast<const char *>(&a), sizeof(int));
            outfile.write(reinterpret_cast<const char *>(&b), sizeof(int));
        } else {
            std::cerr << "Error parsing line: " << line << std::endl;
        }
    }
    std::cout << "Edge list has been successfully converted to binary." << std::endl;
}

// ----------------------------------------------------------------------- CountOnGPU

void CountOnGPU(int *adjs, int *offsets, int nodes, int edges, int device_id) {
    rtg_ctx *ctx = open_ctx(device_id);
    std::printf("BSTC: using the batched intersection kernel\n");
    uint64_t count = 0;
    rtg_timing t{};
    check(rtg_tc_count_host_csr(ctx, offsets, adjs, nodes, edges, RTG_TC_BATCHED, &count, &t), ctx,
          "count");
    rtg_destroy(ctx);
    std::printf("BSTC: counting time = %f ms, counting result = %llu\n", t.count_ms,
                (unsigned long long)count);
}

// ----------------------------------------------------------------------------- RTTC

RTTC::RTTC(int device_id) : device_(device_id) {
    std::printf("RTTC: Using the batched intersection kernel (no ray tracing)\n");
    ctx_ = open_ctx(device_id);
}

RTTC::~RTTC() {
    if (g_) rtg_graph_destroy(g_);
    if (ctx_) rtg_destroy(ctx_);
}

void RTTC::BuildBVHAndComputeRay(const int *adjs, const int *offsets,
                                 const graph_info_t &graph_info, bool /*if_compact*/) {
    const double t0 = now_ms();
    if (g_) rtg_graph_destroy(g_);
    check(rtg_graph_from_host_csr(ctx_, offsets, adjs, graph_info.nodes, graph_info.edges, &g_),
          ctx_, "CSR upload");
    bvh_memory_size_ = rtg_graph_device_bytes(g_);
    bvh_building_time_ = now_ms() - t0;
    convert_time_ = bvh_building_time_;
    std::cout << "RTTC: time of converting graph to RT = " << convert_time_ << " ms\n";
}

void RTTC::CountTriangles() {
    if (!g_) {
        std::printf("RTTC: BuildBVHAndComputeRay must run first\n");
        std::exit(2);
    }
    uint64_t total = 0;
    rtg_timing t{};
    check(rtg_tc_count(ctx_, g_, RTG_TC_BATCHED, &total, &t), ctx_, "count");
    total_triangles_ = total;
    counting_time_ = t.count_ms;
    count_size_ = 1;
    std::cout << "RTTC: Trace time = " << counting_time_ << " ms\n";
}
