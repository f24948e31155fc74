// Host-side mirror of RT-Graph's public interface for the set-intersection path, implemented
// over librtg's C ABI (include/rtg.h). Same names, argument meanings and console lines as
// the reference, so its drivers and scripts work unchanged; counts are uint64 where the
// reference used uint32. Errors print a message and exit(2), as the reference's CUDA_CHECK
// does (tc/utils/common.h:13-32).
//
//   Graph                      tc/graph/include/graph.h:8-30
//   CountOnGPU                 tc/bs_tc/bs_tc.h:5
//   RTTC                       tc/rt_tc/include/rt_tc.h:7-59
//   Tile, Dataset, Baseline,
//   ReadData/PrintDataInfo/Check   set_intersection/utils/util.h:11-36
//   XxxBasedIntersection       set_intersection/baseline/{bs,hi,ip,bi_naive,bi_dynamic}.cu
//   RTInter                    set_intersection/rt/include/rt_intersection.h:7-29
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "rtg.h"

using uint = unsigned int;

// tc/utils/model.h:10-29
typedef struct GraphInfo {
    int nodes;
    int edges;
} graph_info_t;

typedef struct edge {
    int src;
    int dst;
    bool operator<(const edge &x) const {
        return src == x.src ? dst < x.dst : src < x.src;
    }
} edge_t;

// ------------------------------------------------------------- triangle counting

class Graph {
public:
    explicit Graph(int device_id);
    Graph();
    ~Graph();
    Graph(const Graph &) = delete;
    Graph &operator=(const Graph &) = delete;

    void ReadBinaryEdges(std::string &input_file_path);
    void ConvertToCSR();
    void TCPreprocessing();
    static void Txt2Bin(const std::string &txt_file, const std::string &bin_file);

    std::vector<int> adjs_;
    std::vector<int> offsets_;
    graph_info_t graph_info_{0, 0};

private:
    int device_ = 0;
    std::vector<uint32_t> src_, dst_;
    rtg_ctx *ctx_ = nullptr;
    rtg_graph *g_ = nullptr;
};

void CountOnGPU(int *adjs, int *offsets, int nodes, int edges, int device_id = 0);

class RTTC {
public:
    explicit RTTC(int device_id = 0);
    ~RTTC();
    RTTC(const RTTC &) = delete;
    RTTC &operator=(const RTTC &) = delete;
    void BuildBVHAndComputeRay(const int *adjs, const int *offsets,
                               const graph_info_t &graph_info, bool if_compact = false);
    void CountTriangles();

    uint count_size_{0};
    double convert_time_{0.0};
    double counting_time_{0.0};
    unsigned long long total_triangles_{0};
    // the counting structures resident on the GPU stand where the reference kept its BVH
    size_t bvh_memory_size_{0};
    double bvh_building_time_{0.0};

private:
    int device_ = 0;
    rtg_ctx *ctx_ = nullptr;
    rtg_graph *g_ = nullptr;
};

// ------------------------------------------------------------- set intersection

struct Tile {
    uint start;
    uint end;
    uint size;
};
using tile_t = Tile;

struct Dataset {
    uint num_of_sets_a;
    uint num_of_sets_b;
    uint num_of_sets;
    uint max_element;
    uint intersection;
    std::vector<uint> set_offsets;
    std::vector<uint> elements;
};

enum Baseline { BinarySearch = 0, Hash = 1, Bitmap = 2, IntersectPath = 3 };

void ReadData(const std::string &path, Dataset &dataset);
void PrintDataInfo(const Dataset &dataset);
void Check(const Dataset &dataset, const std::vector<uint> &results);

// Every A x B pair count, row-major by A (set_intersection/baseline/bs.cu:93-96,148). The
// block / thread / bucket arguments of the reference's launch shapes are accepted and
// ignored: the GB300 kernels size their own grids.
void BinarySearchBasedIntersection(const Dataset &dataset, uint blocks, uint block_size,
                                   std::vector<uint> &results);
void HashBasedIntersection(const Dataset &dataset, uint blocks, uint block_size, uint buckets,
                           uint max_bucket_size, std::vector<uint> &results);
void IntersectPathBasedIntersection(const Dataset &dataset, uint blocks, uint block_size,
                                    std::vector<uint> &results);
void BitmapNaiveBasedIntersection(const Dataset &dataset, uint blocks, uint block_size,
                                  std::vector<uint> &results);
void BitmapDynamicBasedIntersection(const Dataset &dataset, uint blocks, uint block_size,
                                    std::vector<uint> &results);

class RTInter {
public:
    RTInter(uint chunk_length, int device_id = 0);
    ~RTInter();
    RTInter(const RTInter &) = delete;
    RTInter &operator=(const RTInter &) = delete;
    void BuildBVHAndComputeRay(Dataset dataset);
    void CountIntersection(std::vector<uint> &results);

private:
    uint chunk_length_{0};
    int device_ = 0;
    rtg_ctx *ctx_ = nullptr;
    rtg_sets *sets_ = nullptr;
    uint num_a_ = 0, num_b_ = 0;
    double build_time_ = 0.0, count_time_ = 0.0;
};
