// bs | hi | ip | bi_naive | bi_dynamic | rt_intersection — drop-ins for the reference's
// set-intersection baselines (set_intersection/baseline/*.cu, set_intersection/rt/main.cpp).
// The tool is chosen by the program name; options keep the reference's names and defaults:
//   --device --dataset [--threads] [--buckets --bucket_size] [--blocks] [--chunk_length]
// Each tool reads a .s_data/.m_data file, counts every A x B pair on the GPU, prints the
// reference's kernel-time line and "Check: accepted" when every count equals the file's
// known intersection size.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <iostream>
#include <string>

#include "args.h"
#include "rtg_reference.h"

int main(int argc, char *argv[]) {
    std::string tool = argv[0];
    const auto slash = tool.find_last_of('/');
    if (slash != std::string::npos) tool = tool.substr(slash + 1);
    Args args(argc, argv);
    if (args.help()) {
        std::cout << tool << " --device <id> --dataset <path> [--threads 512] [--buckets n "
                             "--bucket_size n] [--blocks n] [--chunk_length n]"
                  << std::endl;
        return 0;
    }
    const unsigned device_id = (unsigned)args.u("device", "0");
    const std::string path = args.str("dataset");
    const unsigned block_size = std::min<unsigned>((unsigned)args.u("threads", "512"), 1024u);
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || (int)device_id >= count) {
        std::cerr << "Device id (" << device_id << ") is larger than device count (" << count
                  << ")" << std::endl;
        return 1;
    }
    cudaSetDevice((int)device_id);

    Dataset dataset;
    ReadData(path, dataset);
    PrintDataInfo(dataset);
    std::vector<uint> results;
    const unsigned blocks = std::min(dataset.num_of_sets_a, 65535u);
    if (tool == "bs") {
        BinarySearchBasedIntersection(dataset, blocks, block_size, results);
    } else if (tool == "hi") {
        HashBasedIntersection(dataset, blocks, block_size, (unsigned)args.u("buckets", "12000"),
                              (unsigned)args.u("bucket_size", "100"), results);
    } else if (tool == "ip") {
        IntersectPathBasedIntersection(dataset, blocks, block_size, results);
    } else if (tool == "bi_naive") {
        BitmapNaiveBasedIntersection(dataset, blocks, block_size, results);
    } else if (tool == "bi_dynamic") {
        unsigned b = (unsigned)args.u("blocks", "0");
        BitmapDynamicBasedIntersection(dataset, b ? b : blocks, block_size, results);
    } else if (tool == "rt_intersection") {
        RTInter rt_inter((unsigned)args.u("chunk_length", "1024"), (int)device_id);
        rt_inter.BuildBVHAndComputeRay(dataset);
        rt_inter.CountIntersection(results);
    } else {
        std::cerr << "unknown tool name " << tool << std::endl;
        return 1;
    }
    Check(dataset, results);
    return 0;
}
