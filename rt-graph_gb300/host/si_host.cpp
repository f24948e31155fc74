// Set-intersection side of the reference interface over librtg: the dataset file reader and
// checker, the five per-baseline entry points (each mapped to the librtg kernel family of
// the same idea) and RTInter (mapped to the batched form).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>

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

// the reference's drivers select the GPU with cudaSetDevice before calling these functions
int current_device() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess) d = 0;
    return d;
}

// A x B counts (row-major by A) with one kernel family; returns the kernel time in ms.
double dense_counts(const Dataset &ds, uint32_t family, int device, std::vector<uint> &results) {
    rtg_ctx *ctx = nullptr;
    check(rtg_init(device, &ctx), nullptr, "rtg_init");
    rtg_sets *sets = nullptr;
    check(rtg_sets_from_host_u32(ctx, ds.set_offsets.data(), ds.num_of_sets, ds.elements.data(),
                                 &sets),
          ctx, "dataset upload");
    const uint64_t combinations = (uint64_t)ds.num_of_sets_a * ds.num_of_sets_b;
    std::cout << "combinations = " << combinations << std::endl;
    results.assign(combinations, 0u);
    rtg_timing t{};
    check(rtg_si_count_dense(ctx, sets, 0, ds.num_of_sets_a, ds.num_of_sets_a, ds.num_of_sets,
                             results.data(), family, &t),
          ctx, "set intersection");
    rtg_sets_destroy(sets);
    rtg_destroy(ctx);
    return t.count_ms;
}

}  // namespace

void ReadData(const std::string &path, Dataset &dataset) {
    rtg_dataset_info info{};
    check(rtg_dataset_read(path.c_str(), &info, nullptr, nullptr), nullptr, "read dataset");
    dataset.num_of_sets_a = info.num_a;
    dataset.num_of_sets_b = info.num_b;
    dataset.num_of_sets = info.num_a + info.num_b;
    dataset.max_element = info.max_element;
    dataset.intersection = info.intersection;
    dataset.set_offsets.resize(dataset.num_of_sets + 1);
    dataset.elements.resize(info.elems ? info.elems : 1);
    check(rtg_dataset_read(path.c_str(), &info, dataset.set_offsets.data(), dataset.elements.data()),
          nullptr, "read dataset");
    dataset.elements.resize(info.elems);
}

void PrintDataInfo(const Dataset &dataset) {
    std::cout << "Dataset: number of sets = (" << dataset.num_of_sets_a << ", "
              << dataset.num_of_sets_b << ")" << std::endl;
    std::cout << "Dataset: length of set a = " << dataset.set_offsets[1] - dataset.set_offsets[0];
    std::cout << ", length of set b = "
              << dataset.set_offsets[dataset.num_of_sets] -
                     dataset.set_offsets[dataset.num_of_sets - 1]
              << std::endl;
    std::cout << "Dataset: intersection size = " << dataset.intersection << std::endl;
}

void Check(const Dataset &dataset, const std::vector<uint> &results) {
    for (size_t i = 0; i < results.size(); ++i) {
        if (results[i] != dataset.intersection) {
            std::cout << "Check: " << i << "-th result (" << results[i]
                      << " != " << dataset.intersection << ") is incorrect" << std::endl;
            return;
        }
    }
    std::cout << "Check: accepted" << std::endl;
}

void BinarySearchBasedIntersection(const Dataset &dataset, uint blocks, uint block_size,
                                   std::vector<uint> &results) {
    std::cout << "blocks = " << blocks << ", block size = " << block_size << std::endl;
    const double ms = dense_counts(dataset, RTG_SI_FORCE_SEARCH, current_device(), results);
    std::cout << "Binary Search based Set Intertsection: kernel time = " << ms << " ms\n";
}

void HashBasedIntersection(const Dataset &dataset, uint blocks, uint block_size, uint buckets,
                           uint max_bucket_size, std::vector<uint> &results) {
    std::cout << "blocks = " << blocks << ", block size = " << block_size << std::endl;
    (void)buckets;
    (void)max_bucket_size;
    const double ms = dense_counts(dataset, RTG_SI_FORCE_BITMAP, current_device(), results);
    std::cout << "Hash based Set Intertsection: kernel time = " << ms << " ms\n";
}

void IntersectPathBasedIntersection(const Dataset &dataset, uint blocks, uint block_size,
                                    std::vector<uint> &results) {
    std::cout << "blocks = " << blocks << ", block size = " << block_size << std::endl;
    const double ms = dense_counts(dataset, RTG_SI_FORCE_MERGE, current_device(), results);
    std::cout << "Intersect Path based Set Intertsection: kernel time = " << ms << " ms\n";
}

void BitmapNaiveBasedIntersection(const Dataset &dataset, uint blocks, uint block_size,
                                  std::vector<uint> &results) {
    std::cout << "blocks = " << blocks << ", block size = " << block_size << std::endl;
    const double ms = dense_counts(dataset, RTG_SI_FORCE_BITMAP, current_device(), results);
    std::cout << "Bitmap(naive) based Set Intertsection:\nconstruction time = 0 ms";
    std::cout << ", counting time = " << ms << " ms ";
    std::cout << ", kernel time = " << ms << " ms\n";
}

void BitmapDynamicBasedIntersection(const Dataset &dataset, uint blocks, uint block_size,
                                    std::vector<uint> &results) {
    std::cout << "blocks = " << blocks << ", block size = " << block_size << std::endl;
    const double ms = dense_counts(dataset, RTG_SI_FORCE_BITMAP, current_device(), results);
    std::cout << "Bitmap(dynamic) based Set Intertsection: kernel time = " << ms << " ms\n";
}

// --------------------------------------------------------------------------- RTInter

RTInter::RTInter(uint chunk_length, int device_id) : chunk_length_(chunk_length), device_(device_id) {
    check(rtg_init(device_, &ctx_), nullptr, "rtg_init");
}

RTInter::~RTInter() {
    std::cout << "RT based Set Intersection:\n";
    std::cout << "BVH memory size = 0 GB\n";
    std::cout << "BVH building time = " << build_time_ << " ms, BVH compaction time = 0 ms,";
    std::cout << " RT counting time = " << count_time_ << " ms\n";
    std::cout << "RT total time = " << build_time_ + count_time_ << " ms\n";
    if (sets_) rtg_sets_destroy(sets_);
    if (ctx_) rtg_destroy(ctx_);
}

void RTInter::BuildBVHAndComputeRay(Dataset dataset) {
    const double t0 = now_ms();
    num_a_ = dataset.num_of_sets_a;
    num_b_ = dataset.num_of_sets_b;
    std::cout << "combinations = " << (uint64_t)num_a_ * num_b_ << std::endl;
    if (sets_) rtg_sets_destroy(sets_);
    check(rtg_sets_from_host_u32(ctx_, dataset.set_offsets.data(), dataset.num_of_sets,
                                 dataset.elements.data(), &sets_),
          ctx_, "dataset upload");
    build_time_ = now_ms() - t0;
}

void RTInter::CountIntersection(std::vector<uint> &results) {
    if (!sets_) {
        std::printf("RTInter: BuildBVHAndComputeRay must run first\n");
        std::exit(2);
    }
    results.assign((uint64_t)num_a_ * num_b_, 0u);
    rtg_timing t{};
    check(rtg_si_count_dense(ctx_, sets_, 0, num_a_, num_a_, num_a_ + num_b_, results.data(),
                             RTG_SI_AUTO, &t),
          ctx_, "set intersection");
    count_time_ = t.count_ms;
}
