// s_generator — set-intersection dataset generator with the options, algorithm and file
// format of the reference's set_intersection/data_generator (s_generator.cpp:4-46,
// data.cpp:21-166, 344-373):
//   -a/--num_a (1000) -l/--len -r/--skew_ratio -s/--selectivity -d/--density (0.1)
//   -b/--lambda (0: uniform values; > 0: exponential values) -n/--num_b (1)
//   -f/--output_dir ("../dataset/")
// |A| = len, |B| = len / skew_ratio, |C| = len * selectivity. One A set of distinct values,
// copied num_a times; every B set holds the first |C| elements of A plus values drawn outside
// A, so every A x B pair intersects in exactly |C| elements (the file header records |C|).
// Uniform values come from the C library's rand() stream (as in the reference), exponential
// values from std::default_random_engine with std::exponential_distribution.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <random>
#include <string>
#include <unordered_set>
#include <vector>

#include "args.h"
#include "gen_sets.h"

namespace {

std::vector<char *> long_options(int argc, char **argv, std::vector<std::string> &store) {
    static const char *alias[][2] = {{"-a", "--num_a"},      {"-l", "--len"},
                                     {"-r", "--skew_ratio"}, {"-s", "--selectivity"},
                                     {"-d", "--density"},    {"-b", "--lambda"},
                                     {"-n", "--num_b"},      {"-f", "--output_dir"}};
    store.assign(argv, argv + argc);
    for (auto &s : store)
        for (auto &al : alias)
            if (s == al[0]) s = al[1];
    std::vector<char *> out;
    for (auto &s : store) out.push_back(&s[0]);
    return out;
}

}  // namespace

int main(int argc, char *argv[]) {
    std::vector<std::string> store;
    std::vector<char *> av = long_options(argc, argv, store);
    Args args((int)av.size(), av.data());
    if (args.help()) {
        std::cout << "s_generator -l len -r skew_ratio -s selectivity [-d density] [-b lambda] "
                     "[-a num_a] [-n num_b] [-f output_dir]"
                  << std::endl;
        return 0;
    }
    const uint32_t len = (uint32_t)args.u("len");
    const double skew = args.d("skew_ratio");
    const double selectivity = args.d("selectivity");
    const double density = args.d("density", "0.1");
    const double lambda = args.d("lambda", "0");
    const uint32_t num_a = (uint32_t)args.u("num_a", "1000");
    const uint32_t num_b = (uint32_t)args.u("num_b", "1");
    const std::string dir = args.str("output_dir", "../dataset/");
    if (selectivity < 0 || selectivity > 1 || skew <= 0 || density <= 0) {
        std::cerr << "invalid skew ratio, selectivity or density" << std::endl;
        return 1;
    }
    const uint32_t len_a = len;
    const uint32_t len_b = (uint32_t)(len / skew);
    const uint32_t len_c = (uint32_t)(len * selectivity);
    if (len_c > len_a || len_c > len_b) {
        std::cerr << "selectivity too large for the set lengths" << std::endl;
        return 1;
    }
    const uint32_t range = std::min((uint32_t)((len_a + len_b - len_c) / density), (uint32_t)RAND_MAX);
    if ((uint64_t)len_a + len_b - len_c > range) {
        std::cerr << "value range too small for distinct elements" << std::endl;
        return 1;
    }

    std::default_random_engine engine;
    std::exponential_distribution<double> expo(lambda > 0 ? lambda : 1.0);
    auto draw_a = [&]() -> uint32_t {
        if (lambda <= 0) return (uint32_t)(std::rand() % range);
        uint32_t x;
        do x = (uint32_t)std::round(range * expo(engine));
        while (x > range);
        return x;
    };
    auto draw_b = [&]() -> uint32_t {
        if (lambda <= 0) return (uint32_t)(std::rand() % range);
        double v;
        do v = expo(engine);
        while (v >= 1.0);
        return (uint32_t)std::round(range * v);
    };

    std::vector<uint32_t> a;
    std::vector<std::vector<uint32_t>> bs;
    build_sets(len_a, len_b, len_c, num_b, draw_a, draw_b, a, bs);

    std::string name;
    if (lambda > 0)
        name = std::to_string(lambda) + "_" + std::to_string(len_a) + "_" + std::to_string(len_b) +
               "_" + std::to_string(len_c) + "_" + std::to_string(range) + ".exponential";
    else
        name = std::to_string(len_a) + "_" + std::to_string(len_b) + "_" + std::to_string(len_c) +
               "_" + std::to_string(range) + ".s_data";
    const std::string path = dir + name;
    if (!write_sets_file(path, num_a, range, len_c, a, bs)) {
        std::cerr << "File error" << std::endl;
        return 1;
    }
    std::cout << "Data: length of set A = " << len_a << ", length of set B = " << len_b
              << ", length of set C = " << len_c << ", element range = " << range << std::endl;
    std::cout << "Data has been written to path: " << path << std::endl;
    return 0;
}
