// m_generator — multi-set dataset generator with the options, value distributions and file
// format of the reference's set_intersection/data_generator (m_generator.cpp:4-41,
// data.cpp:168-342, 344-373):
//   -l/--len -s/--selectivity -n/--num_b (1) -d/--distribution (0 uniform, 1 normal,
//   2 exponential) -b/--lambda (1) -r/--skew_ratio (1) -f/--output_dir ("../../dataset/")
//   -a/--num_a (1000: the reference's fixed number of A sets; an extension for small files)
// |A| = len, |B| = len / skew_ratio, |C| = len * selectivity, values in [0, range] with
// range = min((|A| + |B| - |C|) / 0.01, RAND_MAX). One A set of distinct values copied
// num_a times; every B set holds the first |C| elements of A plus distinct values outside A,
// so every A x B pair intersects in exactly |C| elements. All draws come from one
// default-seeded std::default_random_engine in this order: A, then each B set; a value that
// is already taken (or, for the normal and exponential shapes, above the range) is drawn
// again. The normal shape is N(range / 2, range / 50) rounded; the exponential shape is
// range * Exp(lambda) rounded, whose B draws are taken from Exp(lambda) values below 1.
// Output: <|A|>_<|B|>_<|C|>_<num_b>_<range> + "_uni.m_data" / "_nor.m_data" /
// "_<int lambda>_exp.m_data" in output_dir, in the .s_data layout.
#include <sys/stat.h>

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
    static const char *alias[][2] = {{"-l", "--len"},        {"-s", "--selectivity"},
                                     {"-n", "--num_b"},      {"-d", "--distribution"},
                                     {"-b", "--lambda"},     {"-r", "--skew_ratio"},
                                     {"-f", "--output_dir"}, {"-a", "--num_a"}};
    store.assign(argv, argv + argc);
    for (auto &s : store)
        for (auto &al : alias)
            if (s == al[0]) s = al[1];
    std::vector<char *> out;
    for (auto &s : store) out.push_back(&s[0]);
    return out;
}

enum Shape { kUniform = 0, kNormal = 1, kExponential = 2 };

}  // namespace

int main(int argc, char *argv[]) {
    std::vector<std::string> store;
    std::vector<char *> av = long_options(argc, argv, store);
    Args args((int)av.size(), av.data());
    if (args.help()) {
        std::cout << "m_generator -l len -s selectivity [-n num_b] [-d distribution] "
                     "[-b lambda] [-r skew_ratio] [-f output_dir] [-a num_a]"
                  << std::endl;
        return 0;
    }
    const uint32_t len = (uint32_t)args.u("len");
    const double selectivity = args.d("selectivity");
    const uint32_t num_b = (uint32_t)args.u("num_b", "1");
    const unsigned shape_arg = (unsigned)args.u("distribution", "0");
    const double lambda = args.d("lambda", "1");
    const double skew = args.d("skew_ratio", "1");
    const std::string dir = args.str("output_dir", "../../dataset/");
    const uint32_t num_a = (uint32_t)args.u("num_a", "1000");
    if (selectivity < 0 || selectivity > 1 || skew <= 0 || num_b < 1) {
        std::cerr << "invalid selectivity, skew ratio or number of B sets" << std::endl;
        return 1;
    }
    const Shape shape = shape_arg == 1 ? kNormal : (shape_arg == 2 ? kExponential : kUniform);
    const uint32_t len_a = len;
    const uint32_t len_b = (uint32_t)(len / skew);
    const uint32_t len_c = (uint32_t)(len * selectivity);
    if (len_c > len_a || len_c > len_b) {
        std::cerr << "selectivity too large for the set lengths" << std::endl;
        return 1;
    }
    const double density = 0.01;
    const uint32_t range =
        std::min((uint32_t)((len_a + len_b - len_c) / density), (uint32_t)RAND_MAX);

    std::default_random_engine engine;
    std::uniform_int_distribution<uint32_t> uni(0u, range);
    std::normal_distribution<double> nor(1.0 * range / 2, 1.0 * range / 50);
    std::exponential_distribution<double> expo(lambda);
    auto draw = [&](bool for_b) -> uint32_t {
        if (shape == kUniform) return uni(engine);
        if (shape == kNormal) {
            double y;
            do y = std::round(nor(engine));
            while (y < 0 || y > range);
            return (uint32_t)y;
        }
        if (for_b) {
            double v;
            do v = expo(engine);
            while (v >= 1.0);
            return (uint32_t)std::round(range * v);
        }
        double y;
        do y = std::round(range * expo(engine));
        while (y > range);
        return (uint32_t)y;
    };

    std::vector<uint32_t> a;
    std::vector<std::vector<uint32_t>> bs;
    build_sets(len_a, len_b, len_c, num_b, [&]() { return draw(false); }, [&]() { return draw(true); },
               a, bs);

    const std::string suffix = shape == kNormal      ? "_nor.m_data"
                               : shape == kExponential ? "_" + std::to_string((int)lambda) + "_exp.m_data"
                                                       : "_uni.m_data";
    const std::string name = std::to_string(len_a) + "_" + std::to_string(len_b) + "_" +
                             std::to_string(len_c) + "_" + std::to_string(num_b) + "_" +
                             std::to_string(range) + suffix;
    std::cout << "Data: length of set A = " << len_a << ", length of set B = " << len_b
              << ", length of set C = " << len_c << ", number of set B = " << num_b
              << ", element range = " << range << std::endl;
    struct stat st;
    if (stat(dir.c_str(), &st) != 0) {
        std::cerr << "directory (" << dir << ") does not exist" << std::endl;
        return 1;
    }
    const std::string path = dir + name;
    if (!write_sets_file(path, num_a, range, len_c, a, bs)) {
        std::cerr << "File error" << std::endl;
        return 1;
    }
    std::cout << "Data has been written to path: " << path << std::endl;
    return 0;
}
