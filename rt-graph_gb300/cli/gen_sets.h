// The part the two dataset generators share (s_generator, m_generator): one A set of
// distinct values and num_b B sets that each hold the first |C| elements of A plus distinct
// values outside A, drawn in the order the reference's set_intersection/data_generator
// draws them (data.cpp:21-342: all of A first, then each B set in turn, a value already taken
// drawn again), and the .s_data / .m_data file layout (data.cpp:344-373): header
// {num_a, num_b, range, |C|}, num_a + num_b + 1 uint32 offsets, A num_a times, then the B sets.
#pragma once

#include <algorithm>
#include <cstdint>
#include <fstream>
#include <string>
#include <unordered_set>
#include <vector>

template <class DrawA, class DrawB>
void build_sets(uint32_t len_a, uint32_t len_b, uint32_t len_c, uint32_t num_b, DrawA draw_a,
                DrawB draw_b, std::vector<uint32_t> &a, std::vector<std::vector<uint32_t>> &bs) {
    a.assign(len_a, 0);
    std::unordered_set<uint32_t> in_a;
    for (uint32_t i = 0; i < len_a; ++i) {
        uint32_t x;
        do x = draw_a();
        while (in_a.count(x));
        in_a.insert(x);
        a[i] = x;
    }
    std::sort(a.begin(), a.end());
    bs.assign(num_b, std::vector<uint32_t>(len_b));
    for (auto &b : bs) {
        std::copy(a.begin(), a.begin() + len_c, b.begin());
        std::unordered_set<uint32_t> used = in_a;
        for (uint32_t j = len_c; j < len_b; ++j) {
            uint32_t x;
            do x = draw_b();
            while (used.count(x));
            used.insert(x);
            b[j] = x;
        }
        std::sort(b.begin(), b.end());
    }
}

// false when the file cannot be opened
inline bool write_sets_file(const std::string &path, uint32_t num_a, uint32_t range,
                            uint32_t len_c, const std::vector<uint32_t> &a,
                            const std::vector<std::vector<uint32_t>> &bs) {
    std::ofstream f(path, std::ios::binary);
    if (!f) return false;
    const uint32_t num_b = (uint32_t)bs.size();
    const uint32_t len_a = (uint32_t)a.size(), len_b = num_b ? (uint32_t)bs[0].size() : 0u;
    const uint32_t header[4] = {num_a, num_b, range, len_c};
    f.write(reinterpret_cast<const char *>(header), sizeof header);
    uint32_t off = 0;
    for (uint32_t i = 0; i < num_a + num_b; ++i) {
        f.write(reinterpret_cast<const char *>(&off), 4);
        off += (i < num_a) ? len_a : len_b;
    }
    f.write(reinterpret_cast<const char *>(&off), 4);
    for (uint32_t i = 0; i < num_a; ++i) f.write(reinterpret_cast<const char *>(a.data()), 4ull * len_a);
    for (auto &b : bs) f.write(reinterpret_cast<const char *>(b.data()), 4ull * len_b);
    return true;
}
