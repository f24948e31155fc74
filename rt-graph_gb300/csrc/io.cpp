// File formats: the reference's binary edge list (int32 pairs, tc/graph/graph.cpp:23-38),
// text edge lists (graph.cpp:179-214), MatrixMarket coordinate files with the BFS loader's
// rules (1-based, zero index rejected, symmetric files expanded; bfs/graph/graph.cpp:17-117)
// and the set-intersection dataset files (.s_data/.m_data: u32 num_a, num_b, max_element,
// intersection, u32 offsets[num_a+num_b+1], u32 elements[];
// set_intersection/utils/util.cpp:3-23, data_generator/data.cpp:344-373).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "rtg.h"

namespace {

rtg_status read_edge_bin(const char *path, std::vector<uint32_t> &s, std::vector<uint32_t> &d) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return RTG_ERR_IO;
    std::fseek(f, 0, SEEK_END);
    long long bytes = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (bytes < 0 || bytes % 8) {
        std::fclose(f);
        return RTG_ERR_FORMAT;
    }
    uint64_t m = (uint64_t)bytes / 8;
    std::vector<int32_t> raw(2 * m);
    size_t got = m ? std::fread(raw.data(), 8, m, f) : 0;
    std::fclose(f);
    if (got != m) return RTG_ERR_IO;
    s.resize(m);
    d.resize(m);
    for (uint64_t i = 0; i < m; ++i) {
        if (raw[2 * i] < 0 || raw[2 * i + 1] < 0) return RTG_ERR_FORMAT;
        s[i] = (uint32_t)raw[2 * i];
        d[i] = (uint32_t)raw[2 * i + 1];
    }
    return RTG_OK;
}

rtg_status read_edge_txt(const char *path, std::vector<uint32_t> &s, std::vector<uint32_t> &d) {
    std::ifstream in(path);
    if (!in) return RTG_ERR_IO;
    std::string line;
    while (std::getline(in, line)) {
        std::stringstream ss(line);
        long long a, b;
        if (!(ss >> a >> b)) continue;  // comment / malformed lines are skipped, as Txt2Bin does
        if (a < 0 || b < 0 || a > 0x7FFFFFFFll || b > 0x7FFFFFFFll) return RTG_ERR_FORMAT;
        s.push_back((uint32_t)a);
        d.push_back((uint32_t)b);
    }
    return RTG_OK;
}

rtg_status read_mtx(const char *path, std::vector<uint32_t> &s, std::vector<uint32_t> &d) {
    std::ifstream in(path);
    if (!in) return RTG_ERR_IO;
    std::string line;
    if (!std::getline(in, line)) return RTG_ERR_FORMAT;
    if (line.rfind("%%MatrixMarket", 0) != 0) return RTG_ERR_FORMAT;
    std::string lower = line;
    for (auto &ch : lower) ch = (char)std::tolower((unsigned char)ch);
    if (lower.find("coordinate") == std::string::npos) return RTG_ERR_FORMAT;
    const bool symmetric = lower.find("symmetric") != std::string::npos;
    long long rows = -1, cols = -1, nnz = -1;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '%') continue;
        std::stringstream ss(line);
        if (!(ss >> rows >> cols >> nnz)) return RTG_ERR_FORMAT;
        break;
    }
    if (nnz < 0) return RTG_ERR_FORMAT;
    s.reserve((size_t)nnz * (symmetric ? 2 : 1));
    d.reserve(s.capacity());
    long long seen = 0;
    while (seen < nnz && std::getline(in, line)) {
        if (line.empty() || line[0] == '%') continue;
        std::stringstream ss(line);
        long long r, c;
        if (!(ss >> r >> c)) return RTG_ERR_FORMAT;
        if (r <= 0 || c <= 0 || r > rows || c > cols) return RTG_ERR_FORMAT;
        s.push_back((uint32_t)(r - 1));
        d.push_back((uint32_t)(c - 1));
        if (symmetric && r != c) {
            s.push_back((uint32_t)(c - 1));
            d.push_back((uint32_t)(r - 1));
        }
        ++seen;
    }
    if (seen != nnz) return RTG_ERR_FORMAT;
    return RTG_OK;
}

}  // namespace

extern "C" {

rtg_status rtg_edges_read(const char *path, rtg_format fmt, uint64_t *m, uint32_t *src,
                          uint32_t *dst) {
    if (!path || !m) return RTG_ERR_INVALID_ARG;
    std::vector<uint32_t> s, d;
    rtg_status st;
    switch (fmt) {
    case RTG_FMT_EDGE_BIN: st = read_edge_bin(path, s, d); break;
    case RTG_FMT_EDGE_TXT: st = read_edge_txt(path, s, d); break;
    case RTG_FMT_MTX: st = read_mtx(path, s, d); break;
    default: return RTG_ERR_INVALID_ARG;
    }
    if (st != RTG_OK) return st;
    if (!src || !dst) {
        *m = s.size();
        return RTG_OK;
    }
    if (*m < s.size()) return RTG_ERR_INVALID_ARG;
    std::memcpy(src, s.data(), s.size() * 4);
    std::memcpy(dst, d.data(), d.size() * 4);
    *m = s.size();
    return RTG_OK;
}

extern "C++" {
namespace rtg {
rtg_status graph_load_cached(rtg_ctx *ctx, const char *path, rtg_graph **out);  // csr_cache.cpp
}
}

rtg_status rtg_graph_load(rtg_ctx *ctx, const char *path, rtg_format fmt, rtg_graph **out) {
    if (!ctx || !path || !out) return RTG_ERR_INVALID_ARG;
    if (fmt == RTG_FMT_RTG_CSR) return rtg::graph_load_cached(ctx, path, out);
    uint64_t m = 0;
    rtg_status st = rtg_edges_read(path, fmt, &m, nullptr, nullptr);
    if (st != RTG_OK) return st;
    std::vector<uint32_t> s(m ? m : 1), d(m ? m : 1);
    st = rtg_edges_read(path, fmt, &m, s.data(), d.data());
    if (st != RTG_OK) return st;
    st = rtg_graph_from_host_edges(ctx, s.data(), d.data(), m, out);
    if (st == RTG_OK) st = rtg_synchronize(ctx);  // host vectors are freed on return
    return st;
}

rtg_status rtg_edges_write_bin(const char *path, const uint32_t *src, const uint32_t *dst,
                               uint64_t m) {
    if (!path || (m && (!src || !dst))) return RTG_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return RTG_ERR_IO;
    std::vector<int32_t> buf;
    const uint64_t chunk = 1 << 20;
    for (uint64_t i = 0; i < m; i += chunk) {
        uint64_t n = (m - i < chunk) ? m - i : chunk;
        buf.resize(2 * n);
        for (uint64_t k = 0; k < n; ++k) {
            if (src[i + k] > 0x7FFFFFFFu || dst[i + k] > 0x7FFFFFFFu) {
                std::fclose(f);
                return RTG_ERR_INVALID_ARG;
            }
            buf[2 * k] = (int32_t)src[i + k];
            buf[2 * k + 1] = (int32_t)dst[i + k];
        }
        if (std::fwrite(buf.data(), 8, n, f) != n) {
            std::fclose(f);
            return RTG_ERR_IO;
        }
    }
    return std::fclose(f) == 0 ? RTG_OK : RTG_ERR_IO;
}

rtg_status rtg_dataset_read(const char *path, rtg_dataset_info *info, uint32_t *offsets,
                            uint32_t *elems) {
    if (!path || !info) return RTG_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "rb");
    if (!f) return RTG_ERR_IO;
    uint32_t hdr[4];
    if (std::fread(hdr, 4, 4, f) != 4) {
        std::fclose(f);
        return RTG_ERR_FORMAT;
    }
    const uint64_t nsets = (uint64_t)hdr[0] + hdr[1];
    std::vector<uint32_t> off(nsets + 1);
    if (std::fread(off.data(), 4, nsets + 1, f) != nsets + 1) {
        std::fclose(f);
        return RTG_ERR_FORMAT;
    }
    for (uint64_t i = 0; i < nsets; ++i)
        if (off[i + 1] < off[i]) {
            std::fclose(f);
            return RTG_ERR_FORMAT;
        }
    info->num_a = hdr[0];
    info->num_b = hdr[1];
    info->max_element = hdr[2];
    info->intersection = hdr[3];
    info->elems = off[nsets];
    if (!offsets || !elems) {
        std::fclose(f);
        return RTG_OK;
    }
    std::memcpy(offsets, off.data(), (nsets + 1) * 4);
    size_t got = info->elems ? std::fread(elems, 4, info->elems, f) : 0;
    std::fclose(f);
    return got == info->elems ? RTG_OK : RTG_ERR_FORMAT;
}

rtg_status rtg_dataset_write(const char *path, const rtg_dataset_info *info,
                             const uint32_t *offsets, const uint32_t *elems) {
    if (!path || !info || !offsets || (info->elems && !elems)) return RTG_ERR_INVALID_ARG;
    const uint64_t nsets = (uint64_t)info->num_a + info->num_b;
    if (offsets[nsets] != info->elems) return RTG_ERR_INVALID_ARG;
    FILE *f = std::fopen(path, "wb");
    if (!f) return RTG_ERR_IO;
    uint32_t hdr[4] = {info->num_a, info->num_b, info->max_element, info->intersection};
    bool ok = std::fwrite(hdr, 4, 4, f) == 4 &&
              std::fwrite(offsets, 4, nsets + 1, f) == nsets + 1 &&
              (info->elems == 0 || std::fwrite(elems, 4, info->elems, f) == info->elems);
    ok = (std::fclose(f) == 0) && ok;
    return ok ? RTG_OK : RTG_ERR_IO;
}

}  // extern "C"
