// File formats: the reference's binary edge list (int32 pairs, tc/graph/graph.cpp:23-38),
// text edge lists (graph.cpp:179-214), MatrixMarket coordinate files with the BFS loader's
// rules (1-based, zero index rejected, symmetric files expanded; bfs/graph/graph.cpp:17-117)
// and the set-intersection dataset files (.s_data/.m_data: u32 num_a, num_b, max_element,
// intersection, u32 offsets[num_a+num_b+1], u32 elements[];
// set_intersection/utils/util.cpp:3-23, data_generator/data.cpp:344-373).
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <omp.h>

#include "host_guard.h"
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

// Text formats are read whole (one fread) and scanned line by line with the semantics of
// `std::istringstream(line) >> long long` that the reference's loaders use (getline, then
// extraction): leading blanks skipped, an optional sign, at least one digit, digits until
// the first other character; a value past the range of long long fails the extraction.
// Scanning the buffer instead of building a string stream per line is about 20x faster
// (8.4 M R-MAT edges: 105 MB in 4.4 s before).
bool read_file(const char *path, std::vector<char> &buf) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::vector<char> out;
    long long size = -1;
    if (std::fseek(f, 0, SEEK_END) == 0) {
        size = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
    }
    if (size > 0) out.reserve((size_t)size);
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) out.insert(out.end(), chunk, chunk + got);
    const bool ok = !std::ferror(f);
    std::fclose(f);
    buf.swap(out);
    return ok;
}

inline bool blank(char c) { return c == ' ' || c == '\t' || c == '\v' || c == '\f' || c == '\r'; }

// One `>> long long` on [p, e): false where the stream would fail.
inline bool read_ll(const char *&p, const char *e, long long &v) {
    while (p < e && blank(*p)) ++p;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) {
        neg = *p == '-';
        ++p;
    }
    if (p >= e || *p < '0' || *p > '9') return false;
    const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
    unsigned long long x = 0;
    bool over = false;
    for (; p < e && *p >= '0' && *p <= '9'; ++p) {
        const unsigned dgt = (unsigned)(*p - '0');
        if (x > (lim - dgt) / 10) over = true;
        else x = x * 10 + dgt;
    }
    if (over) return false;
    v = neg ? (long long)(0ull - x) : (long long)x;
    return true;
}

// Calls f(line_begin, line_end) for every line of the buffer (a last line without a
// newline included, as getline gives it); f returns false to stop.
template <class F>
void for_lines(const std::vector<char> &buf, F f) {
    const char *p = buf.data(), *e = p + buf.size();
    while (p < e) {
        const char *nl = static_cast<const char *>(std::memchr(p, '\n', (size_t)(e - p)));
        const char *le = nl ? nl : e;
        if (!f(p, le)) return;
        p = nl ? nl + 1 : e;
    }
}

// Lines [b, e) of a text edge list into s/d; FORMAT on an id outside [0, 2^31).
rtg_status parse_txt_lines(const char *b, const char *e, std::vector<uint32_t> &s,
                           std::vector<uint32_t> &d) {
    rtg_status st = RTG_OK;
    while (b < e) {
        // a number never spans a newline (it is not a blank), so the two extractions read
        // the buffer directly and stop inside the line; then the rest of the line is skipped
        const char *p = b;
        long long x, y;
        // comment / malformed lines are skipped, as Txt2Bin does
        if (read_ll(p, e, x) && read_ll(p, e, y)) {
            if (x < 0 || y < 0 || x > 0x7FFFFFFFll || y > 0x7FFFFFFFll) {
                st = RTG_ERR_FORMAT;
                break;
            }
            s.push_back((uint32_t)x);
            d.push_back((uint32_t)y);
        }
        const char *nl = p < e && *p == '\n'
                             ? p
                             : static_cast<const char *>(std::memchr(p, '\n', (size_t)(e - p)));
        b = nl ? nl + 1 : e;
    }
    return st;
}

// Parsed in parallel: the buffer is cut after a newline into one piece per thread, each
// piece parsed on its own, the pieces joined in order.
rtg_status read_edge_txt(const char *path, std::vector<uint32_t> &s, std::vector<uint32_t> &d) {
    std::vector<char> buf;
    if (!read_file(path, buf)) return RTG_ERR_IO;
    const char *base = buf.data();
    const size_t n = buf.size();
    const int T = (int)std::max<size_t>(1, std::min<size_t>((size_t)omp_get_max_threads(),
                                                            n / (1u << 20) + 1));
    std::vector<size_t> cut(T + 1, n);
    cut[0] = 0;
    for (int t = 1; t < T; ++t) {
        size_t at = std::max(cut[t - 1], n / T * t);
        const char *nl = at < n ? static_cast<const char *>(std::memchr(base + at, '\n', n - at))
                                : nullptr;
        cut[t] = nl ? (size_t)(nl - base) + 1 : n;
    }
    std::vector<std::vector<uint32_t>> ps(T), pd(T);
    std::vector<rtg_status> st(T, RTG_OK);
#pragma omp parallel for num_threads(T) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
        const size_t len = cut[t + 1] - cut[t];
        // a failed allocation inside the parallel region stays in its piece
        try {
            ps[t].reserve(len / 4 + 1);
            pd[t].reserve(len / 4 + 1);
            st[t] = parse_txt_lines(base + cut[t], base + cut[t + 1], ps[t], pd[t]);
        } catch (...) {
            st[t] = RTG_ERR_OOM;
        }
    }
    size_t total = 0;
    for (int t = 0; t < T; ++t) {
        if (st[t] != RTG_OK) return st[t];
        total += ps[t].size();
    }
    s.resize(total);
    d.resize(total);
    size_t at = 0;
    for (int t = 0; t < T; ++t) {
        std::copy(ps[t].begin(), ps[t].end(), s.begin() + at);
        std::copy(pd[t].begin(), pd[t].end(), d.begin() + at);
        at += ps[t].size();
    }
    return RTG_OK;
}

// Entry lines [b, e) of a MatrixMarket body: (row, col) pairs, 1-based and checked against
// the size line, into er/ec; empty and comment lines skipped. Stops at the first line that
// is not an entry in range and returns its rank among the entries (er.size()), else -1.
long long parse_mtx_entries(const char *b, const char *e, long long rows, long long cols,
                            std::vector<uint32_t> &er, std::vector<uint32_t> &ec) {
    while (b < e) {
        const char *nl = static_cast<const char *>(std::memchr(b, '\n', (size_t)(e - b)));
        const char *le = nl ? nl : e;
        if (le != b && *b != '%') {
            const char *p = b;
            long long r, c;
            if (!read_ll(p, le, r) || !read_ll(p, le, c) || r <= 0 || c <= 0 || r > rows ||
                c > cols)
                return (long long)er.size();
            er.push_back((uint32_t)r);
            ec.push_back((uint32_t)c);
        }
        b = nl ? nl + 1 : e;
    }
    return -1;
}

// Header and size line in order, then the entry lines in parallel pieces (cut after a
// newline, one per thread); the pieces are joined in order up to nnz entries, a bad line
// among those is a format error, lines after them are not read, and symmetric files get the
// mirrored entry after each off-diagonal one.
rtg_status read_mtx(const char *path, std::vector<uint32_t> &s, std::vector<uint32_t> &d) {
    std::vector<char> buf;
    if (!read_file(path, buf)) return RTG_ERR_IO;
    const char *base = buf.data(), *end = base + buf.size();
    bool symmetric = false, bad = false, have_head = false, have_size = false;
    long long rows = -1, cols = -1, nnz = -1;
    const char *body = end;
    for_lines(buf, [&](const char *p, const char *e) {
        if (!have_head) {
            const std::string head(p, e);
            std::string lower = head;
            for (auto &ch : lower) ch = (char)std::tolower((unsigned char)ch);
            if (head.rfind("%%MatrixMarket", 0) != 0 ||
                lower.find("coordinate") == std::string::npos) {
                bad = true;
                return false;
            }
            symmetric = lower.find("symmetric") != std::string::npos;
            have_head = true;
            return true;
        }
        if (p == e || *p == '%') return true;  // empty and comment lines
        if (!read_ll(p, e, rows) || !read_ll(p, e, cols) || !read_ll(p, e, nnz) || nnz < 0) {
            bad = true;
            return false;
        }
        have_size = true;
        body = e < end ? e + 1 : end;
        return false;
    });
    if (bad || !have_size) return RTG_ERR_FORMAT;
    const size_t n = (size_t)(end - body);
    const int T = nnz ? (int)std::max<size_t>(1, std::min<size_t>((size_t)omp_get_max_threads(),
                                                                  n / (1u << 20) + 1))
                      : 0;
    std::vector<size_t> cut(T + 1, n);
    if (T) cut[0] = 0;
    for (int t = 1; t < T; ++t) {
        const size_t at = std::max(cut[t - 1], n / T * t);
        const char *nl = at < n ? static_cast<const char *>(std::memchr(body + at, '\n', n - at))
                                : nullptr;
        cut[t] = nl ? (size_t)(nl - body) + 1 : n;
    }
    std::vector<std::vector<uint32_t>> pr(T), pc(T);
    std::vector<long long> stop(T, -1);
    std::vector<char> oom(T, 0);
#pragma omp parallel for num_threads(T > 0 ? T : 1) schedule(static, 1)
    for (int t = 0; t < T; ++t) {
        const size_t len = cut[t + 1] - cut[t];
        // a failed allocation inside the parallel region stays in its piece
        try {
            pr[t].reserve(len / 4 + 1);
            pc[t].reserve(len / 4 + 1);
            stop[t] = parse_mtx_entries(body + cut[t], body + cut[t + 1], rows, cols, pr[t], pc[t]);
        } catch (...) {
            oom[t] = 1;
        }
    }
    for (int t = 0; t < T; ++t)
        if (oom[t]) return RTG_ERR_OOM;
    // the first nnz entries in file order; a bad line before them is a format error
    long long seen = 0;
    std::vector<std::pair<int, size_t>> take;  // (piece, entries taken from it)
    for (int t = 0; t < T && seen < nnz; ++t) {
        const long long k = std::min<long long>((long long)pr[t].size(), nnz - seen);
        take.push_back({t, (size_t)k});
        seen += k;
        if (stop[t] >= 0 && seen < nnz) return RTG_ERR_FORMAT;
    }
    if (seen != nnz) return RTG_ERR_FORMAT;
    size_t edges = 0;
    for (auto &tk : take)
        for (size_t i = 0; i < tk.second; ++i)
            edges += (symmetric && pr[tk.first][i] != pc[tk.first][i]) ? 2 : 1;
    s.resize(edges);
    d.resize(edges);
    size_t at = 0;
    for (auto &tk : take)
        for (size_t i = 0; i < tk.second; ++i) {
            const uint32_t r = pr[tk.first][i], c = pc[tk.first][i];
            s[at] = r - 1;
            d[at++] = c - 1;
            if (symmetric && r != c) {
                s[at] = c - 1;
                d[at++] = r - 1;
            }
        }
    return RTG_OK;
}

}  // namespace

extern "C" {

static rtg_status rtg_edges_read_body(const char *path, rtg_format fmt, uint64_t *m, uint32_t *src,
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

rtg_status rtg_edges_read(const char *path, rtg_format fmt, uint64_t *m, uint32_t *src,
                          uint32_t *dst) {
    return rtg::host_alloc_guard([&] { return rtg_edges_read_body(path, fmt, m, src, dst); });
}

extern "C++" {
namespace rtg {
rtg_status graph_load_cached(rtg_ctx *ctx, const char *path, rtg_graph **out);  // csr_cache.cpp
}
}

static rtg_status rtg_graph_load_body(rtg_ctx *ctx, const char *path, rtg_format fmt, rtg_graph **out) {
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

rtg_status rtg_graph_load(rtg_ctx *ctx, const char *path, rtg_format fmt, rtg_graph **out) {
    return rtg::host_alloc_guard([&] { return rtg_graph_load_body(ctx, path, fmt, out); });
}

static rtg_status rtg_edges_write_bin_body(const char *path, const uint32_t *src, const uint32_t *dst,
                               uint64_t m) {
    if (!path || (m && (!src || !dst))) return RTG_ERR_INVALID_ARG;
    const uint64_t chunk = 1 << 20;
    std::vector<int32_t> buf;
    buf.reserve(2 * std::min<uint64_t>(m, chunk));  // before the file is opened
    FILE *f = std::fopen(path, "wb");
    if (!f) return RTG_ERR_IO;
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

rtg_status rtg_edges_write_bin(const char *path, const uint32_t *src, const uint32_t *dst,
                               uint64_t m) {
    return rtg::host_alloc_guard([&] { return rtg_edges_write_bin_body(path, src, dst, m); });
}

static rtg_status rtg_dataset_read_body(const char *path, rtg_dataset_info *info, uint32_t *offsets,
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
    // the offsets must fit the file before they are allocated
    long long size = -1;
    if (std::fseek(f, 0, SEEK_END) == 0) size = std::ftell(f);
    if (size < 0 || std::fseek(f, 16, SEEK_SET) != 0) {
        std::fclose(f);
        return RTG_ERR_IO;
    }
    if ((uint64_t)size < 16 + (nsets + 1) * 4) {
        std::fclose(f);
        return RTG_ERR_FORMAT;
    }
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

rtg_status rtg_dataset_read(const char *path, rtg_dataset_info *info, uint32_t *offsets,
                            uint32_t *elems) {
    return rtg::host_alloc_guard([&] { return rtg_dataset_read_body(path, info, offsets, elems); });
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
