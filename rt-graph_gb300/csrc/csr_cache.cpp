// On-disk CSR cache: the CSRs a graph holds on the device (oriented, counting form,
// symmetric), written to one file and read back without the sort-based build. The layout
// is this library's own; the CSR arrays are the same ones the reference keeps in
// Graph::offsets_/adjs_ (tc/graph/graph.cpp:71-102), widened to 64-bit offsets.
//
// File (little endian):
//   char magic[8] = "RTGCSR01"; u32 version = 2; u32 parts (bit 0 oriented, 1 counting,
//   2 symmetric); u64 m_input; i32 orient; u32 zero;
//   oriented : u32 n, u32 max_deg, u64 m, u64 work_elems, u32 has_src, u32 zero,
//              u64 off[n+1], u32 adj[m], (u32 src[m])
//   counting : u32 n, u32 max_deg, u64 m, u64 off[n+1], u32 adj[m], u64 in_off[n+1],
//              uint2 in_rng[m]
//   symmetric: u32 n, u32 max_deg, u64 m, u64 work_elems, u64 off[n+1], u32 adj[m]
//   u64 checksum of every byte between the magic and the checksum (the payload): FNV-1a-64
//   over the 64-bit words of each 1 MiB block (a block's last bytes one at a time), the
//   blocks' values chained in order by FNV-1a-64 seeded with the payload length, so that
//   the blocks are summed in parallel.
// A file is accepted only if its checksum matches and every array describes a valid CSR
// (offsets non-decreasing from 0 to m, ids below n, suffix ranges inside their rows), so a
// damaged or foreign file fails with RTG_ERR_FORMAT before anything reaches a kernel. The
// file is built whole in host memory (device arrays copied straight into it) and written
// in pieces by the host threads; it is read whole the same way, and its checks run in
// parallel, each suffix range checked against a table of row ends (R-MAT-20 counting
// form, 205 MB, 8 threads:
// 1.9 s with a binary search per range, 0.5 s with the table).
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include <fcntl.h>
#include <omp.h>
#include <sys/stat.h>
#include <unistd.h>

#include "internal.h"

namespace rtg {
namespace {

constexpr char kMagic[8] = {'R', 'T', 'G', 'C', 'S', 'R', '0', '1'};
constexpr uint32_t kVersion = 2;
constexpr size_t kSumBlock = size_t(1) << 20;

uint64_t block_sum(const unsigned char *p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    size_t i = 0;
    for (; i + 8 <= n; i += 8) {
        uint64_t w;
        std::memcpy(&w, p + i, 8);
        h = (h ^ w) * 1099511628211ull;
    }
    for (; i < n; ++i) h = (h ^ p[i]) * 1099511628211ull;
    return h;
}

uint64_t payload_sum(const unsigned char *p, size_t n) {
    const size_t nb = (n + kSumBlock - 1) / kSumBlock;
    std::vector<uint64_t> bs(nb);
#pragma omp parallel for schedule(static)
    for (long long b = 0; b < (long long)nb; ++b)
        bs[b] = block_sum(p + b * kSumBlock, std::min(kSumBlock, n - (size_t)b * kSumBlock));
    uint64_t h = (1469598103934665603ull ^ (uint64_t)n) * 1099511628211ull;
    for (uint64_t v : bs) h = (h ^ v) * 1099511628211ull;
    return h;
}
constexpr uint32_t kPartOri = 1, kPartCnt = 2, kPartSym = 4;

// The payload of a file read whole.
// Host arrays filled by copies: resized without zeroing them first.
template <class T> struct NoInit {
    using value_type = T;
    NoInit() = default;
    template <class U> NoInit(const NoInit<U> &) {}
    T *allocate(size_t k) { return static_cast<T *>(::operator new(k * sizeof(T))); }
    void deallocate(T *q, size_t) { ::operator delete(q); }
    template <class U> void construct(U *q) { ::new ((void *)q) U; }
    template <class U, class A, class... B> void construct(U *q, A &&a, B &&...b) {
        ::new ((void *)q) U(std::forward<A>(a), std::forward<B>(b)...);
    }
    template <class U> bool operator==(const NoInit<U> &) const { return true; }
    template <class U> bool operator!=(const NoInit<U> &) const { return false; }
};
template <class T> using HostVec = std::vector<T, NoInit<T>>;

// Large copies split over the host threads.
void copy_parallel(void *dst, const void *src, size_t bytes) {
    constexpr size_t kPiece = size_t(4) << 20;
    const long long pieces = (long long)((bytes + kPiece - 1) / kPiece);
#pragma omp parallel for schedule(static) if (pieces > 1)
    for (long long i = 0; i < pieces; ++i) {
        const size_t at = (size_t)i * kPiece;
        std::memcpy((char *)dst + at, (const char *)src + at, std::min(kPiece, bytes - at));
    }
}

// The whole file in host memory (magic, payload, checksum), sized up front and touched by
// the host threads before anything is copied in (a device-to-host copy into pages not yet
// mapped maps them one fault at a time: R-MAT-21's 686 MB saved in 0.51-0.59 s that way);
// device arrays are copied straight into it.
struct Writer {
    HostVec<unsigned char> buf;
    size_t at = 0;
    explicit Writer(size_t bytes) {
        buf.resize(bytes);
        constexpr size_t kPiece = size_t(4) << 20;
        const long long pieces = (long long)((bytes + kPiece - 1) / kPiece);
#pragma omp parallel for schedule(static) if (pieces > 1)
        for (long long i = 0; i < pieces; ++i) {
            const size_t a = (size_t)i * kPiece;
            std::memset(buf.data() + a, 0, std::min(kPiece, bytes - a));
        }
    }
    unsigned char *take(size_t bytes) {
        if (at + bytes > buf.size()) buf.resize(at + bytes);
        unsigned char *q = buf.data() + at;
        at += bytes;
        return q;
    }
    void put(const void *p, size_t bytes) {
        if (bytes) std::memcpy(take(bytes), p, bytes);
    }
    template <class T> void val(T v) { put(&v, sizeof v); }
    rtg_status dev(rtg_ctx *ctx, const void *d, size_t bytes) {
        unsigned char *q = take(bytes);
        if (bytes) RTG_CUDA(ctx, cudaMemcpy(q, d, bytes, cudaMemcpyDeviceToHost));
        return RTG_OK;
    }
};

// Write n bytes at p to a new file at path, in pieces by the host threads; on any failure
// the partial file is removed.
bool write_file(const char *path, const unsigned char *p, size_t n) {
    const int fd = ::open(path, O_WRONLY | O_CREAT | O_TRUNC | O_CLOEXEC, 0644);
    if (fd < 0) return false;
    constexpr size_t kPiece = size_t(8) << 20;
    const long long pieces = (long long)((n + kPiece - 1) / kPiece);
    int bad = 0;
#pragma omp parallel for schedule(static) reduction(| : bad) if (pieces > 1)
    for (long long i = 0; i < pieces; ++i) {
        size_t at = (size_t)i * kPiece;
        const size_t end = std::min(n, at + kPiece);
        while (at < end) {
            const ssize_t put = ::pwrite(fd, p + at, end - at, (off_t)at);
            if (put < 0 && errno == EINTR) continue;
            if (put <= 0) {
                bad = 1;
                break;
            }
            at += (size_t)put;
        }
    }
    if (::close(fd) != 0) bad = 1;
    if (bad) std::remove(path);
    return !bad;
}

struct Reader {
    const unsigned char *p;
    uint64_t left;
    bool ok = true;
    bool get(void *dst, size_t bytes) {
        if (!ok || bytes > left) return ok = false;
        if (bytes) copy_parallel(dst, p, bytes);
        p += bytes;
        left -= bytes;
        return true;
    }
    template <class T> bool val(T &v) { return get(&v, sizeof v); }
};


// offsets non-decreasing from 0 to m
bool valid_offsets(const HostVec<uint64_t> &off, uint64_t n, uint64_t m) {
    if (off[0] != 0 || off[n] != m) return false;
    int bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static)
    for (long long v = 0; v < (long long)n; ++v) bad |= off[v + 1] < off[v];
    return !bad;
}

bool valid_ids(const HostVec<uint32_t> &ids, uint64_t m, uint64_t n) {
    int bad = 0;
#pragma omp parallel for reduction(| : bad) schedule(static)
    for (long long i = 0; i < (long long)m; ++i) bad |= ids[i] >= n;
    return !bad;
}

template <class T>
rtg_status upload(rtg_ctx *ctx, T **d, const HostVec<T> &h, uint64_t count, size_t pad) {
    RTG_TRY(dev_alloc(ctx, (void **)d, count * sizeof(T) + pad));
    if (count) RTG_CUDA(ctx, cudaMemcpy(*d, h.data(), count * sizeof(T), cudaMemcpyHostToDevice));
    if (pad) RTG_CUDA(ctx, cudaMemset((char *)*d + count * sizeof(T), 0, pad));
    return RTG_OK;
}

}  // namespace
}  // namespace rtg

using namespace rtg;

static rtg_status graph_save_body(rtg_ctx *ctx, const rtg_graph *g, const char *path);

extern "C" rtg_status rtg_graph_save(rtg_ctx *ctx, const rtg_graph *g, const char *path) {
    if (!ctx || !g || !path) return RTG_ERR_INVALID_ARG;
    // the payload is assembled in host memory before the file is opened
    const rtg_status st = host_alloc_guard([&] { return graph_save_body(ctx, g, path); });
    if (st == RTG_ERR_OOM) return fail(ctx, st, "no host memory for the file of %s", path);
    return st;
}

static rtg_status graph_save_body(rtg_ctx *ctx, const rtg_graph *g, const char *path) {
    const uint32_t parts = (g->ori.built ? kPartOri : 0) | (g->cnt.built ? kPartCnt : 0) |
                           (g->sym.built ? kPartSym : 0);
    if (!parts) return fail(ctx, RTG_ERR_STATE, "graph holds no CSR to save");
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // a form holding part of its in-edges (a one-shot count's) is never written
    if ((parts & kPartCnt) && g->cnt.inedges() != g->cnt.m) return RTG_ERR_STATE;
    auto csr_bytes = [](const Csr &c, bool with_src) {
        return 24 + (with_src ? 8 : 0) + (c.n + 1ull) * 8 + c.m * 4 +
               (with_src && c.src ? c.m * 4 : 0);
    };
    uint64_t total = 8 + 24 + 8;
    if (parts & kPartOri) total += csr_bytes(g->ori, true);
    if (parts & kPartCnt) total += 16 + (g->cnt.n + 1ull) * 16 + g->cnt.m * 12;
    if (parts & kPartSym) total += csr_bytes(g->sym, false);
    Writer w(total);
    w.put(kMagic, 8);
    w.val(kVersion);
    w.val(parts);
    w.val(g->m_input);
    w.val((int32_t)g->orient);
    w.val((uint32_t)0);
    auto csr = [&](const Csr &c, bool with_src) -> rtg_status {
        w.val(c.n);
        w.val(c.max_deg);
        w.val(c.m);
        w.val(c.work_elems);
        if (with_src) {
            w.val((uint32_t)(c.src ? 1 : 0));
            w.val((uint32_t)0);
        }
        RTG_TRY(w.dev(ctx, c.off, (c.n + 1ull) * 8));
        RTG_TRY(w.dev(ctx, c.adj, c.m * 4));
        if (with_src && c.src) RTG_TRY(w.dev(ctx, c.src, c.m * 4));
        return RTG_OK;
    };
    if (parts & kPartOri) RTG_TRY(csr(g->ori, true));
    if (parts & kPartCnt) {
        const CountCsr &c = g->cnt;
        w.val(c.n);
        w.val(c.max_deg);
        w.val(c.m);
        RTG_TRY(w.dev(ctx, c.off, (c.n + 1ull) * 8));
        RTG_TRY(w.dev(ctx, c.adj, c.m * 4));
        RTG_TRY(w.dev(ctx, c.in_off, (c.n + 1ull) * 8));
        RTG_TRY(w.dev(ctx, c.in_rng, c.m * 8));
    }
    if (parts & kPartSym) RTG_TRY(csr(g->sym, false));
    w.val(payload_sum(w.buf.data() + 8, w.at - 8));
    if (!write_file(path, w.buf.data(), w.at))
        return fail(ctx, RTG_ERR_IO, "cannot write %s", path);
    return RTG_OK;
}

namespace rtg {
namespace {

// One CSR part of a cache file, read and checked on the host.
struct HostCsr {
    uint32_t n = 0, max_deg = 0, has_src = 0;
    uint64_t m = 0, work = 0;
    HostVec<uint64_t> off, in_off;
    HostVec<uint32_t> adj, src;
    HostVec<uint2> rng;
};

struct CacheFile {
    uint32_t parts = 0;
    uint64_t m_input = 0;
    int32_t orient = -1;
    HostCsr ori, cnt, sym;
};

// Read and check a file written by rtg_graph_save, on the host only (no device, no
// context). RTG_ERR_IO when it cannot be opened, RTG_ERR_FORMAT with the reason in `why`
// when it is not a valid cache file. Without `structure` (the checked build's test hook)
// only the sizes and the checksum are checked, so that a forged form reaches the device
// checks of that build.
rtg_status read_cache_file(const char *path, CacheFile &cf, std::string &why,
                           bool structure = true) {
    const int fd = ::open(path, O_RDONLY | O_CLOEXEC);
    if (fd < 0) {
        why = "cannot open file";
        return RTG_ERR_IO;
    }
    // the whole file, read in pieces by the host threads
    HostVec<unsigned char> file;
    {
        struct stat sb;
        bool err = ::fstat(fd, &sb) != 0 || !S_ISREG(sb.st_mode);
        const size_t size = err ? 0 : (size_t)sb.st_size;
        file.resize(size);
        constexpr size_t kPiece = size_t(8) << 20;
        const long long pieces = (long long)((size + kPiece - 1) / kPiece);
        int short_read = 0;
#pragma omp parallel for schedule(static) reduction(| : short_read) if (pieces > 1)
        for (long long i = 0; i < pieces; ++i) {
            size_t at = (size_t)i * kPiece;
            const size_t end = std::min(size, at + kPiece);
            while (at < end) {
                const ssize_t got = ::pread(fd, file.data() + at, end - at, (off_t)at);
                if (got < 0 && errno == EINTR) continue;
                if (got <= 0) {
                    short_read = 1;
                    break;
                }
                at += (size_t)got;
            }
        }
        ::close(fd);
        if (err || short_read) {
            why = "cannot read file";
            return RTG_ERR_IO;
        }
    }
    auto bad = [&](const char *w) {
        why = w;
        return RTG_ERR_FORMAT;
    };
    if (file.size() < 8 + 8 || std::memcmp(file.data(), kMagic, 8))
        return bad("not a CSR cache file");
    Reader r{file.data() + 8, (uint64_t)file.size() - 8 - 8};  // checksum excluded
    uint32_t version = 0, zero = 0;
    r.val(version);
    r.val(cf.parts);
    r.val(cf.m_input);
    r.val(cf.orient);
    r.val(zero);
    if (!r.ok || version != kVersion || !cf.parts || (cf.parts & ~7u)) return bad("bad header");
    {
        uint64_t want = 0;
        std::memcpy(&want, file.data() + file.size() - 8, 8);
        if (payload_sum(file.data() + 8, file.size() - 16) != want)
            return bad("checksum mismatch");
    }
    auto read_csr = [&](HostCsr &c, bool with_src, bool with_work) -> bool {
        if (!r.val(c.n) || !r.val(c.max_deg) || !r.val(c.m)) return false;
        if (with_work && !r.val(c.work)) return false;
        if (with_src && (!r.val(c.has_src) || !r.val(zero))) return false;
        // sizes must fit what is left of the file before anything is allocated
        const uint64_t need = (c.n + 1ull) * 8 + c.m * 4 + (c.has_src ? c.m * 4 : 0);
        if (c.m > r.left || need > r.left) return false;
        c.off.resize(c.n + 1ull);
        c.adj.resize(c.m ? c.m : 1);
        if (!r.get(c.off.data(), (c.n + 1ull) * 8) || !r.get(c.adj.data(), c.m * 4)) return false;
        if (c.has_src) {
            c.src.resize(c.m ? c.m : 1);
            if (!r.get(c.src.data(), c.m * 4)) return false;
        }
        if (!structure) return true;
        return valid_offsets(c.off, c.n, c.m) && valid_ids(c.adj, c.m, c.n) &&
               (!c.has_src || valid_ids(c.src, c.m, c.n));
    };
    if ((cf.parts & kPartOri) && !read_csr(cf.ori, true, true)) return bad("oriented CSR");
    if (cf.parts & kPartCnt) {
        HostCsr &hc = cf.cnt;
        if (!read_csr(hc, false, false)) return bad("counting CSR");
        const uint64_t need = (hc.n + 1ull) * 8 + hc.m * 8;
        if (need > r.left) return bad("counting CSR");
        hc.in_off.resize(hc.n + 1ull);
        hc.rng.resize(hc.m ? hc.m : 1);
        if (!r.get(hc.in_off.data(), (hc.n + 1ull) * 8) || !r.get(hc.rng.data(), hc.m * 8))
            return bad("counting CSR");
        if (structure && !valid_offsets(hc.in_off, hc.n, hc.m)) return bad("counting CSR in-edges");
        // the batched kernel indexes its per-warp bitmap by (element - window origin) and
        // takes every element of a suffix of an in-edge of v to be a rank above v: every
        // row of v must hold ascending ranks above v, and every suffix range of an in-edge
        // of v must lie inside one row and hold only ranks above v; the in-edges of v are
        // ordered by source (a range never starts before the previous in-edge's), which the
        // dense-core split relies on (the in-edges from core rows are the last ones of v)
        int row_bad = 0, range_bad = 0, order_bad = 0;
        const long long nv = structure ? (long long)hc.n : 0;
#pragma omp parallel for reduction(| : row_bad) schedule(dynamic, 4096)
        for (long long v = 0; v < nv; ++v)
            for (uint64_t q = hc.off[v]; q < hc.off[v + 1]; ++q)
                row_bad |= hc.adj[q] <= (uint64_t)v || (q > hc.off[v] && hc.adj[q] <= hc.adj[q - 1]);
        if (row_bad) return bad("counting CSR row order");
        // the end of the row holding each position (the offsets are checked: every
        // position lies in exactly one row), so that a range is checked in O(1)
        std::unique_ptr<uint32_t[]> row_end(new uint32_t[structure && hc.m ? hc.m : 1]);
#pragma omp parallel for schedule(dynamic, 4096)
        for (long long v = 0; v < nv; ++v)
            for (uint64_t q = hc.off[v]; q < hc.off[v + 1]; ++q) row_end[q] = (uint32_t)hc.off[v + 1];
#pragma omp parallel for reduction(| : range_bad, order_bad) schedule(dynamic, 4096)
        for (long long v = 0; v < nv; ++v)
            for (uint64_t e = hc.in_off[v]; e < hc.in_off[v + 1]; ++e) {
                const uint2 rg = hc.rng[e];
                if (rg.x > rg.y || rg.y > hc.m) {
                    range_bad = 1;
                    continue;
                }
                if (e > hc.in_off[v] && rg.x < hc.rng[e - 1].x) order_bad = 1;
                if (rg.x == rg.y) continue;
                if (rg.y > row_end[rg.x] || hc.adj[rg.x] <= (uint64_t)v) range_bad = 1;
            }
        if (range_bad) return bad("suffix range");
        if (order_bad) return bad("in-edge order");
    }
    if ((cf.parts & kPartSym) && !read_csr(cf.sym, false, true)) return bad("symmetric CSR");
    if (!r.ok || r.left != 0) return bad("trailing bytes");
    return RTG_OK;
}

}  // namespace

// Read a file written by rtg_graph_save into a new graph of ctx (no raw edges).
rtg_status graph_load_cached(rtg_ctx *ctx, const char *path, rtg_graph **out) {
    CacheFile cf;
    std::string why = "no host memory for the file";
    const rtg_status rs = host_alloc_guard(
        [&] { return read_cache_file(path, cf, why, !(kChecked && g_skip_file_structure_checks)); });
    if (rs != RTG_OK) return fail(ctx, rs, "%s: %s", path, why.c_str());
    const uint32_t parts = cf.parts;
    const uint64_t m_input = cf.m_input;
    const int32_t orient = cf.orient;
    HostCsr &ho = cf.ori, &hc = cf.cnt, &hs = cf.sym;
    rtg_graph *g = nullptr;
    // an empty edge list gives a graph with no raw edges to which the CSRs are attached
    RTG_TRY(rtg_graph_from_host_edges(ctx, nullptr, nullptr, 0, &g));
    g->m_input = m_input;
    g->edges_released = true;
    g->orient = orient;
    rtg_status st = RTG_OK;
    auto up_csr = [&](Csr &c, HostCsr &hcsr) {
        c.n = hcsr.n;
        c.m = hcsr.m;
        c.max_deg = hcsr.max_deg;
        c.work_elems = hcsr.work;
        if (st == RTG_OK) st = upload(ctx, &c.off, hcsr.off, hcsr.n + 1ull, 0);
        if (st == RTG_OK) st = upload(ctx, &c.adj, hcsr.adj, hcsr.m, kAdjPadBytes);
        if (st == RTG_OK && hcsr.has_src) st = upload(ctx, &c.src, hcsr.src, hcsr.m, 0);
        c.built = st == RTG_OK;
    };
    if (parts & kPartOri) up_csr(g->ori, ho);
    if (parts & kPartCnt) {
        CountCsr &c = g->cnt;
        c.n = hc.n;
        c.m = hc.m;
        c.max_deg = hc.max_deg;
        if (st == RTG_OK) st = upload(ctx, &c.off, hc.off, hc.n + 1ull, 0);
        if (st == RTG_OK) st = upload(ctx, &c.adj, hc.adj, hc.m, kAdjPadBytes);
        if (st == RTG_OK) st = upload(ctx, &c.in_off, hc.in_off, hc.n + 1ull, 0);
        if (st == RTG_OK) st = upload(ctx, &c.in_rng, hc.rng, hc.m, 0);
        // the library's dense-core size, from the offsets already on the host
        c.core_auto = hc.m ? core_auto_host(hc.off.data(), hc.n, hc.m) : 0;
        c.built = st == RTG_OK;
    }
    if (parts & kPartSym) up_csr(g->sym, hs);
    if (st != RTG_OK) {
        rtg_graph_destroy(g);
        return st;
    }
    *out = g;
    return RTG_OK;
}

}  // namespace rtg

extern "C" rtg_status rtg_graph_file_check(const char *path) {
    if (!path) return RTG_ERR_INVALID_ARG;
    rtg::CacheFile cf;
    std::string why;
    return rtg::host_alloc_guard([&] { return rtg::read_cache_file(path, cf, why); });
}
