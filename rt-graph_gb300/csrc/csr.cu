// GPU CSR builder.
//
// Edges are packed into 64-bit keys (hi << B | lo, B = bits needed for the largest id),
// sorted with CUB's radix sort (only the 2B significant bits), deduplicated, and the CSR
// offsets are written from the sorted keys without atomics.
//
// Two oriented forms are built:
//  DEGREE          – simple graph first (self loops and duplicates removed on the
//                    canonical (min,max) key), then each edge oriented from the lower
//                    (degree, id) endpoint to the higher one.
//  DEGREE_RAW_REF  – the reference preprocessing of tc/graph/graph.cpp, stage by stage:
//                    ids compacted to dense ranks of the used ids (graph.cpp:40-62),
//                    degree counted on the raw list including duplicates and self loops
//                    (graph.cpp:108-114), orientation "swap when deg[src] > deg[dst] or
//                    equal degrees and src > dst" (graph.cpp:116-124), vertices of raw
//                    degree <= 1 dropped and ids shifted down by the number of dropped
//                    smaller ids (graph.cpp:126-149), sort (graph.cpp:157), duplicates and
//                    self loops removed (graph.cpp:160-173), CSR (graph.cpp:71-102).
//  SYMMETRIC       – simple graph with both directions stored.
#include <cub/cub.cuh>
#include <thrust/iterator/zip_iterator.h>

#include <algorithm>

#include "internal.h"

namespace rtg {

namespace {

constexpr int kThreads = 256;

inline int grid_for(rtg_ctx *ctx, uint64_t n) {
    uint64_t g = (n + kThreads - 1) / kThreads;
    uint64_t cap = (uint64_t)ctx->sm_count * 16;
    return (int)std::max<uint64_t>(1, std::min(g, cap));
}

inline int bits_for(uint64_t x) {  // bits needed to represent x (x >= 1)
    int b = 0;
    while (b < 64 && (x >> b)) ++b;
    return std::max(b, 1);
}

#define GRID_STRIDE(i, n)                                                              \
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < (n);         \
         i += (uint64_t)gridDim.x * blockDim.x)

__global__ void k_max_id(const uint32_t *s, const uint32_t *d, uint64_t m, unsigned int *out) {
    unsigned int mx = 0;
    GRID_STRIDE(i, m) { mx = max(mx, max(s[i], d[i])); }
    for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

// canonical undirected key; self loops become the sentinel
__global__ void k_canon_keys(const uint32_t *s, const uint32_t *d, uint64_t m, int B,
                             uint64_t sentinel, uint64_t *keys) {
    GRID_STRIDE(i, m) {
        uint32_t a = s[i], b = d[i];
        keys[i] = (a == b) ? sentinel : (((uint64_t)min(a, b) << B) | max(a, b));
    }
}

__global__ void k_degree_from_keys(const uint64_t *keys, uint64_t m, int B, uint32_t *deg) {
    const uint64_t lo_mask = (1ull << B) - 1;
    GRID_STRIDE(i, m) {
        uint64_t k = keys[i];
        atomicAdd(&deg[k >> B], 1u);
        atomicAdd(&deg[k & lo_mask], 1u);
    }
}

__global__ void k_orient_keys(uint64_t *keys, uint64_t m, int B, const uint32_t *deg) {
    const uint64_t lo_mask = (1ull << B) - 1;
    GRID_STRIDE(i, m) {
        uint64_t k = keys[i];
        uint32_t a = (uint32_t)(k >> B), b = (uint32_t)(k & lo_mask);  // a < b
        uint32_t da = deg[a], db = deg[b];
        bool keep = (da < db) || (da == db);  // ties go to the smaller id, which is a
        keys[i] = keep ? k : (((uint64_t)b << B) | a);
    }
}

__global__ void k_sym_keys(const uint64_t *ukeys, uint64_t m, int B, uint64_t *out) {
    const uint64_t lo_mask = (1ull << B) - 1;
    GRID_STRIDE(i, m) {
        uint64_t k = ukeys[i];
        uint64_t a = k >> B, b = k & lo_mask;
        out[2 * i] = k;
        out[2 * i + 1] = (b << B) | a;
    }
}

// row offsets of keys sorted by (key >> shift): off[x] = first i with (keys[i] >> shift) >= x
__global__ void k_row_offsets(const uint64_t *keys, uint64_t m, int shift, uint32_t n,
                              uint64_t *off) {
    GRID_STRIDE(x, (uint64_t)n + 1) {
        uint64_t lo = 0, hi = m;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if ((keys[mid] >> shift) < x) lo = mid + 1;
            else hi = mid;
        }
        off[x] = lo;
    }
}

// adj/src from sorted keys
__global__ void k_csr_fill(const uint64_t *keys, uint64_t m, int B, uint32_t *adj,
                           uint32_t *src) {
    const uint64_t lo_mask = (1ull << B) - 1;
    GRID_STRIDE(i, m) {
        const uint64_t k = keys[i];
        adj[i] = (uint32_t)(k & lo_mask);
        if (src) src[i] = (uint32_t)(k >> B);
    }
}

__global__ void k_stats(const uint64_t *off, const uint32_t *adj, const uint32_t *src, uint64_t m,
                        uint32_t n, unsigned long long *work, unsigned int *maxdeg) {
    unsigned long long acc = 0;
    unsigned int md = 0;
    if (src) {
        GRID_STRIDE(e, m) {
            uint32_t u = src[e], v = adj[e];
            acc += (off[u + 1] - off[u]) + (off[v + 1] - off[v]);
        }
    }
    GRID_STRIDE(v, (uint64_t)n) { md = max(md, (unsigned int)(off[v + 1] - off[v])); }
    for (int o = 16; o; o >>= 1) {
        acc += __shfl_down_sync(0xffffffffu, acc, o);
        md = max(md, __shfl_down_sync(0xffffffffu, md, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (acc) atomicAdd(work, acc);
        atomicMax(maxdeg, md);
    }
}

// ---- reference-exact (DEGREE_RAW_REF) stages
__global__ void k_mark_used(const uint32_t *s, const uint32_t *d, uint64_t m, uint32_t *used) {
    GRID_STRIDE(i, m) {
        used[s[i]] = 1u;
        used[d[i]] = 1u;
    }
}

__global__ void k_relabel_raw_degree(const uint32_t *s, const uint32_t *d, uint64_t m,
                                     const uint32_t *rank, uint32_t *s2, uint32_t *d2,
                                     uint32_t *deg) {
    GRID_STRIDE(i, m) {
        uint32_t a = rank[s[i]] - 1, b = rank[d[i]] - 1;
        s2[i] = a;
        d2[i] = b;
        atomicAdd(&deg[a], 1u);
        atomicAdd(&deg[b], 1u);
    }
}

__global__ void k_flag_low_degree(const uint32_t *deg, uint32_t n, uint32_t *flag) {
    GRID_STRIDE(v, (uint64_t)n) { flag[v] = deg[v] <= 1 ? 1u : 0u; }
}

__global__ void k_ref_orient_keys(const uint32_t *s2, const uint32_t *d2, uint64_t m,
                                  const uint32_t *deg, const uint32_t *removes, int B,
                                  uint64_t sentinel, uint64_t *keys) {
    GRID_STRIDE(i, m) {
        uint32_t a = s2[i], b = d2[i];
        if (deg[a] > deg[b] || (deg[a] == deg[b] && a > b)) {
            uint32_t t = a;
            a = b;
            b = t;
        }
        if (deg[a] <= 1 || deg[b] <= 1) {
            keys[i] = sentinel;
        } else {
            a -= removes[a];
            b -= removes[b];
            keys[i] = ((uint64_t)a << B) | b;
        }
    }
}

__global__ void k_ref_keep_flags(const uint64_t *keys, uint64_t m, int B, uint64_t sentinel,
                                 uint8_t *flags) {
    const uint64_t lo_mask = (1ull << B) - 1;
    GRID_STRIDE(i, m) {
        uint64_t k = keys[i];
        bool keep = k != sentinel && (k >> B) != (k & lo_mask) && (i == 0 || keys[i - 1] != k);
        flags[i] = keep ? 1 : 0;
    }
}

// Temporaries of one build step, taken in order from the context's grow-only work slots
// (one Buffers at a time per context; builds on a context are stream-ordered, so a slot
// is never reused while earlier work on it is pending).
struct Buffers {
    rtg_ctx *ctx;
    int next = 0;
    template <class T>
    rtg_status alloc(T **p, uint64_t count) {
        constexpr int kSlots = sizeof(ctx->work) / sizeof(ctx->work[0]);
        if (next >= kSlots) return fail(ctx, RTG_ERR_STATE, "builder work slots exhausted");
        DeviceBuffer &b = ctx->work[next++];
        const size_t bytes = std::max<size_t>(count * sizeof(T), 256);
        if (b.bytes < bytes) {
            dev_free(b.ptr);
            b.ptr = nullptr;
            b.bytes = 0;
            RTG_TRY(dev_alloc(ctx, &b.ptr, bytes));
            b.bytes = bytes;
        }
        *p = (T *)b.ptr;
        return RTG_OK;
    }
};

rtg_status radix_sort(rtg_ctx *ctx, cub::DoubleBuffer<uint64_t> &db, uint64_t m, int end_bit) {
    if (m < 2) return RTG_OK;
    size_t bytes = 0;
    RTG_CUDA(ctx, cub::DeviceRadixSort::SortKeys(nullptr, bytes, db, (int64_t)m, 0, end_bit,
                                                 ctx->stream));
    void *tmp = nullptr;
    RTG_TRY(scratch(ctx, 0, bytes, &tmp));
    RTG_CUDA(ctx, cub::DeviceRadixSort::SortKeys(tmp, bytes, db, (int64_t)m, 0, end_bit,
                                                 ctx->stream));
    ctx->launches += (end_bit + 7) / 8 + 1;
    return RTG_OK;
}

template <class T>
rtg_status inclusive_sum(rtg_ctx *ctx, const T *in, T *out, uint64_t n) {
    size_t bytes = 0;
    RTG_CUDA(ctx, cub::DeviceScan::InclusiveSum(nullptr, bytes, in, out, (int64_t)n, ctx->stream));
    void *tmp = nullptr;
    RTG_TRY(scratch(ctx, 0, bytes, &tmp));
    RTG_CUDA(ctx, cub::DeviceScan::InclusiveSum(tmp, bytes, in, out, (int64_t)n, ctx->stream));
    ctx->launches += 2;
    return RTG_OK;
}

rtg_status read_u32(rtg_ctx *ctx, const uint32_t *d, uint32_t *h) {
    RTG_CUDA(ctx, cudaMemcpyAsync(h, d, 4, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RTG_OK;
}

// Fill a CSR (offsets, adj, optional src) from sorted keys and compute its stats.
rtg_status fill_csr(rtg_ctx *ctx, const uint64_t *keys, uint64_t m, int B, uint32_t n,
                    bool with_src, Csr &c) {
    graph_free_csr(c);
    c.n = n;
    c.m = m;
    RTG_TRY(dev_alloc(ctx, (void **)&c.off, (n + 1ull) * 8));
    RTG_TRY(dev_alloc(ctx, (void **)&c.adj, m * 4 + kAdjPadBytes));
    RTG_CUDA(ctx, cudaMemsetAsync((char *)c.adj + m * 4, 0, kAdjPadBytes, ctx->stream));
    if (with_src) RTG_TRY(dev_alloc(ctx, (void **)&c.src, m * 4));
    if (m == 0) {
        RTG_CUDA(ctx, cudaMemsetAsync(c.off, 0, (n + 1ull) * 8, ctx->stream));
    } else {
        k_csr_fill<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(keys, m, B, c.adj, c.src);
        k_row_offsets<<<grid_for(ctx, n + 1ull), kThreads, 0, ctx->stream>>>(keys, m, B, n, c.off);
        ctx->launches += 2;
        RTG_CUDA(ctx, cudaGetLastError());
    }
    unsigned long long *w = ctx->d_scalars;
    RTG_CUDA(ctx, cudaMemsetAsync(w, 0, 16, ctx->stream));
    k_stats<<<grid_for(ctx, m + n), kThreads, 0, ctx->stream>>>(c.off, c.adj, c.src, m, n, w,
                                                                 (unsigned int *)(w + 1));
    ctx->launches++;
    RTG_CUDA(ctx, cudaGetLastError());
    unsigned long long h[2];
    RTG_CUDA(ctx, cudaMemcpyAsync(h, w, 16, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    c.work_elems = h[0];
    c.max_deg = (uint32_t)h[1];
    c.built = true;
    return RTG_OK;
}

// Simple undirected edge keys (sorted, unique, no self loops). Returns the count in *mu.
rtg_status simple_keys(rtg_ctx *ctx, rtg_graph *g, uint32_t maxid, int B, uint64_t *k0,
                       uint64_t *k1, uint64_t **ukeys, uint64_t *mu) {
    uint64_t m = g->m_input;
    uint64_t sentinel = (uint64_t)(maxid + 1ull) << B;
    int end_bit = std::min(64, B + bits_for(maxid + 1ull));
    k_canon_keys<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(g->d_src, g->d_dst, m, B,
                                                                  sentinel, k0);
    ctx->launches++;
    RTG_CUDA(ctx, cudaGetLastError());
    cub::DoubleBuffer<uint64_t> db(k0, k1);
    RTG_TRY(radix_sort(ctx, db, m, end_bit));
    uint64_t *sorted = db.Current();
    uint64_t *uniq = db.Alternate();
    int64_t *d_num = (int64_t *)(ctx->d_scalars + 4);
    size_t bytes = 0;
    RTG_CUDA(ctx, cub::DeviceSelect::Unique(nullptr, bytes, sorted, uniq, d_num, (int64_t)m,
                                            ctx->stream));
    void *tmp = nullptr;
    RTG_TRY(scratch(ctx, 0, bytes, &tmp));
    RTG_CUDA(ctx, cub::DeviceSelect::Unique(tmp, bytes, sorted, uniq, d_num, (int64_t)m,
                                            ctx->stream));
    ctx->launches += 2;
    int64_t nu = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&nu, d_num, 8, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nu > 0) {
        uint64_t last = 0;
        RTG_CUDA(ctx, cudaMemcpyAsync(&last, uniq + nu - 1, 8, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (last == sentinel) --nu;
    }
    *ukeys = uniq;
    *mu = (uint64_t)nu;
    return RTG_OK;
}

// ---- counting form: rank relabel + in-edge suffix ranges
__global__ void k_total_degree(const uint64_t *off, const uint32_t *adj, uint64_t m, uint32_t n,
                               uint32_t *tdeg) {
    GRID_STRIDE(v, (uint64_t)n) { atomicAdd(&tdeg[v], (uint32_t)(off[v + 1] - off[v])); }
    GRID_STRIDE(e, m) { atomicAdd(&tdeg[adj[e]], 1u); }
}

__global__ void k_rank_keys(const uint32_t *tdeg, uint32_t n, int B, uint64_t *keys) {
    GRID_STRIDE(v, (uint64_t)n) { keys[v] = ((uint64_t)tdeg[v] << B) | v; }
}

__global__ void k_rank_scatter(const uint64_t *sorted, uint32_t n, int B, uint32_t *rank) {
    const uint64_t mask = (1ull << B) - 1;
    GRID_STRIDE(i, (uint64_t)n) { rank[sorted[i] & mask] = (uint32_t)i; }
}

// edge keys in rank ids, lower rank first; self loops become the sentinel (n << B)
__global__ void k_rank_edge_keys(const uint32_t *src, const uint32_t *adj, uint64_t m,
                                 const uint32_t *rank, int B, uint64_t sentinel, uint64_t *keys) {
    GRID_STRIDE(e, m) {
        uint32_t a = rank[src[e]], b = rank[adj[e]];
        keys[e] = (a == b) ? sentinel : (((uint64_t)min(a, b) << B) | max(a, b));
    }
}

// degrees on the raw edge list (duplicates and self loops included), counted on every
// stride-th edge: the ranking only has to be a total order close to the degree order
__global__ void k_degree_raw(const uint32_t *s, const uint32_t *d, uint64_t m, uint32_t stride,
                             uint32_t *deg) {
    GRID_STRIDE(i, (m + stride - 1) / stride) {
        atomicAdd(&deg[s[i * stride]], 1u);
        atomicAdd(&deg[d[i * stride]], 1u);
    }
}

// Edge lists of kDegreeSampleFrom edges or more rank by a 1-in-kDegreeSample sample of the
// raw degrees (constants in internal.h): an eighth of the atomics (whose hub contention
// made this pass 0.36 ms of the R-MAT-21 build at 1 in 4), hubs ordered the same (their
// counts are large), and the count is exact for any total order. On R-MAT-21, 1 in 8
// against 1 in 4: build 0.12 ms shorter, count unchanged within 0.3 %; 1 in 16 saved
// 0.07 ms more but cost 0.7 % of the count.

// degrees of the simple graph from its sorted canonical keys: the row length of the
// smaller endpoint (offsets of the sorted keys, no atomics on the hub rows) ...
__global__ void k_degree_lo(const uint64_t *off_lo, uint32_t n, uint32_t *deg) {
    GRID_STRIDE(v, (uint64_t)n) { deg[v] = (uint32_t)(off_lo[v + 1] - off_lo[v]); }
}
// ... plus one per key for the larger endpoint
__global__ void k_degree_hi(const uint64_t *keys, uint64_t m, int B, uint32_t *deg) {
    const uint64_t lo_mask = (1ull << B) - 1;
    GRID_STRIDE(i, m) { atomicAdd(&deg[keys[i] & lo_mask], 1u); }
}

// rank edge keys straight from canonical (min id, max id) keys of the simple graph
__global__ void k_rank_canon_keys(const uint64_t *ukeys, uint64_t m, int B, const uint32_t *rank,
                                  uint64_t *keys) {
    const uint64_t lo_mask = (1ull << B) - 1;
    GRID_STRIDE(i, m) {
        const uint64_t k = ukeys[i];
        const uint32_t a = rank[k >> B], b = rank[k & lo_mask];
        keys[i] = ((uint64_t)min(a, b) << B) | max(a, b);
    }
}

// in-edges: (head rank, position) pairs, grouped by a stable 32-bit key sort so positions
// stay ascending within a head. The row end of every position replaces its row id in
// src_r here, where the rows are read in order, so that the fill after the sort reads one
// scattered word per in-edge instead of two dependent ones. Four in-edges per thread, a
// grid's width apart, so that their row-end gathers overlap.
__global__ void k_in_pairs(const uint32_t *__restrict__ adj_r, uint64_t m,
                           const uint64_t *__restrict__ off_r, uint32_t *__restrict__ keys,
                           uint32_t *__restrict__ pos, uint32_t *__restrict__ src_r) {
    const uint64_t T = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t e0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e0 < m; e0 += 4 * T) {
        uint32_t w[4], r[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint64_t e = e0 + k * T;
            w[k] = e < m ? adj_r[e] : 0u;
            r[k] = e < m ? src_r[e] : 0u;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) r[k] = (uint32_t)__ldg(off_r + r[k] + 1);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint64_t e = e0 + k * T;
            if (e < m) {
                keys[e] = w[k];
                pos[e] = (uint32_t)e;
                src_r[e] = r[k];
            }
        }
    }
}

// rng[i] = [e + 1, end of e's row) for the in-edge at position e (rend: row end per position).
// One gather per thread in flight: four per thread was 0.12 ms slower on 31.8M in-edges
// (their random reads of the 127 MB row-end array hit L2 less often).
__global__ void k_in_fill(const uint32_t *pos, uint64_t m, const uint32_t *rend, uint2 *rng) {
    GRID_STRIDE(i, m) {
        const uint32_t e = pos[i];
        rng[i] = make_uint2(e + 1, rend[e]);
    }
}

// row offsets of sorted 32-bit keys: off[x] = first i with keys[i] >= x
__global__ void k_row_offsets32(const uint32_t *keys, uint64_t m, uint32_t n, uint64_t *off) {
    GRID_STRIDE(x, (uint64_t)n + 1) {
        uint64_t lo = 0, hi = m;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (keys[mid] < x) lo = mid + 1;
            else hi = mid;
        }
        off[x] = lo;
    }
}

rtg_status in_edge_tail(rtg_ctx *ctx, CountCsr &cc, uint64_t *ek, uint64_t *other, uint64_t mr,
                        uint32_t n, int B, uint32_t *src_r, bool stats,
                        uint64_t m_in = CountCsr::kAllInEdges);

__global__ void k_iota32(uint32_t *p, uint64_t n) {
    GRID_STRIDE(i, n) { p[i] = (uint32_t)i; }
}

// rank[ids[i]] = i for the ids in rank order
__global__ void k_rank_scatter32(const uint32_t *ids, uint32_t n, uint32_t *rank) {
    GRID_STRIDE(i, (uint64_t)n) { rank[ids[i]] = (uint32_t)i; }
}

// Stable sort of 32-bit (key, value) pairs over the low `bits` key bits.
rtg_status sort_pairs32(rtg_ctx *ctx, cub::DoubleBuffer<uint32_t> &k,
                        cub::DoubleBuffer<uint32_t> &v, uint64_t m, int bits) {
    if (m < 2) return RTG_OK;
    size_t bytes = 0;
    RTG_CUDA(ctx, cub::DeviceRadixSort::SortPairs(nullptr, bytes, k, v, (int64_t)m, 0, bits,
                                                  ctx->stream));
    void *tmp = nullptr;
    RTG_TRY(scratch(ctx, 0, bytes, &tmp));
    RTG_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, bytes, k, v, (int64_t)m, 0, bits,
                                                  ctx->stream));
    ctx->launches += (bits + 7) / 8 + 1;
    return RTG_OK;
}

// (higher rank, lower rank) of every input edge; a self loop gets (n, n), which sorts last
__global__ void k_rank_pairs(const uint32_t *s, const uint32_t *d, uint64_t m,
                             const uint32_t *rank, uint32_t n, uint32_t *hi, uint32_t *lo) {
    GRID_STRIDE(i, m) {
        const uint32_t a = rank[s[i]], b = rank[d[i]];
        hi[i] = a == b ? n : max(a, b);
        lo[i] = a == b ? n : min(a, b);
    }
}

// The same four edges at a time with 16-byte loads and stores (every array 16-byte
// aligned); the last m % 4 edges are left to k_rank_pairs.
__global__ void k_rank_pairs4(const uint4 *__restrict__ s, const uint4 *__restrict__ d,
                              uint64_t m4, const uint32_t *__restrict__ rank, uint32_t n,
                              uint4 *hi, uint4 *lo) {
    GRID_STRIDE(q, m4) {
        const uint4 a = s[q], b = d[q];
        const uint32_t a0 = __ldg(rank + a.x), a1 = __ldg(rank + a.y), a2 = __ldg(rank + a.z),
                       a3 = __ldg(rank + a.w);
        const uint32_t b0 = __ldg(rank + b.x), b1 = __ldg(rank + b.y), b2 = __ldg(rank + b.z),
                       b3 = __ldg(rank + b.w);
        hi[q] = make_uint4(a0 == b0 ? n : max(a0, b0), a1 == b1 ? n : max(a1, b1),
                           a2 == b2 ? n : max(a2, b2), a3 == b3 ? n : max(a3, b3));
        lo[q] = make_uint4(a0 == b0 ? n : min(a0, b0), a1 == b1 ? n : min(a1, b1),
                           a2 == b2 ? n : min(a2, b2), a3 == b3 ? n : min(a3, b3));
    }
}

// After the unique pass over the sorted (lower, higher) pairs (*num runs kept): the rows end
// before the (n, n) entry the self loops leave last, if any; *mr = the row entries, and the
// kAdjPadBytes after them are zeroed.
__global__ void k_unique_rows_end(const int64_t *num, const uint32_t *src, uint32_t *adj,
                                  uint32_t n, uint32_t *mr) {
    const int64_t k = *num;
    const uint64_t r = (k > 0 && src[k - 1] == n) ? (uint64_t)(k - 1) : (uint64_t)k;
    for (uint32_t q = threadIdx.x; q < kAdjPadBytes / 4; q += blockDim.x) adj[r + q] = 0u;
    if (threadIdx.x == 0) *mr = (uint32_t)r;
}

// Rows, in-edge suffix ranges and stats of the counting form from its rank edge keys
// (sorted, unique, mr of them) in ek; `other` is a key buffer of mr entries and src_r one
// of mr words.
rtg_status count_tail(rtg_ctx *ctx, CountCsr &cc, uint64_t *ek, uint64_t *other, uint64_t mr,
                      uint32_t n, int B, uint32_t *src_r, bool stats = true) {
    cc.m = mr;
    if (mr == 0) {
        RTG_CUDA(ctx, cudaMemsetAsync(cc.off, 0, (n + 1ull) * 8, ctx->stream));
        RTG_CUDA(ctx, cudaMemsetAsync(cc.in_off, 0, (n + 1ull) * 8, ctx->stream));
        cc.built = true;
        return RTG_OK;
    }
    k_csr_fill<<<grid_for(ctx, mr), kThreads, 0, ctx->stream>>>(ek, mr, B, cc.adj, src_r);
    k_row_offsets<<<grid_for(ctx, n + 1ull), kThreads, 0, ctx->stream>>>(ek, mr, B, n, cc.off);
    ctx->launches += 2;
    // ek is free once rows are filled
    return in_edge_tail(ctx, cc, ek, other, mr, n, B, src_r, stats);
}

// In-edge suffix ranges and stats of a counting form whose rows (cc.off, cc.adj, and the
// row of every position in src_r) are filled: ek and other are scratch of mr u64 each, for
// the pair sort that groups the in-edges by head. With m_in < mr only the in-edges at row
// positions below m_in (the rows of the first sources) are grouped.
rtg_status in_edge_tail(rtg_ctx *ctx, CountCsr &cc, uint64_t *ek, uint64_t *other, uint64_t mr,
                        uint32_t n, int B, uint32_t *src_r, bool stats, uint64_t m_in) {
    uint32_t *ka = reinterpret_cast<uint32_t *>(other), *pa = ka + mr;
    uint32_t *kb = reinterpret_cast<uint32_t *>(ek), *pb = kb + mr;
    cc.m_in = m_in < mr ? m_in : CountCsr::kAllInEdges;
    const uint64_t mi = cc.inedges();
    if (mi == 0) {
        RTG_CUDA(ctx, cudaMemsetAsync(cc.in_off, 0, (n + 1ull) * 8, ctx->stream));
    } else {
        k_in_pairs<<<grid_for(ctx, mi), kThreads, 0, ctx->stream>>>(cc.adj, mi, cc.off, ka, pa,
                                                                    src_r);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        cub::DoubleBuffer<uint32_t> dk(ka, kb), dv(pa, pb);
        size_t bytes = 0;
        RTG_CUDA(ctx, cub::DeviceRadixSort::SortPairs(nullptr, bytes, dk, dv, (int64_t)mi, 0, B,
                                                      ctx->stream));
        void *tmp = nullptr;
        RTG_TRY(scratch(ctx, 0, bytes, &tmp));
        RTG_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, bytes, dk, dv, (int64_t)mi, 0, B,
                                                      ctx->stream));
        ctx->launches += (B + 7) / 8 + 1;
        k_in_fill<<<grid_for(ctx, mi), kThreads, 0, ctx->stream>>>(dv.Current(), mi, src_r,
                                                                    cc.in_rng);
        k_row_offsets32<<<grid_for(ctx, n + 1ull), kThreads, 0, ctx->stream>>>(dk.Current(), mi, n,
                                                                                cc.in_off);
        ctx->launches += 2;
    }
    RTG_CUDA(ctx, cudaGetLastError());
    if (!stats) {  // max_deg stays 0: the one-shot count does not read it
        cc.max_deg = 0;
        cc.built = true;
        return RTG_OK;
    }
    unsigned long long *w = ctx->d_scalars;
    RTG_CUDA(ctx, cudaMemsetAsync(w, 0, 24, ctx->stream));
    k_stats<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(cc.off, cc.adj, nullptr, mr, n, w,
                                                             (unsigned int *)(w + 1));
    enqueue_core_auto(ctx->stream, cc, w + 2);
    ctx->launches += 2;
    RTG_CUDA(ctx, cudaGetLastError());
    unsigned long long h[3];
    RTG_CUDA(ctx, cudaMemcpyAsync(h, w, 24, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cc.max_deg = (uint32_t)h[1];
    cc.core_auto = (int64_t)h[2];
    cc.built = true;
    return RTG_OK;
}

rtg_status count_alloc(rtg_ctx *ctx, CountCsr &cc, uint32_t n, uint64_t m) {
    count_csr_free(cc);
    cc.n = n;
    cc.core_auto = -1;
    cc.m_in = CountCsr::kAllInEdges;
    RTG_TRY(dev_alloc(ctx, (void **)&cc.off, (n + 1ull) * 8));
    RTG_TRY(dev_alloc(ctx, (void **)&cc.in_off, (n + 1ull) * 8));
    RTG_TRY(dev_alloc(ctx, (void **)&cc.adj, m * 4 + kAdjPadBytes));
    RTG_TRY(dev_alloc(ctx, (void **)&cc.in_rng, m * 8 + 16));
    RTG_CUDA(ctx, cudaMemsetAsync((char *)cc.adj + m * 4, 0, kAdjPadBytes, ctx->stream));
    return RTG_OK;
}

// The same arrays carved from the context's scratch slot kCountScratch (a one-shot count
// whose graph dies with the call; the caller detaches them before destroying the graph).
constexpr int kCountScratch = 7;

rtg_status count_alloc_scratch(rtg_ctx *ctx, CountCsr &cc, uint32_t n, uint64_t m) {
    auto up = [](uint64_t b) { return (b + 255) & ~255ull; };
    const uint64_t b_off = up((n + 1ull) * 8), b_adj = up(m * 4 + kAdjPadBytes),
                   b_rng = up(m * 8 + 16);
    void *p = nullptr;
    RTG_TRY(scratch(ctx, kCountScratch, 2 * b_off + b_adj + b_rng, &p));
    char *c = static_cast<char *>(p);
    cc.n = n;
    cc.core_auto = -1;
    cc.m_in = CountCsr::kAllInEdges;
    cc.off = reinterpret_cast<uint64_t *>(c);
    cc.in_off = reinterpret_cast<uint64_t *>(c + b_off);
    cc.adj = reinterpret_cast<uint32_t *>(c + 2 * b_off);
    cc.in_rng = reinterpret_cast<uint2 *>(c + 2 * b_off + b_adj);
    RTG_CUDA(ctx, cudaMemsetAsync((char *)cc.adj + m * 4, 0, kAdjPadBytes, ctx->stream));
    return RTG_OK;
}

}  // namespace

rtg_status csr_build_count(rtg_ctx *ctx, const Csr &c, CountCsr &cc) {
    const uint64_t m = c.m;
    const uint32_t n = c.n;
    RTG_TRY(count_alloc(ctx, cc, n, m));
    if (m == 0 || n == 0) {
        RTG_CUDA(ctx, cudaMemsetAsync(cc.off, 0, (n + 1ull) * 8, ctx->stream));
        RTG_CUDA(ctx, cudaMemsetAsync(cc.in_off, 0, (n + 1ull) * 8, ctx->stream));
        cc.m = 0;
        cc.built = true;
        return RTG_OK;
    }
    Buffers buf{ctx, {}};
    const int B = bits_for(n);
    uint32_t *tdeg, *rank, *src_r;
    uint64_t *k0, *k1;
    RTG_TRY(buf.alloc(&tdeg, n));
    RTG_TRY(buf.alloc(&rank, n));
    RTG_TRY(buf.alloc(&src_r, m));
    RTG_TRY(buf.alloc(&k0, std::max<uint64_t>(m, n)));
    RTG_TRY(buf.alloc(&k1, std::max<uint64_t>(m, n)));
    RTG_CUDA(ctx, cudaMemsetAsync(tdeg, 0, n * 4ull, ctx->stream));
    k_total_degree<<<grid_for(ctx, m + n), kThreads, 0, ctx->stream>>>(c.off, c.adj, m, n, tdeg);
    k_rank_keys<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(tdeg, n, B, k0);
    ctx->launches += 2;
    RTG_CUDA(ctx, cudaGetLastError());
    cub::DoubleBuffer<uint64_t> dr(k0, k1);
    RTG_TRY(radix_sort(ctx, dr, n, std::min(64, B + 32)));
    k_rank_scatter<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(dr.Current(), n, B, rank);
    const uint64_t sentinel = (uint64_t)n << B;
    k_rank_edge_keys<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(c.src, c.adj, m, rank, B,
                                                                      sentinel, k0);
    ctx->launches += 2;
    RTG_CUDA(ctx, cudaGetLastError());
    cub::DoubleBuffer<uint64_t> de(k0, k1);
    RTG_TRY(radix_sort(ctx, de, m, std::min(64, 2 * B)));
    // duplicates and self loops cannot occur in a CSR built here; a caller-given CSR is
    // cleaned the same way
    int64_t *d_num = (int64_t *)(ctx->d_scalars + 4);
    size_t bytes = 0;
    RTG_CUDA(ctx, cub::DeviceSelect::Unique(nullptr, bytes, de.Current(), de.Alternate(), d_num,
                                            (int64_t)m, ctx->stream));
    void *tmp = nullptr;
    RTG_TRY(scratch(ctx, 0, bytes, &tmp));
    RTG_CUDA(ctx, cub::DeviceSelect::Unique(tmp, bytes, de.Current(), de.Alternate(), d_num,
                                            (int64_t)m, ctx->stream));
    ctx->launches += 2;
    int64_t mu = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&mu, d_num, 8, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint64_t *ek = de.Alternate(), *other = de.Current();
    if (mu > 0) {
        uint64_t last = 0;
        RTG_CUDA(ctx, cudaMemcpy(&last, ek + mu - 1, 8, cudaMemcpyDeviceToHost));
        if (last == sentinel) --mu;
    }
    return count_tail(ctx, cc, ek, other, (uint64_t)mu, n, B, src_r);
}

rtg_status build_count_direct(rtg_ctx *ctx, rtg_graph *g, bool in_scratch, bool raw_degree,
                              const EdgePrePass *pre) {
    const uint64_t m = g->m_input;
    tc_plan_free(g->plan_batched);
    tc_plan_free(g->plan_plain);
    tc_plan_free(g->plan_bucketed);
    g->plan_batched = g->plan_plain = g->plan_bucketed = nullptr;
    uint32_t maxid = 0;
    if (pre && raw_degree) {
        maxid = pre->maxid;
        if (m && maxid == kEmpty)
            return fail(ctx, RTG_ERR_INVALID_ARG, "vertex id 0xFFFFFFFF is reserved");
    } else if (m) {
        unsigned int *d_mx = (unsigned int *)ctx->d_scalars;
        RTG_CUDA(ctx, cudaMemsetAsync(d_mx, 0, 4, ctx->stream));
        k_max_id<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(g->d_src, g->d_dst, m, d_mx);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        RTG_TRY(read_u32(ctx, d_mx, &maxid));
        if (maxid == kEmpty)
            return fail(ctx, RTG_ERR_INVALID_ARG, "vertex id 0xFFFFFFFF is reserved");
    }
    // the arrays below are sized by the largest id, and the count takes fewer than 2^31
    // vertices: refuse larger ids before allocating for them
    if (m && maxid > 0x7FFFFFFEu)
        return fail(ctx, RTG_ERR_INVALID_ARG,
                    "vertex ids must be below 2^31 - 1 for a one-shot count (largest %u)", maxid);
    const uint32_t n = m ? maxid + 1 : 0;
    const int B = bits_for(maxid + 1ull);
    Buffers buf{ctx, {}};
    uint64_t *k0, *k1, *r0, *r1;
    uint32_t *deg, *rank, *src_r;
    const uint64_t cap = std::max<uint64_t>(m, 1);
    RTG_TRY(buf.alloc(&k0, cap));
    RTG_TRY(buf.alloc(&k1, cap));
    if (raw_degree && m) {
        // row positions and the row count below are 32-bit
        if (m > 0xFFFFFFFFull)
            return fail(ctx, RTG_ERR_INVALID_ARG, "one-shot count takes at most 2^32 - 1 edges");
        // ranks by degree in the input list (duplicates and self loops counted)
        RTG_TRY(buf.alloc(&rank, n));
        RTG_TRY(buf.alloc(&r0, n + 1ull));
        RTG_TRY(buf.alloc(&r1, n + 1ull));
        RTG_TRY(buf.alloc(&src_r, m));
        const uint32_t stride = m >= kDegreeSampleFrom ? kDegreeSample : 1u;
        if (pre && pre->deg_valid) {
            void *p = nullptr;
            RTG_TRY(scratch(ctx, kDegreeSlot, n * 4ull, &p));  // counted by the pre-pass
            deg = static_cast<uint32_t *>(p);
        } else {
            void *p = nullptr;
            RTG_TRY(scratch(ctx, kDegreeSlot, n * 4ull, &p));
            deg = static_cast<uint32_t *>(p);
            RTG_CUDA(ctx, cudaMemsetAsync(deg, 0, n * 4ull, ctx->stream));
            k_degree_raw<<<grid_for(ctx, m / stride), kThreads, 0, ctx->stream>>>(
                g->d_src, g->d_dst, m, stride, deg);
            ctx->launches++;
        }
        // (degree, id) order: a stable sort of the ids, ascending, by degree (32-bit pairs:
        // the order a sort of the 64-bit keys degree << B | id gives, at fewer bytes)
        uint32_t *ids = reinterpret_cast<uint32_t *>(r1), *ids_alt = ids + (n + 1ull);
        uint32_t *deg_alt = reinterpret_cast<uint32_t *>(r0);
        k_iota32<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(ids, n);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        cub::DoubleBuffer<uint32_t> dk(deg, deg_alt), dv(ids, ids_alt);
        RTG_TRY(sort_pairs32(ctx, dk, dv, n, 32));
        k_rank_scatter32<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(dv.Current(), n, rank);
        ctx->launches++;
        // (lower, higher) order from two stable sorts of 32-bit pairs, least significant key
        // first: by the higher endpoint, then by the lower one (a sort of the 64-bit keys
        // (lower << B | higher) orders them the same, at twice the bytes per pass); self
        // loops carry (n, n) and sort last, the copies of an edge end up adjacent
        uint32_t *A = reinterpret_cast<uint32_t *>(k0), *C = A + cap;
        uint32_t *Bv = reinterpret_cast<uint32_t *>(k1), *D = Bv + cap;
        const bool vec = ((reinterpret_cast<uintptr_t>(g->d_src) | reinterpret_cast<uintptr_t>(g->d_dst) |
                           reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(Bv)) & 15u) == 0;
        const uint64_t m4 = vec ? m / 4 : 0;
        if (m4) {
            k_rank_pairs4<<<grid_for(ctx, m4), kThreads, 0, ctx->stream>>>(
                reinterpret_cast<const uint4 *>(g->d_src), reinterpret_cast<const uint4 *>(g->d_dst),
                m4, rank, n, reinterpret_cast<uint4 *>(A), reinterpret_cast<uint4 *>(Bv));
            ctx->launches++;
        }
        if (m > 4 * m4) {
            k_rank_pairs<<<grid_for(ctx, m - 4 * m4), kThreads, 0, ctx->stream>>>(
                g->d_src + 4 * m4, g->d_dst + 4 * m4, m - 4 * m4, rank, n, A + 4 * m4,
                Bv + 4 * m4);
            ctx->launches++;
        }
        RTG_CUDA(ctx, cudaGetLastError());
        cub::DoubleBuffer<uint32_t> kh(A, C), vl(Bv, D);
        RTG_TRY(sort_pairs32(ctx, kh, vl, m, B));
        cub::DoubleBuffer<uint32_t> kl(vl.Current(), vl.Alternate()), vh(kh.Current(), kh.Alternate());
        RTG_TRY(sort_pairs32(ctx, kl, vh, m, B));
        const uint32_t *lo = kl.Current(), *hi = vh.Current();
        // the rows are sized for every input edge (copies included) and trimmed to the
        // unique ones below
        RTG_TRY(in_scratch ? count_alloc_scratch(ctx, g->cnt, n, m)
                           : count_alloc(ctx, g->cnt, n, m));
        g->orient = RTG_ORIENT_DEGREE;
        CountCsr &cc = g->cnt;
        // the copies of an edge are adjacent: one pass keeps the first pair of every run as
        // a row entry (src = lower, adj = higher); the self loops' (n, n) pairs sort last
        // and leave one entry there, which k_unique_rows_end drops
        int64_t *d_num = reinterpret_cast<int64_t *>(ctx->d_scalars + 4);
        uint32_t *d_mr = reinterpret_cast<uint32_t *>(ctx->d_scalars + 12);
        auto pin = thrust::make_zip_iterator(lo, hi);
        auto pout = thrust::make_zip_iterator(src_r, cc.adj);
        size_t ubytes = 0;
        RTG_CUDA(ctx, cub::DeviceSelect::Unique(nullptr, ubytes, pin, pout, d_num, (int64_t)m,
                                                ctx->stream));
        void *utmp = nullptr;
        RTG_TRY(scratch(ctx, 0, ubytes, &utmp));
        RTG_CUDA(ctx, cub::DeviceSelect::Unique(utmp, ubytes, pin, pout, d_num, (int64_t)m,
                                                ctx->stream));
        k_unique_rows_end<<<1, 32, 0, ctx->stream>>>(d_num, src_r, cc.adj, n, d_mr);
        ctx->launches += 3;
        RTG_CUDA(ctx, cudaGetLastError());
        uint32_t mr = 0;
        RTG_TRY(read_u32(ctx, d_mr, &mr));
        cc.m = mr;
        k_row_offsets32<<<grid_for(ctx, n + 1ull), kThreads, 0, ctx->stream>>>(src_r, mr, n,
                                                                                cc.off);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        if (mr == 0) {
            RTG_CUDA(ctx, cudaMemsetAsync(cc.in_off, 0, (n + 1ull) * 8, ctx->stream));
            cc.built = true;
            return RTG_OK;
        }
        // the sorted pairs are dead once the rows are filled: their buffers hold the in-edge
        // pair sort. A one-shot count's form dies with the call and is counted with the
        // context's core setting: the in-edges whose source lies in that dense core are never
        // read (the core count takes them from its bit matrix), so only the rows below the
        // core get in-edges (R-MAT-21: 70 % of them, 0.3 ms less).
        uint64_t m_in = CountCsr::kAllInEdges;
        if (in_scratch) {
            unsigned long long *w = ctx->d_scalars + 14, h[2] = {0, 0};
            enqueue_core_choice(ctx->stream, cc, ctx->cfg.tc_core_ranks, w);
            ctx->launches++;
            RTG_CUDA(ctx, cudaGetLastError());
            RTG_CUDA(ctx, cudaMemcpyAsync(h, w, 16, cudaMemcpyDeviceToHost, ctx->stream));
            RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            if (ctx->cfg.tc_core_ranks == 0) cc.core_auto = (int64_t)h[0];
            if (h[0]) m_in = h[1];
        }
        return in_edge_tail(ctx, cc, k0, k1, mr, n, B, src_r, !in_scratch, m_in);
    }
    uint64_t *ukeys = k0;
    uint64_t mu = 0;
    if (m) RTG_TRY(simple_keys(ctx, g, maxid, B, k0, k1, &ukeys, &mu));
    RTG_TRY(in_scratch ? count_alloc_scratch(ctx, g->cnt, n, mu) : count_alloc(ctx, g->cnt, n, mu));
    if (mu == 0) return count_tail(ctx, g->cnt, nullptr, nullptr, 0, n, B, nullptr);
    RTG_TRY(buf.alloc(&deg, n));
    RTG_TRY(buf.alloc(&rank, n));
    RTG_TRY(buf.alloc(&r0, n + 1ull));
    RTG_TRY(buf.alloc(&r1, n + 1ull));
    RTG_TRY(buf.alloc(&src_r, mu));
    // (degree, id) ranks: the degree order of the oriented CSR. The keys are sorted by
    // their smaller endpoint, so its share of the degree is a row length (r0 holds the
    // row offsets for a moment); the larger endpoint's share is counted with atomics.
    k_row_offsets<<<grid_for(ctx, n + 1ull), kThreads, 0, ctx->stream>>>(ukeys, mu, B, n, r0);
    k_degree_lo<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(r0, n, deg);
    k_degree_hi<<<grid_for(ctx, mu), kThreads, 0, ctx->stream>>>(ukeys, mu, B, deg);
    k_rank_keys<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(deg, n, B, r0);
    ctx->launches += 4;
    RTG_CUDA(ctx, cudaGetLastError());
    cub::DoubleBuffer<uint64_t> dr(r0, r1);
    RTG_TRY(radix_sort(ctx, dr, n, std::min(64, B + 32)));
    k_rank_scatter<<<grid_for(ctx, n), kThreads, 0, ctx->stream>>>(dr.Current(), n, B, rank);
    uint64_t *other = (ukeys == k0) ? k1 : k0;
    k_rank_canon_keys<<<grid_for(ctx, mu), kThreads, 0, ctx->stream>>>(ukeys, mu, B, rank, other);
    ctx->launches += 2;
    RTG_CUDA(ctx, cudaGetLastError());
    cub::DoubleBuffer<uint64_t> de(other, ukeys);
    RTG_TRY(radix_sort(ctx, de, mu, std::min(64, 2 * B)));
    g->orient = RTG_ORIENT_DEGREE;
    return count_tail(ctx, g->cnt, de.Current(), de.Alternate(), mu, n, B, src_r);
}

rtg_status build_csr(rtg_ctx *ctx, rtg_graph *g, rtg_orient orient) {
    uint64_t m = g->m_input;
    Buffers buf{ctx, {}};
    // largest id
    uint32_t maxid = 0;
    if (m) {
        unsigned int *d_mx = (unsigned int *)ctx->d_scalars;
        RTG_CUDA(ctx, cudaMemsetAsync(d_mx, 0, 4, ctx->stream));
        k_max_id<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(g->d_src, g->d_dst, m, d_mx);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        RTG_TRY(read_u32(ctx, d_mx, &maxid));
        if (maxid == kEmpty)
            return fail(ctx, RTG_ERR_INVALID_ARG, "vertex id 0xFFFFFFFF is reserved");
    }

    if (orient == RTG_ORIENT_DEGREE_RAW_REF) {
        if (maxid > 0x7FFFFFFEu)
            return fail(ctx, RTG_ERR_INVALID_ARG, "ids must fit int32 in reference mode");
        if (m == 0) {
            RTG_TRY(fill_csr(ctx, nullptr, 0, 1, 0, true, g->ori));
            g->orient = orient;
            return RTG_OK;
        }
        uint32_t *used, *rank, *s2, *d2, *deg, *removes;
        RTG_TRY(buf.alloc(&used, maxid + 1ull));
        RTG_TRY(buf.alloc(&rank, maxid + 1ull));
        RTG_CUDA(ctx, cudaMemsetAsync(used, 0, (maxid + 1ull) * 4, ctx->stream));
        k_mark_used<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(g->d_src, g->d_dst, m, used);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        RTG_TRY(inclusive_sum(ctx, used, rank, maxid + 1ull));
        uint32_t n_used = 0;
        RTG_TRY(read_u32(ctx, rank + maxid, &n_used));
        RTG_TRY(buf.alloc(&s2, m));
        RTG_TRY(buf.alloc(&d2, m));
        RTG_TRY(buf.alloc(&deg, n_used));
        RTG_TRY(buf.alloc(&removes, n_used));
        RTG_CUDA(ctx, cudaMemsetAsync(deg, 0, n_used * 4ull, ctx->stream));
        k_relabel_raw_degree<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(
            g->d_src, g->d_dst, m, rank, s2, d2, deg);
        ctx->launches++;
        k_flag_low_degree<<<grid_for(ctx, n_used), kThreads, 0, ctx->stream>>>(deg, n_used, used);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        RTG_TRY(inclusive_sum(ctx, used, removes, (uint64_t)n_used));
        uint32_t removed = 0;
        RTG_TRY(read_u32(ctx, removes + n_used - 1, &removed));
        uint32_t n_ref = n_used - removed;
        int B = bits_for(std::max<uint64_t>(n_ref, 1));
        uint64_t sentinel = (uint64_t)(n_ref + 1ull) << B;
        // n_ref may be 0; sentinel hi = n_ref + 1 must still exceed every kept id
        int end_bit = std::min(64, B + bits_for(n_ref + 1ull));
        uint64_t *k0, *k1;
        RTG_TRY(buf.alloc(&k0, m));
        RTG_TRY(buf.alloc(&k1, m));
        k_ref_orient_keys<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(s2, d2, m, deg, removes,
                                                                           B, sentinel, k0);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        cub::DoubleBuffer<uint64_t> db(k0, k1);
        RTG_TRY(radix_sort(ctx, db, m, end_bit));
        uint8_t *flags;
        RTG_TRY(buf.alloc(&flags, m));
        k_ref_keep_flags<<<grid_for(ctx, m), kThreads, 0, ctx->stream>>>(db.Current(), m, B,
                                                                          sentinel, flags);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        int64_t *d_num = (int64_t *)(ctx->d_scalars + 4);
        size_t bytes = 0;
        RTG_CUDA(ctx, cub::DeviceSelect::Flagged(nullptr, bytes, db.Current(), flags,
                                                 db.Alternate(), d_num, (int64_t)m, ctx->stream));
        void *tmp = nullptr;
        RTG_TRY(scratch(ctx, 0, bytes, &tmp));
        RTG_CUDA(ctx, cub::DeviceSelect::Flagged(tmp, bytes, db.Current(), flags, db.Alternate(),
                                                 d_num, (int64_t)m, ctx->stream));
        ctx->launches += 2;
        int64_t mk = 0;
        RTG_CUDA(ctx, cudaMemcpyAsync(&mk, d_num, 8, cudaMemcpyDeviceToHost, ctx->stream));
        RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        RTG_TRY(fill_csr(ctx, db.Alternate(), (uint64_t)mk, B, n_ref, true, g->ori));
        g->orient = orient;
        return RTG_OK;
    }

    int B = bits_for(maxid + 1ull);
    uint32_t n = m ? maxid + 1 : 0;
    uint64_t *k0 = nullptr, *k1 = nullptr;
    uint64_t cap = std::max<uint64_t>(m, 1);
    if (orient == RTG_ORIENT_SYMMETRIC) cap = std::max<uint64_t>(2 * m, 1);
    RTG_TRY(buf.alloc(&k0, cap));
    RTG_TRY(buf.alloc(&k1, cap));
    uint64_t *ukeys = k0;
    uint64_t mu = 0;
    if (m) RTG_TRY(simple_keys(ctx, g, maxid, B, k0, k1, &ukeys, &mu));
    int end_bit = std::min(64, B + bits_for(maxid + 1ull));

    if (orient == RTG_ORIENT_SYMMETRIC) {
        uint64_t *other = (ukeys == k0) ? k1 : k0;
        if (mu) {
            k_sym_keys<<<grid_for(ctx, mu), kThreads, 0, ctx->stream>>>(ukeys, mu, B, other);
            ctx->launches++;
            RTG_CUDA(ctx, cudaGetLastError());
        }
        cub::DoubleBuffer<uint64_t> db(other, ukeys);
        RTG_TRY(radix_sort(ctx, db, 2 * mu, end_bit));
        RTG_TRY(fill_csr(ctx, db.Current(), 2 * mu, B, n, false, g->sym));
        return RTG_OK;
    }

    // DEGREE
    uint32_t *deg = nullptr;
    RTG_TRY(buf.alloc(&deg, std::max<uint64_t>(n, 1)));
    if (n) RTG_CUDA(ctx, cudaMemsetAsync(deg, 0, n * 4ull, ctx->stream));
    if (mu) {
        k_degree_from_keys<<<grid_for(ctx, mu), kThreads, 0, ctx->stream>>>(ukeys, mu, B, deg);
        ctx->launches++;
        k_orient_keys<<<grid_for(ctx, mu), kThreads, 0, ctx->stream>>>(ukeys, mu, B, deg);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
    }
    uint64_t *other = (ukeys == k0) ? k1 : k0;
    cub::DoubleBuffer<uint64_t> db(ukeys, other);
    RTG_TRY(radix_sort(ctx, db, mu, end_bit));
    RTG_TRY(fill_csr(ctx, db.Current(), mu, B, n, true, g->ori));
    g->orient = orient;
    return RTG_OK;
}

}  // namespace rtg
