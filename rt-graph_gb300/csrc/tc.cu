// Triangle counting on the oriented CSR.
//
// Every triangle {u, v, w} of the simple graph appears exactly once as an oriented edge
// u->v with w in N+(u) ∩ N+(v); the count is the sum over oriented edges of
// |N+(u) ∩ N+(v)| (the reference computes the same sum edge by edge with binary searches,
// tc/bs_tc/bs_tc.cu:120-148, or from aggregated two-hop triples, bs_tc.cu:153-229).
//
// PLAIN   : classify edges into (family, size) buckets, copy the bucket sizes to the host,
//           scatter edge ids per bucket, then one grid-stride launch per bucket with one warp
//           per edge (merge family for balanced pairs, search family for skewed ones).
// BATCHED : runs on the counting form of the graph (vertices relabelled by (degree, id)
//           rank, edges low rank -> high rank, rows ascending). For an in-edge u->v only the
//           suffix of N+(u) after v can meet N+(v), so each in-edge is a ready-made element
//           range. A work item is (v, first in-edge): up to E in-edges of one vertex v, taken
//           by one warp from a device queue (persistent kernel, no block barriers). The warp
//           marks N+(v) in its shared-memory region: a bitmap over the top ranks of the graph
//           (from v + 1 when they fit, which holds for the high-rank v that carry almost all
//           of the work on power-law graphs), plus a small hash table for the few elements
//           of N+(v) below that window; out-lists with too many such elements fall back to
//           a tile merge. It then streams the suffixes of the item's in-edges 32 at a time:
//           whole 128-, 64- and 32-element units of each suffix with unchecked coalesced
//           loads, then the remainders (under 32 elements) of all 32 suffixes as one flat
//           sequence in full 32-lane windows, testing every element with one shared-memory
//           load.
//           Streamed elements: sum over u of d+(u)(d+(u)-1)/2, about a quarter of the
//           push-order work on power-law graphs.
//           Dense core: on power-law graphs most of those elements belong to in-edges whose
//           source sits among the top ranks (R-MAT scale 21: sources in the top 16,384 ranks
//           stream 51 % of them, in a core whose edge density is 4.9 %). A triangle whose
//           lowest vertex u lies in the top K ranks [c0, n) has all three vertices there,
//           so the core's share of the count is the sum over core edges u->v of
//           popcount(M[u] & M[v]), M the core's adjacency bit matrix (row r: N+(c0 + r) as
//           bits of ranks from c0). The count builds M (one warp per row), counts the core
//           edges word by word (k_tc_core: one warp per core row, the row staged in shared
//           memory, the word ranges of all its edges swept as one flat sequence), and
//           streams only the in-edges whose source lies below c0: the in-edges of a head
//           are ordered by source, so those are the first sdeg[v] of them. K is picked on
//           the device from the offsets when the items are built (the largest of 32768 ..
//           1024 top ranks with edge density >= 2.5 %, or none), or set by the schedule.
//           The items are built once per (graph, schedule); the count (counter resets,
//           core matrix, core count, the persistent kernel) is one CUDA graph, captured
//           once and replayed. uint64 totals: lane partials -> warp shuffle sum -> block
//           sum -> one atomicAdd per block.
#include <cub/cub.cuh>

#include <algorithm>
#include <mutex>

#include "internal.h"
#include "intersect.cuh"
#include "tma.cuh"

namespace rtg {

namespace {

constexpr uint32_t kDefaultItemEdges = 256;
constexpr uint32_t kDefaultBlockWarps = 8;
constexpr uint32_t kDefaultRegionWords = 1024;   // 4 KB per warp: bitmap of 32,768 ranks
constexpr uint32_t kPlainRatio = 16;    // long/short above this -> search family (PLAIN)
constexpr int kPlainBuckets = 6;         // 2 families x 3 size classes

__device__ __forceinline__ void block_add_total(unsigned long long v, unsigned long long *total,
                                                unsigned long long *red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum_u64(v);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned long long s = (lane < nw) ? red[lane] : 0ull;
        s = warp_sum_u64(s);
        if (lane == 0 && s) atomicAdd(total, s);
    }
}

// ------------------------------------------------------------------ PLAIN form

__global__ void k_plain_classify(const uint64_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                 const uint32_t *__restrict__ src, uint64_t m, uint8_t *bucket,
                                 unsigned long long *counts) {
    __shared__ unsigned int local[kPlainBuckets];
    if (threadIdx.x < kPlainBuckets) local[threadIdx.x] = 0;
    __syncthreads();
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t u = src[e], v = adj[e];
        uint32_t a = (uint32_t)(off[u + 1] - off[u]), b = (uint32_t)(off[v + 1] - off[v]);
        uint8_t id = 0xFF;
        if (a >= 2 && b >= 1) {
            uint32_t lo = min(a, b), hi = max(a, b);
            uint32_t fam = (hi > kPlainRatio * lo) ? 1u : 0u;
            uint32_t sum = a + b;
            uint32_t cls = sum <= 128 ? 0u : (sum <= 1024 ? 1u : 2u);
            id = (uint8_t)(fam * 3 + cls);
            atomicAdd(&local[id], 1u);
        }
        bucket[e] = id;
    }
    __syncthreads();
    if (threadIdx.x < kPlainBuckets && local[threadIdx.x])
        atomicAdd(&counts[threadIdx.x], (unsigned long long)local[threadIdx.x]);
}

// Scatter edge ids into their bucket lists. Positions are reserved per tile of
// blockDim * kScatterPerThread edges: shared-memory counters rank the tile's edges within
// each bucket, then one global atomicAdd per (tile, bucket) reserves their range.
constexpr int kScatterPerThread = 16;

__global__ void k_plain_scatter(const uint8_t *__restrict__ bucket, uint64_t m,
                                const unsigned long long *__restrict__ base,
                                unsigned long long *cursor, uint32_t *lists) {
    __shared__ unsigned int cnt[kPlainBuckets];
    __shared__ unsigned long long pos[kPlainBuckets];
    const uint64_t tile = (uint64_t)blockDim.x * kScatterPerThread;
    for (uint64_t t0 = blockIdx.x * tile; t0 < m; t0 += (uint64_t)gridDim.x * tile) {
        if (threadIdx.x < kPlainBuckets) cnt[threadIdx.x] = 0;
        __syncthreads();
        uint8_t id[kScatterPerThread];
        unsigned int rank[kScatterPerThread];
#pragma unroll
        for (int k = 0; k < kScatterPerThread; ++k) {
            const uint64_t e = t0 + (uint64_t)k * blockDim.x + threadIdx.x;
            id[k] = e < m ? bucket[e] : (uint8_t)0xFF;
            rank[k] = id[k] != 0xFF ? atomicAdd(&cnt[id[k]], 1u) : 0u;
        }
        __syncthreads();
        if (threadIdx.x < kPlainBuckets && cnt[threadIdx.x])
            pos[threadIdx.x] = base[threadIdx.x] +
                               atomicAdd(&cursor[threadIdx.x], (unsigned long long)cnt[threadIdx.x]);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kScatterPerThread; ++k) {
            const uint64_t e = t0 + (uint64_t)k * blockDim.x + threadIdx.x;
            if (id[k] != 0xFF) lists[pos[id[k]] + rank[k]] = (uint32_t)e;
        }
        __syncthreads();
    }
}

template <bool kSearch>
__global__ void __launch_bounds__(256) k_plain_edges(const uint64_t *__restrict__ off,
                                                    const uint32_t *__restrict__ adj,
                                                    const uint32_t *__restrict__ src,
                                                    const uint32_t *__restrict__ list, uint64_t ne,
                                                    unsigned long long *total) {
    __shared__ unsigned long long red[8];
    const int lane = threadIdx.x & 31;
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long cnt = 0;
    for (uint64_t k = warp; k < ne; k += nwarps) {
        uint32_t e = list[k];
        uint32_t u = src[e], v = adj[e];
        uint64_t ou = off[u], ov = off[v];
        uint32_t a = (uint32_t)(off[u + 1] - ou), b = (uint32_t)(off[v + 1] - ov);
        const uint32_t *A = adj + ou, *B = adj + ov;
        if (kSearch) {
            if (a <= b) cnt += warp_search_count(A, a, B, b, lane);
            else cnt += warp_search_count(B, b, A, a, lane);
        } else {
            cnt += warp_merge_count(A, a, B, b, lane);
        }
    }
    block_add_total(cnt, total, red);
}

// ---------------------------------------------------------------- BATCHED form

// acc (kAccWords u64 per count): [0] total, [1] item queue head, [2] number of items,
// [3..5] items per size bucket (BUCKETED), [6] core queue head, [8] core ranks K (0: no
// core), [9] c0 = n - K, [10] words per core matrix row, [11] off[c0] (the first adj index
// of a core row)
constexpr int kAccWords = 16;
constexpr int kAccCoreQ = 6, kAccCoreK = 8, kAccCoreC0 = 9, kAccCoreRw = 10, kAccCoreXc = 11;

// Core sizes the library picks from (largest first), and the edge density the core must
// reach (per mille of K (K - 1) / 2): the largest candidate at or above it. Cost measured on
// R-MAT scale 21 (edge factor 16, 16384 and 32768 core ranks): 4.8e-10 ms per streamed
// element, 3.8e-10 ms per swept matrix word. With those rates the best candidate is the
// largest of 2.5 % density or more on R-MAT scale 18, 20 and 21 (edge factor 16: 12288,
// 16384 and 24576 ranks) and within 2 % of the best at edge factor 8 (16384 for 12288); on
// Holme-Kim and Barabasi-Albert graphs of 2^20 vertices no core reaches 1.5 % and none would
// pay.
constexpr int kCoreCandidates = 11;
constexpr uint32_t kCoreMinDensityPerMille = 25;

// candidate i, largest first: 32768, 24576, 16384, 12288, ..., 1536, 1024
__host__ __device__ constexpr uint32_t core_candidate(int i) {
    return (i & 1) ? 24576u >> (i / 2) : 32768u >> (i / 2);
}

// The core count sweeps the matrix in groups of kCoreGroupWords words (16 bytes, one load per
// lane and position). Measured on R-MAT scale 21 with 16384 core ranks: 0.25-0.27 ms with
// 16-byte groups, 0.30 ms with 32-byte and 0.50 ms with 64-byte groups (a word range averages
// 17 groups of 4 words but most are short, and wider groups sweep more zero words), 0.50 ms
// with 4-byte positions (the per-position segment search then runs for every word).
constexpr uint32_t kCoreGroupWords = 4;
constexpr uint32_t kCoreVec = kCoreGroupWords / 4;

// words of a core matrix row for K ranks: a power of two of at least one group, so that a
// group's place within its row is its matrix group index masked
__host__ __device__ constexpr uint32_t core_row_words(uint32_t K) {
    uint32_t w = kCoreGroupWords;
    while (w * 32 < K) w <<= 1;
    return K ? w : 0u;
}

// The library's choice: the largest candidate whose m - off[n - K] core edges reach the
// density bar, 0 if none does (on the device, and on the host for forms read from a file).
__host__ __device__ uint32_t auto_core(const uint64_t *__restrict__ off, uint32_t n, uint64_t m) {
    for (int i = 0; i < kCoreCandidates; ++i) {
        const uint32_t c = core_candidate(i);
        if (c > n) continue;
        const uint64_t ce = m - off[n - c];
        if (1000ull * ce >= (uint64_t)kCoreMinDensityPerMille * c * (c - 1) / 2) return c;
    }
    return 0;
}

__global__ void k_core_auto(const uint64_t *__restrict__ off, uint32_t n, uint64_t m,
                            unsigned long long *out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *out = auto_core(off, n, m);
}

// out[0] = the core size of a schedule setting (as k_core_pick), out[1] = off[n - size]
__global__ void k_core_choice(const uint64_t *__restrict__ off, uint32_t n, uint64_t m,
                              uint32_t setting, unsigned long long *out) {
    if (blockIdx.x || threadIdx.x) return;
    const uint32_t K = setting == RTG_TC_CORE_NONE ? 0u
                       : setting                   ? min(setting, n)
                                                   : auto_core(off, n, m);
    out[0] = K;
    out[1] = off[n - K];
}

// The core size a schedule gives a counting form: RTG_TC_CORE_NONE -> 0, a forced size ->
// min(size, n), the library's choice -> the size cached when the form was built, or, for a
// form built without it (one-shot counts, cache files), the largest candidate that fits
// (the buffers' bound; the device picks the actual size).
uint32_t core_max_ranks(uint32_t forced, const CountCsr &c) {
    if (forced == RTG_TC_CORE_NONE) return 0;
    if (forced) return std::min(forced, c.n);
    if (c.core_auto >= 0) return (uint32_t)c.core_auto;
    for (int i = 0; i < kCoreCandidates; ++i)
        if (core_candidate(i) <= c.n) return core_candidate(i);
    return 0;
}

// The core of this count: `forced` ranks (RTG_TC_CORE_NONE: none), or with forced == 0 the
// library's choice.
__global__ void k_core_pick(const uint64_t *__restrict__ off, uint32_t n, uint64_t m,
                            uint32_t forced, unsigned long long *acc) {
    if (blockIdx.x || threadIdx.x) return;
    uint32_t K = 0;
    if (forced == RTG_TC_CORE_NONE) K = 0;
    else if (forced) K = min(forced, n);
    else K = auto_core(off, n, m);
    acc[kAccCoreK] = K;
    acc[kAccCoreC0] = n - K;
    acc[kAccCoreRw] = core_row_words(K);
    acc[kAccCoreXc] = off[n - K];
}

// Per vertex v: sdeg[v] = the in-edges streamed by the persistent kernel, those whose
// suffix range starts before the first core row (x < off[c0]); the in-edges of a head are
// ordered by source, and x grows with the source, so they are a prefix (binary search for
// heads in the core, all in-edges below it; an empty range at the end of a row may count as
// core, which drops nothing). Items per vertex: ceil(sdeg(v) / E) when v has out-neighbours.
__global__ void k_item_counts(const uint64_t *__restrict__ off,
                              const uint64_t *__restrict__ in_off,
                              const uint2 *__restrict__ in_rng, uint32_t n, uint32_t E,
                              const unsigned long long *acc, uint32_t *cnt, uint32_t *sdeg) {
    const uint32_t c0 = (uint32_t)acc[kAccCoreC0];
    const uint64_t xc = acc[kAccCoreXc];
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v <= n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t c = 0;
        if (v < n) {
            const uint32_t b = (uint32_t)(off[v + 1] - off[v]);
            const uint64_t k0 = in_off[v];
            const uint32_t indeg = (uint32_t)(in_off[v + 1] - k0);
            uint32_t sd = indeg;
            if (v >= c0 && indeg) {
                uint32_t lo = 0, hi = indeg;
                while (lo < hi) {
                    const uint32_t mid = lo + (hi - lo) / 2;
                    if (in_rng[k0 + mid].x < xc) lo = mid + 1;
                    else hi = mid;
                }
                sd = lo;
            }
            sdeg[v] = sd;
            c = (b >= 1 && sd >= 1) ? (sd + E - 1) / E : 0u;
        }
        cnt[v] = c;
    }
}

__global__ void k_item_fill(const uint64_t *__restrict__ off, const uint32_t *__restrict__ sdeg,
                            uint32_t n, uint32_t E, const uint32_t *__restrict__ base,
                            uint64_t *items, unsigned long long *acc) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t b = (uint32_t)(off[v + 1] - off[v]);
        uint32_t indeg = sdeg[v];
        if (b < 1 || indeg < 1) continue;
        // descending rank order: the many light items of low-rank vertices come last and
        // fill in behind the heavier ones (1.4 % shorter than ascending order on R-MAT-21)
        const uint32_t last = base[n] - 1 - base[v];
        uint32_t k = 0;
        for (uint32_t j = 0; j < indeg; j += E, ++k) items[last - k] = (v << 32) | j;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) acc[2] = base[n];
}

// BUCKETED form: the items sorted by the in-edges they hold (at most 32, at most 256, more)
// into kItemBuckets regions of cap entries; cnt[r] counts region r.
constexpr int kItemBuckets = 3;

__global__ void k_item_bucket(const uint64_t *__restrict__ items,
                              const unsigned long long *__restrict__ nitems,
                              const uint32_t *__restrict__ sdeg, uint32_t E, uint64_t cap,
                              uint64_t *out, unsigned long long *cnt) {
    const unsigned long long ni = *nitems;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ni;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t it = items[i];
        const uint32_t v = (uint32_t)(it >> 32), k0 = (uint32_t)it;
        const uint32_t ne = min(E, sdeg[v] - k0);
        const int r = ne <= 32 ? 0 : (ne <= 256 ? 1 : 2);
        out[r * cap + atomicAdd(&cnt[r], 1ull)] = it;
    }
}

struct WarpCfg {
    uint32_t E;      // in-edges per item
    uint32_t R;      // 32-bit words of the per-warp shared-memory region (bitmap or table)
    uint32_t n;      // vertices of the counting form
    uint32_t first;  // one-item-per-warp launches: the items [first, last) of `items`
    uint32_t last;
    uint64_t m;        // edges of the counting form (checked build: range checks)
    uint32_t *status;  // device status word (checked build: index violations)
};

// 1 << s for s < 32, 0 for s >= 32 (PTX clamps the shift amount; C++ leaves it undefined)
__device__ __forceinline__ uint32_t bit_or_zero(uint32_t s) {
    uint32_t r;
    asm("shl.b32 %0, 1, %1;" : "=r"(r) : "r"(s));
    return r;
}

// Unchecked units of one batch of 32 in-edges (lane k holds in-edge k): this lane's in-edge
// has nu units of 32 * S elements, unit i starting at adj index base + i * 32 * S. Unit j of
// the batch (0 <= j < U, in in-edge order) belongs to the first in-edge whose units end
// after j: one ballot, one popcount and one shuffle per unit, no branch per in-edge. Each
// unit is S coalesced 32-bit loads per lane; kUnitDepth units are in flight ahead of the one
// being tested (units past the last hold idle elements).
constexpr int kUnitDepth = 2;

template <int S, class F>
__device__ __forceinline__ uint32_t stream_units(const uint32_t *__restrict__ adjl, uint32_t nu,
                                                 uint32_t base, int lane, uint32_t idle,
                                                 const F &f) {
    constexpr uint32_t kSize = 32 * S;
    uint32_t ue = nu;  // inclusive scan: units up to and including this lane's in-edge
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, ue, o);
        if (lane >= o) ue += t;
    }
    const uint32_t U = __shfl_sync(kFull, ue, 31);
    uint32_t cnt = 0;
    if (!U) return cnt;
    // adj index of unit j of this lane's in-edge: ub + j * kSize (mod 2^32)
    const uint32_t ub = base - (ue - nu) * kSize;
    auto unit_at = [&](uint32_t j) -> const uint32_t * {
        const int e = __popc(__ballot_sync(kFull, ue <= j));
        return adjl + (__shfl_sync(kFull, ub, e & 31) + j * kSize);
    };
    uint32_t a[kUnitDepth][S];
#pragma unroll
    for (int d = 0; d < kUnitDepth; ++d) {
#pragma unroll
        for (int t = 0; t < S; ++t) a[d][t] = idle;
        if ((uint32_t)d < U) {
            const uint32_t *src = unit_at(d);
#pragma unroll
            for (int t = 0; t < S; ++t) a[d][t] = __ldg(src + 32 * t);
        }
    }
    for (uint32_t j0 = 0; j0 < U; j0 += kUnitDepth) {
#pragma unroll
        for (int d = 0; d < kUnitDepth; ++d) {
#pragma unroll
            for (int t = 0; t < S; ++t) cnt += f(a[d][t]);
            const uint32_t j = j0 + kUnitDepth + d;
#pragma unroll
            for (int t = 0; t < S; ++t) a[d][t] = idle;
            if (j < U) {
                const uint32_t *src = unit_at(j);
#pragma unroll
                for (int t = 0; t < S; ++t) a[d][t] = __ldg(src + 32 * t);
            }
        }
    }
    return cnt;
}

// Stream the suffix ranges of the item's in-edges [k0, k1) (edge k's range is in_rng[k]),
// 32 in-edges at a time (lane k holds in-edge kb + k; `first` holds the first batch's
// ranges, each next batch's are loaded one batch ahead), and test every element with f
// (f(idle) must be 0). Per batch:
//  1. units: every whole 128-element unit of every suffix (four unchecked coalesced loads
//     per lane), then one 64-element unit where 64 or more elements are left, then one
//     32-element unit where 32 or more are left;
//  2. remainders: the last (length mod 32) elements of all 32 suffixes, concatenated into
//     one sequence (in-edges with an empty remainder compacted out through `cmp`, 32
//     entries of per-warp shared memory) and swept in 32-position windows with every lane
//     busy: the in-edges that start inside a window are one OR-reduction of a bit per
//     in-edge, and lane L finds its in-edge by counting the starts at or before it.
// The per-lane count of one item fits 32 bits (at most E in-edges of at most n elements).
constexpr int kWin = 4;  // remainder windows whose loads are in flight together

template <class F>
__device__ __forceinline__ uint32_t stream_item(const uint32_t *__restrict__ adj,
                                                const uint2 *__restrict__ rng, uint32_t k0,
                                                uint32_t k1, int lane, uint32_t idle,
                                                uint2 *cmp, uint2 first, F f,
                                                const WarpCfg &p) {
    uint32_t cnt = 0;
    const uint32_t le = 0xFFFFFFFFu >> (31 - lane);  // lanes 0..lane
    const uint32_t lt = (1u << lane) - 1u;           // lanes below this one
    const uint32_t *adjl = adj + lane;
    uint2 nx = first;  // ranges of the first batch, loaded by the caller
    for (uint32_t kb = k0; kb < k1; kb += 32) {
        uint2 r = nx;
        nx = (kb + 32 + lane < k1) ? __ldg(rng + kb + 32 + lane) : make_uint2(0u, 0u);
        if constexpr (kChecked) {
            if (r.x > r.y || r.y > p.m) {  // a range outside the edges: refused, skipped
                atomicExch(p.status, kStatusBadForm);
                r = make_uint2(0u, 0u);
            }
        }
        const uint32_t len = r.y - r.x;  // 0 past the item
        // ---- 1. units
        cnt += stream_units<4>(adjl, len >> 7, r.x, lane, idle, f);
        cnt += stream_units<2>(adjl, (len >> 6) & 1u, r.x + (len & ~127u), lane, idle, f);
        cnt += stream_units<1>(adjl, (len >> 5) & 1u, r.x + (len & ~63u), lane, idle, f);
        // ---- 2. remainders, one flat sequence
        const uint32_t rl = len & 31u;
        const unsigned Z = __ballot_sync(kFull, rl != 0);
        if (!Z) continue;
        if (rl) cmp[__popc(Z & lt)] = make_uint2(r.x + (len - rl), rl);
        __syncwarp();
        const uint32_t nz = __popc(Z);
        const uint2 c = (uint32_t)lane < nz ? cmp[lane] : make_uint2(0u, 0u);
        __syncwarp();
        uint32_t inc = c.y;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, inc, o);
            if (lane >= o) inc += t;
        }
        const uint32_t T = __shfl_sync(kFull, inc, 31);
        const uint32_t P = inc - c.y;     // first position of this lane's remainder
        const uint32_t delta = c.x - P;   // adj index of position q of it: q + delta
        // start of this lane's remainder relative to the window; lanes without one never
        // start inside a window
        uint32_t dP = (uint32_t)lane < nz ? P : 0x80000000u;
        uint32_t before = 0;  // remainders starting before the window
        for (uint32_t t0 = 0; t0 < T; t0 += 32 * kWin) {
            uint32_t w[kWin];
#pragma unroll
            for (int j = 0; j < kWin; ++j) {
                const uint32_t M = __reduce_or_sync(kFull, bit_or_zero(dP));
                const uint32_t eL = before + __popc(M & le) - 1;
                const uint32_t dl = __shfl_sync(kFull, delta, eL & 31);
                const uint32_t q = t0 + 32 * j + lane;
                w[j] = q < T ? __ldg(adj + (q + dl)) : idle;
                before += __popc(M);
                dP -= 32;
            }
#pragma unroll
            for (int j = 0; j < kWin; ++j) cnt += f(w[j]);
        }
    }
    return cnt;
}

// Words of the per-warp hash table that holds the part of N+(v) below the bitmap window
// when v sits too low for the window to reach it (at most kLowHashWords / 2 elements).
constexpr uint32_t kLowHashWords = 128;
constexpr uint32_t kLowHashLg = 7;
// Per-warp region: R bitmap words, the guard word and one pad word (keeps what follows
// 8-byte aligned; R is a power of two), the low-part hash table, and 32 uint2 entries of
// scratch for compacting the remainders of a batch of in-edges.
constexpr uint32_t kCmpWords = 64;
__host__ __device__ constexpr uint32_t region_words(uint32_t R) {
    return R + 2 + kLowHashWords + kCmpWords;
}

// Per item the warp marks N+(v) in its shared-memory region: a bitmap of R words over the
// ranks [W0, n) (W0 a multiple of 32), with W0 = v + 1 rounded down when n - W0 fits the
// bitmap (high-rank v: every element of N+(v) and of the suffixes is in the window), else
// W0 = the lowest multiple of 32 with n - W0 <= 32 R, and the few elements of N+(v) below
// W0 go to an open-addressing hash table of kLowHashWords words (0 marks an empty slot:
// every element is a rank above v >= 0). A suffix element w is tested in the bitmap when
// w >= W0, else in the table. An out-list with more than kLowHashWords / 2 elements below
// the window (none on R-MAT or Holme-Kim graphs) is merged against each suffix instead.
//
// kPersistent: warps take items from the queue (acc[1]) until acc[2] items are done;
// otherwise warp w of the grid takes item first + w only (one launch per item bucket).
template <bool kPersistent>
__global__ void __maxnreg__(48) k_tc_warp(const uint64_t *__restrict__ off, const uint32_t *__restrict__ adj,
                          const uint64_t *__restrict__ in_off, const uint2 *__restrict__ in_rng,
                          const uint32_t *__restrict__ sdeg,
                          const uint64_t *__restrict__ items, unsigned long long *acc,
                          WarpCfg p) {
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ unsigned long long red[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // R words of bitmap + one guard word (reg[R]) that stays zero (idle lanes of the test
    // read it instead of branching) + the low-part hash table + remainder scratch
    uint32_t *reg = smem + (size_t)warp * region_words(p.R);
    uint32_t *tab = reg + p.R + 2;
    uint2 *cmp = reinterpret_cast<uint2 *>(tab + kLowHashWords);
    for (uint32_t q = lane; q < p.R + 2 + kLowHashWords; q += 32) reg[q] = 0u;  // zero between items
    __syncwarp();
    const uint32_t RB = p.R * 32;  // bitmap capacity in bits
    const uint32_t Wlow = p.n > RB ? ((p.n - RB + 31) & ~31u) : 0u;
    const unsigned long long nitems = acc[2];
    unsigned long long cnt = 0;
    while (true) {
        unsigned long long k = 0;
        if (kPersistent) {
            if (lane == 0) k = atomicAdd(&acc[1], 1ull);
            k = __shfl_sync(kFull, k, 0);
            if (k >= nitems) break;
        } else {
            k = p.first + (unsigned long long)blockIdx.x * (blockDim.x >> 5) + warp;
            if (k >= p.last) break;
        }
        const uint64_t it = items[k];
        const uint32_t v = (uint32_t)(it >> 32), k0 = (uint32_t)it;
        if constexpr (kChecked) {
            if (v >= p.n) {
                if (lane == 0) atomicExch(p.status, kStatusBadForm);
                if (!kPersistent) break;
                continue;
            }
        }
        const uint64_t ov = off[v];
        const uint32_t b = (uint32_t)(off[v + 1] - ov);
        const uint64_t kin = in_off[v];
        const uint32_t k1 = min(k0 + p.E, sdeg[v]);  // streamed in-edges: the first sdeg[v]
        const uint32_t *Nv = adj + ov;
        // the first batch of suffix ranges, loaded before the out-list is marked
        const uint2 first = (k0 + lane < k1) ? __ldg(in_rng + kin + k0 + lane) : make_uint2(0u, 0u);
        const uint32_t base0 = (v + 1) & ~31u;
        // 0: bitmap only; 1: bitmap + low-part table; 2: merge
        int mode = 0;
        uint32_t W0 = base0;
        if (p.n - base0 > RB) {
            W0 = Wlow;
            mode = (b > kLowHashWords / 2 && __ldg(Nv + kLowHashWords / 2) < W0) ? 2 : 1;
        }
        if (mode != 2) {
            for (uint32_t q = lane; q < b; q += 32) {
                const uint32_t w = __ldg(Nv + q);
                if (w >= W0) {
                    const uint32_t o = w - W0;
                    if (kChecked && (w >= p.n || (o >> 5) >= p.R)) {
                        atomicExch(p.status, kStatusBadForm);
                        continue;
                    }
                    atomicOr(&reg[o >> 5], 1u << (o & 31));
                } else {
                    uint32_t sl = hash_slot(w, kLowHashLg);
                    uint32_t probes = 0;
                    while (atomicCAS(&tab[sl], 0u, w) != 0u) {
                        sl = (sl + 1) & (kLowHashWords - 1);
                        if (kChecked && ++probes >= kLowHashWords) {  // table full
                            atomicExch(p.status, kStatusBadForm);
                            break;
                        }
                    }
                }
            }
        }
        __syncwarp();
        // bit w - W0 of the bitmap: word (w >> 5) - (W0 >> 5), bit w & 31 (W0 is a multiple
        // of 32); idle lanes read the guard word reg[R]
        const uint32_t *regp = reg - (W0 >> 5);
        const uint32_t idle = W0 + RB;
        // checked build: an element outside [W0, W0 + 32 R] (the idle value W0 + 32 R reads
        // the guard word) would read another warp's region
        auto outside = [&](uint32_t w) -> bool {
            if (w - W0 <= RB) return false;
            atomicExch(p.status, kStatusBadForm);
            return true;
        };
        if (mode == 0) {
            cnt += stream_item(adj, in_rng + kin, k0, k1, lane, idle, cmp, first,
                               [&](uint32_t w) -> uint32_t {
                                   if (kChecked && outside(w)) return 0u;
                                   return __funnelshift_r(regp[w >> 5], 0u, w) & 1u;
                               }, p);
        } else if (mode == 1) {
            cnt += stream_item(adj, in_rng + kin, k0, k1, lane, idle, cmp, first, [&](uint32_t w) -> uint32_t {
                if (w >= W0) {
                    if (kChecked && outside(w)) return 0u;
                    return __funnelshift_r(regp[w >> 5], 0u, w) & 1u;
                }
                uint32_t sl = hash_slot(w, kLowHashLg);
                uint32_t x = tab[sl];
                uint32_t probes = 0;
                while (x != w && x != 0u) {
                    sl = (sl + 1) & (kLowHashWords - 1);
                    x = tab[sl];
                    if (kChecked && ++probes >= kLowHashWords) break;
                }
                return x == w ? 1u : 0u;
            }, p);
        } else {
            for (uint32_t kk = k0; kk < k1; ++kk) {
                const uint2 r = __ldg(in_rng + kin + kk);
                cnt += warp_merge_count(adj + r.x, r.y - r.x, Nv, b, lane);
            }
        }
        __syncwarp();
        // return the region to all-zero
        if (mode != 2) {
            for (uint32_t q = lane; q < b; q += 32) {
                const uint32_t w = __ldg(Nv + q);
                if (w >= W0) reg[(w - W0) >> 5] = 0u;
            }
            if (mode == 1)
                for (uint32_t q = lane; q < kLowHashWords; q += 32) tab[q] = 0u;
        }
        __syncwarp();
        if (!kPersistent) break;
    }
    block_add_total(cnt, &acc[0], red);
}

// ------------------------------------------------------------------ dense core

// Core matrix rows: one warp per core row r (vertex c0 + r) sets the bits of N+(c0 + r) in a
// shared-memory row of rw words, then writes the whole row (zeros included, so M needs no
// separate clearing) and its word span [first, last] (span (1, 0): empty row). Also resets
// the core queue head for k_tc_core, which runs next on the stream. Dynamic shared memory:
// rw_max words per warp.
__global__ void __launch_bounds__(256) k_core_rows(const uint64_t *__restrict__ off,
                                                   const uint32_t *__restrict__ adj,
                                                   unsigned long long *acc, uint32_t *core_m,
                                                   uint2 *span, uint32_t rw_max,
                                                   uint32_t *status) {
    extern __shared__ __align__(16) uint32_t smem[];
    if (blockIdx.x == 0 && threadIdx.x == 0) acc[kAccCoreQ] = 0ull;
    const uint32_t K = (uint32_t)acc[kAccCoreK], c0 = (uint32_t)acc[kAccCoreC0],
                   rw = (uint32_t)acc[kAccCoreRw];
    if (!K || rw > rw_max) return;  // rw <= rw_max: the plan sized the buffers for its largest K
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *S = smem + (size_t)warp * rw_max;
    for (uint32_t q = lane; q < rw; q += 32) S[q] = 0u;
    __syncwarp();
    const uint32_t nw = gridDim.x * (blockDim.x >> 5);
    for (uint32_t r = blockIdx.x * (blockDim.x >> 5) + warp; r < K; r += nw) {
        const uint64_t ou = off[c0 + r];
        const uint32_t d = (uint32_t)(off[c0 + r + 1] - ou);
        for (uint32_t q = lane; q < d; q += 32) {
            const uint32_t o = __ldg(adj + ou + q) - c0;  // an element of a core row: >= c0
            if (kChecked && o >= K) {
                atomicExch(status, kStatusBadForm);
                continue;
            }
            atomicOr(&S[o >> 5], 1u << (o & 31));
        }
        __syncwarp();
        uint32_t *row = core_m + (size_t)r * rw;
        for (uint32_t q = lane; q < rw; q += 32) {
            row[q] = S[q];
            S[q] = 0u;
        }
        if (lane == 0)
            span[r] = d ? make_uint2((__ldg(adj + ou) - c0) >> 5, (__ldg(adj + ou + d - 1) - c0) >> 5)
                        : make_uint2(1u, 0u);
        __syncwarp();
    }
}

// Per-warp shared memory of k_tc_core: the staged row (rw_max words), one guard group that
// stays zero (positions past the end of a sweep read it), and the compacted segments of a
// batch of 32 edges (first group, matrix row, length: 3 x 32 words).
__host__ __device__ constexpr uint32_t core_region_words(uint32_t rw_max) {
    return rw_max + kCoreGroupWords + 96;
}
constexpr int kCoreWin = 4;  // 32-position windows whose loads are in flight together

// Core count: warps take core rows r from the queue (acc[kAccCoreQ]), heaviest (lowest rank)
// first; for u = c0 + r the warp copies the groups of M[u] that hold its span into shared
// memory, and for each batch of 32 edges u->v (lane k: edge k; the last edge of the row has
// no later element and is skipped) takes the groups of N+(v)'s span up to u's last group (a
// group reaches past a span only over zero words of M[v] or of the staged row, so whole
// groups count exactly). The non-empty group ranges are compacted and swept as one flat
// sequence in 32-position windows with every lane busy: the segment of position q is found
// from the segment starts inside the window (one OR-reduction of a bit per segment) and
// gives the matrix group by one shuffle; the group within the row (the staged row's group)
// is that index masked. Group g of edge u->v adds the popcounts of M[u][g] & M[v][g],
// kCoreGroupWords words, 16-byte loads from each. M[v] comes from L2 (the matrix, 32 MB
// for 16384 ranks, is written by k_core_rows just before).
// Four resident blocks per SM (58 registers): on R-MAT scale 21 with 24,576 core ranks
// 0.418 ms, against 0.422 ms at five (46 registers), 0.436 ms at six and 0.433 ms at three;
// four windows in flight (six: 0.430 ms).
__global__ void __launch_bounds__(256, 4) k_tc_core(const uint64_t *__restrict__ off,
                                                 const uint32_t *__restrict__ adj,
                                                 const uint32_t *__restrict__ core_m,
                                                 const uint2 *__restrict__ span,
                                                 unsigned long long *acc, uint32_t rw_max,
                                                 uint32_t *status) {
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ unsigned long long red[32];
    const uint32_t K = (uint32_t)acc[kAccCoreK], c0 = (uint32_t)acc[kAccCoreC0],
                   rw = (uint32_t)acc[kAccCoreRw];
    unsigned long long cnt = 0;
    if (K && rw <= rw_max) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        uint32_t *B = smem + (size_t)warp * core_region_words(rw_max);
        uint32_t *cj = B + rw_max + kCoreGroupWords, *cr = cj + 32, *cl = cr + 32;
        const uint32_t guard = rw_max / kCoreGroupWords;  // the zero group after the row
        // all-zero between rows, the guard group always
        for (uint32_t q = lane; q < rw_max + kCoreGroupWords; q += 32) B[q] = 0u;
        __syncwarp();
        const uint32_t le = 0xFFFFFFFFu >> (31 - lane);  // lanes 0..lane
        const uint32_t lt = (1u << lane) - 1u;           // lanes below this one
        while (true) {
            unsigned long long k = 0;
            if (lane == 0) k = atomicAdd(&acc[kAccCoreQ], 1ull);
            k = __shfl_sync(kFull, k, 0);
            if (k >= K) break;
            const uint32_t r = (uint32_t)k;
            const uint64_t ou = off[c0 + r];
            const uint32_t d = (uint32_t)(off[c0 + r + 1] - ou);
            if (d < 2) continue;
            const uint2 su = __ldg(span + r);  // words of N+(u)
            if (kChecked && (su.x > su.y || su.y >= rw)) {
                if (lane == 0) atomicExch(status, kStatusBadForm);
                continue;
            }
            const uint32_t rwg = rw / kCoreGroupWords;  // groups per row, a power of two
            const uint4 *M4 = reinterpret_cast<const uint4 *>(core_m);
            uint4 *B4 = reinterpret_cast<uint4 *>(B);
            const uint32_t gu0 = su.x / kCoreGroupWords, gu1 = su.y / kCoreGroupWords;  // N+(u)
            for (uint32_t j = gu0 * kCoreVec + lane; j < (gu1 + 1) * kCoreVec; j += 32)
                B4[j] = __ldg(M4 + (size_t)r * (rw / 4) + j);
            __syncwarp();
            uint32_t part = 0;
            // the batch's heads, loaded one batch ahead
            uint32_t vnx = (uint32_t)lane + 1 < d ? __ldg(adj + ou + lane) : 0u;
            for (uint32_t kb = 0; kb + 1 < d; kb += 32) {
                const uint32_t i = kb + lane;
                uint32_t jlo = 1, jhi = 0, vr = 0;
                const uint32_t vcur = vnx;
                vnx = i + 33 < d ? __ldg(adj + ou + i + 32) : 0u;
                if (i + 1 < d) {
                    vr = vcur - c0;
                    if (kChecked && vr >= K) {
                        atomicExch(status, kStatusBadForm);
                    } else {
                        const uint2 sv = __ldg(span + vr);
                        if (sv.x <= sv.y) {  // groups of N+(v) up to u's last group
                            jlo = sv.x / kCoreGroupWords;
                            jhi = min(sv.y / kCoreGroupWords, gu1);
                        }
                    }
                }
                const uint32_t len = jhi >= jlo ? jhi - jlo + 1 : 0u;
                const unsigned Z = __ballot_sync(kFull, len != 0);
                if (!Z) continue;
                if (len) {
                    const uint32_t c = __popc(Z & lt);
                    cj[c] = jlo;
                    cr[c] = vr;
                    cl[c] = len;
                }
                __syncwarp();
                const uint32_t nz = __popc(Z);
                uint32_t sj = 0, sr = 0, sl = 0;
                if ((uint32_t)lane < nz) {
                    sj = cj[lane];
                    sr = cr[lane];
                    sl = cl[lane];
                }
                __syncwarp();
                uint32_t inc = sl;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t t = __shfl_up_sync(kFull, inc, o);
                    if (lane >= o) inc += t;
                }
                const uint32_t T = __shfl_sync(kFull, inc, 31);
                const uint32_t P = inc - sl;             // first position of this lane's segment
                const uint32_t dM = sr * rwg + sj - P;   // matrix group of position q: q + dM
                uint32_t dP = (uint32_t)lane < nz ? P : 0x80000000u;
                uint32_t before = 0;  // segments starting before the window
                for (uint32_t t0 = 0; t0 < T; t0 += 32 * kCoreWin) {
                    uint4 x[kCoreWin][kCoreVec], y[kCoreWin][kCoreVec];
#pragma unroll
                    for (int w = 0; w < kCoreWin; ++w) {
                        const uint32_t Mk = __reduce_or_sync(kFull, bit_or_zero(dP));
                        const uint32_t eL = (before + __popc(Mk & le) - 1) & 31u;
                        const uint32_t q = t0 + 32 * w + lane;
                        uint32_t g = q + __shfl_sync(kFull, dM, eL);
                        uint32_t gb = g & (rwg - 1);  // the group within the row
                        if (q >= T) {  // past the sweep: matrix group 0 against the zero guard
                            g = 0;
                            gb = guard;
                        }
#pragma unroll
                        for (uint32_t c = 0; c < kCoreVec; ++c) {
                            x[w][c] = __ldg(M4 + (size_t)g * kCoreVec + c);
                            y[w][c] = B4[gb * kCoreVec + c];
                        }
                        before += __popc(Mk);
                        dP -= 32;
                    }
#pragma unroll
                    for (int w = 0; w < kCoreWin; ++w)
#pragma unroll
                        for (uint32_t c = 0; c < kCoreVec; ++c)
                            part += __popc(x[w][c].x & y[w][c].x) + __popc(x[w][c].y & y[w][c].y) +
                                    __popc(x[w][c].z & y[w][c].z) + __popc(x[w][c].w & y[w][c].w);
                }
            }
            cnt += part;
            __syncwarp();
            for (uint32_t j = gu0 * kCoreVec + lane; j < (gu1 + 1) * kCoreVec; j += 32)
                B4[j] = make_uint4(0u, 0u, 0u, 0u);
            __syncwarp();
        }
    }
    block_add_total(cnt, &acc[0], red);
}

}  // namespace

struct TcPlan {
    rtg_tc_mode mode = RTG_TC_BATCHED;
    rtg_config cfg{};
    // batched
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t *items = nullptr;
    uint32_t *vcnt = nullptr;
    uint32_t *sdeg = nullptr;     // streamed in-edges per vertex
    void *cub_tmp = nullptr;
    unsigned long long *acc = nullptr;
    uint32_t *core_m = nullptr;   // dense-core matrix and row spans (sized for the largest K)
    uint2 *core_span = nullptr;
    uint32_t core_ranks = 0;      // the K picked when the items were built
    cudaEvent_t k0 = nullptr, k1 = nullptr, c0 = nullptr;
    uint64_t graph_kernels = 0;
    // plain
    uint8_t *bucket = nullptr;
    uint32_t *lists = nullptr;
    // bucketed: items sorted into kItemBuckets regions of item_cap entries each
    uint64_t *bitems = nullptr;
    cudaEvent_t bev[2 * kPlainBuckets] = {};
};

void tc_plan_free(TcPlan *p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    dev_free(p->items);
    dev_free(p->vcnt);
    dev_free(p->sdeg);
    dev_free(p->core_m);
    dev_free(p->core_span);
    dev_free(p->cub_tmp);
    dev_free(p->acc);
    dev_free(p->bucket);
    dev_free(p->lists);
    dev_free(p->bitems);
    if (p->k0) cudaEventDestroy(p->k0);
    if (p->k1) cudaEventDestroy(p->k1);
    if (p->c0) cudaEventDestroy(p->c0);
    for (auto ev : p->bev)
        if (ev) cudaEventDestroy(ev);
    delete p;
}

namespace {

// In-edges per item when the context leaves it open: larger items on large graphs (R-MAT
// scale 20 and 21, Holme-Kim 2^20: 0-1.7 % faster with 1024 than with 256), smaller ones
// on small graphs (R-MAT scale 18: 15 % faster with 256 than with 512).
constexpr uint64_t kLargeItemsFrom = 1ull << 23;  // oriented edges
constexpr uint32_t kLargeItemEdges = 1024;

rtg_config effective_config(const rtg_ctx *ctx, uint64_t m) {
    rtg_config c = ctx->cfg;
    if (!c.tc_item_edges) c.tc_item_edges = m >= kLargeItemsFrom ? kLargeItemEdges : kDefaultItemEdges;
    if (!c.tc_block_warps) c.tc_block_warps = kDefaultBlockWarps;
    if (!c.tc_region_words) c.tc_region_words = kDefaultRegionWords;
    return c;
}

bool same_tc_config(const rtg_config &a, const rtg_config &b) {
    return a.tc_item_edges == b.tc_item_edges && a.tc_region_words == b.tc_region_words &&
           a.tc_block_warps == b.tc_block_warps && a.tc_blocks_per_sm == b.tc_blocks_per_sm &&
           a.tc_core_ranks == b.tc_core_ranks;
}

// Launch shape of the batched count of one graph under one schedule.
struct BatchedShape {
    WarpCfg pc;
    uint32_t W;
    size_t smem;
    int grid, g1;
    uint64_t item_cap;
    size_t cub_bytes;
    // dense core: the schedule's setting, the largest K it can pick, that K's row words
    uint32_t core_forced, core_max, core_rw;
    size_t core_rows_smem, core_smem;
    int core_rows_grid, core_grid;
    uint64_t core_m_words() const { return (uint64_t)core_max * core_rw; }
};

constexpr int kCoreWarps = 8;  // warps per block of both core kernels

// The core kernels' buffers and launch shape for cores of at most K ranks.
rtg_status core_shape(rtg_ctx *ctx, uint32_t K, BatchedShape *bs) {
    bs->core_max = K;
    bs->core_rw = core_row_words(K);
    bs->core_rows_smem = (size_t)kCoreWarps * bs->core_rw * 4;
    bs->core_smem = (size_t)kCoreWarps * core_region_words(bs->core_rw) * 4;
    bs->core_rows_grid = bs->core_grid = 1;
    if (!K) return RTG_OK;
    if (bs->core_smem + 512 > (size_t)ctx->smem_optin)
        return fail(ctx, RTG_ERR_INVALID_ARG, "core of %u ranks needs %zu B of shared memory", K,
                    bs->core_smem);
    RTG_CUDA(ctx, cudaFuncSetAttribute(k_core_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bs->core_rows_smem));
    RTG_CUDA(ctx, cudaFuncSetAttribute(k_tc_core, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bs->core_smem));
    int per_sm = 0;
    RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tc_core, kCoreWarps * 32,
                                                                bs->core_smem));
    bs->core_grid = ctx->sm_count * std::max(per_sm, 1);
    bs->core_rows_grid = (int)std::max<uint64_t>(
        1, std::min<uint64_t>((K + kCoreWarps - 1) / kCoreWarps, ctx->sm_count * 8ull));
    return RTG_OK;
}

rtg_status batched_shape(rtg_ctx *ctx, const CountCsr &c, const rtg_config &cfg,
                         BatchedShape *bs) {
    bs->W = cfg.tc_block_warps;
    bs->pc.E = cfg.tc_item_edges;
    bs->pc.R = cfg.tc_region_words;
    bs->pc.n = c.n;
    bs->pc.m = c.m;
    bs->pc.status = ctx->d_status;
    bs->smem = (size_t)bs->W * region_words(bs->pc.R) * 4;
    if (bs->smem + 256 > (size_t)ctx->smem_optin)
        return fail(ctx, RTG_ERR_INVALID_ARG, "schedule needs %zu B of shared memory", bs->smem);
    bs->item_cap = c.m / bs->pc.E + c.n + 1;
    bs->cub_bytes = 0;
    RTG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, bs->cub_bytes, (uint32_t *)nullptr,
                                                (uint32_t *)nullptr, (int64_t)c.n + 1,
                                                ctx->stream));
    RTG_CUDA(ctx, cudaFuncSetAttribute(k_tc_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bs->smem));
    int per_sm = 0;
    RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tc_warp<true>, bs->W * 32,
                                                                bs->smem));
    if (cfg.tc_blocks_per_sm) per_sm = std::min<int>(per_sm, (int)cfg.tc_blocks_per_sm);
    per_sm = std::max(per_sm, 1);
    bs->grid = ctx->sm_count * per_sm;
    bs->g1 = (int)std::max<uint64_t>(1, std::min<uint64_t>((c.n + 256ull) / 256,
                                                          ctx->sm_count * 16ull));
    const uint32_t K = core_max_ranks(cfg.tc_core_ranks, c);
    // what the device pick is told: a size known on the host is passed as is
    bs->core_forced = !K ? RTG_TC_CORE_NONE
                         : (cfg.tc_core_ranks || c.core_auto >= 0 ? K : 0u);
    return core_shape(ctx, K, bs);
}

// Device buffers of one batched count (a plan's, or carved from caller scratch).
struct CountBufs {
    uint64_t *items;
    uint32_t *vcnt;  // 2 (n + 1): items per vertex, their exclusive scan
    uint32_t *sdeg;  // n + 1
    void *cub_tmp;
    unsigned long long *acc;  // kAccWords
    uint32_t *core_m;         // core_max x core_rw words
    uint2 *core_span;         // core_max
};

// reset -> core pick -> item counts (and sdeg) -> scan -> item fill (acc[2] = items)
void enqueue_items(cudaStream_t st, const CountCsr &c, const BatchedShape &bs, const CountBufs &b) {
    uint32_t *vbase = b.vcnt + (c.n + 1ull);
    size_t cub_bytes = bs.cub_bytes;
    cudaMemsetAsync(b.acc, 0, kAccWords * sizeof(unsigned long long), st);
    k_core_pick<<<1, 32, 0, st>>>(c.off, c.n, c.m, bs.core_forced, b.acc);
    k_item_counts<<<bs.g1, 256, 0, st>>>(c.off, c.in_off, c.in_rng, c.n, bs.pc.E, b.acc, b.vcnt,
                                         b.sdeg);
    cub::DeviceScan::ExclusiveSum(b.cub_tmp, cub_bytes, b.vcnt, vbase, (int64_t)c.n + 1, st);
    k_item_fill<<<bs.g1, 256, 0, st>>>(c.off, b.sdeg, c.n, bs.pc.E, vbase, b.items, b.acc);
}

void record(cudaEvent_t ev, cudaStream_t st, bool external) {
    if (!ev) return;
    if (external) cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
    else cudaEventRecord(ev, st);
}

// core matrix rows -> core count (both return at once without a core); kCoreKernels launches
constexpr uint64_t kCoreKernels = 2;

void enqueue_core(cudaStream_t st, const CountCsr &c, const BatchedShape &bs, const CountBufs &b,
                  uint32_t *status) {
    k_core_rows<<<bs.core_rows_grid, kCoreWarps * 32, bs.core_rows_smem, st>>>(
        c.off, c.adj, b.acc, b.core_m, b.core_span, bs.core_rw, status);
    k_tc_core<<<bs.core_grid, kCoreWarps * 32, bs.core_smem, st>>>(
        c.off, c.adj, b.core_m, b.core_span, b.acc, bs.core_rw, status);
}

// reset of the total and the queue head (acc[2], the item count, and the core fields stay)
// -> [c0] core stage [k0] persistent count [k1]
void enqueue_count(cudaStream_t st, const CountCsr &c, const BatchedShape &bs, const CountBufs &b,
                   cudaEvent_t ec0, cudaEvent_t k0, cudaEvent_t k1, bool external_events) {
    cudaMemsetAsync(b.acc, 0, 2 * sizeof(unsigned long long), st);
    record(ec0, st, external_events);
    if (bs.core_max) enqueue_core(st, c, bs, b, bs.pc.status);
    record(k0, st, external_events);
    k_tc_warp<true><<<bs.grid, bs.W * 32, bs.smem, st>>>(c.off, c.adj, c.in_off, c.in_rng, b.sdeg,
                                                         b.items, b.acc, bs.pc);
    record(k1, st, external_events);
}

// core pick, item counts, scan (init + sweep), item fill
constexpr uint64_t kItemKernels = 5;

uint64_t count_kernels(const BatchedShape &bs) { return 1 + (bs.core_max ? kCoreKernels : 0); }

void enqueue_batched(cudaStream_t st, const CountCsr &c, const BatchedShape &bs, const CountBufs &b) {
    enqueue_items(st, c, bs, b);
    enqueue_count(st, c, bs, b, nullptr, nullptr, nullptr, false);
}

// A plan's items, built once when the plan is made (the counting form does not change while
// the plan exists), so that a replay launches only the count. Ordering them heaviest first
// by an estimated cost (elements streamed per item) was tried: 2.76 ms on R-MAT-21 against
// 2.72 ms for descending rank order, which keeps the items of one vertex together.
CountBufs plan_bufs(const TcPlan *p) {
    return CountBufs{p->items, p->vcnt, p->sdeg, p->cub_tmp, p->acc, p->core_m, p->core_span};
}

rtg_status plan_items(rtg_ctx *ctx, const CountCsr &c, const BatchedShape &bs, TcPlan *p) {
    enqueue_items(ctx->stream, c, bs, plan_bufs(p));
    ctx->launches += kItemKernels;
    RTG_CUDA(ctx, cudaGetLastError());
    // the plan may be replayed on another context's stream (the serving engine's runs
    // share a graph's plan): the items must be complete before the plan is handed out
    unsigned long long K = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&K, p->acc + kAccCoreK, 8, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    p->core_ranks = (uint32_t)K;
    return RTG_OK;
}

// plan buffers shared by the BATCHED and BUCKETED plans
rtg_status alloc_count_bufs(rtg_ctx *ctx, const CountCsr &c, const BatchedShape &bs, TcPlan *p) {
    RTG_TRY(dev_alloc(ctx, (void **)&p->items, bs.item_cap * 8));
    RTG_TRY(dev_alloc(ctx, (void **)&p->vcnt, (c.n + 1ull) * 4 * 2));
    RTG_TRY(dev_alloc(ctx, (void **)&p->sdeg, (c.n + 1ull) * 4));
    RTG_TRY(dev_alloc(ctx, (void **)&p->acc, kAccWords * sizeof(unsigned long long)));
    RTG_TRY(dev_alloc(ctx, &p->cub_tmp, bs.cub_bytes));
    if (bs.core_max) {
        RTG_TRY(dev_alloc(ctx, (void **)&p->core_m, bs.core_m_words() * 4));
        RTG_TRY(dev_alloc(ctx, (void **)&p->core_span, (uint64_t)bs.core_max * 8));
    }
    return RTG_OK;
}

rtg_status batched_plan(rtg_ctx *ctx, rtg_graph *g, TcPlan **out) {
    rtg_config cfg = effective_config(ctx, g->cnt.m);
    if (g->plan_batched && same_tc_config(g->plan_batched->cfg, cfg)) {
        *out = g->plan_batched;
        return RTG_OK;
    }
    tc_plan_free(g->plan_batched);
    g->plan_batched = nullptr;
    TcPlan *p = new TcPlan();
    p->mode = RTG_TC_BATCHED;
    p->cfg = cfg;
    auto bail = [&](rtg_status s) {
        tc_plan_free(p);
        return s;
    };
    const CountCsr &c = g->cnt;
    if (!c.built)
        return bail(fail(ctx, RTG_ERR_STATE, "counting form of the CSR is missing"));
    BatchedShape bs{};
    rtg_status s;
    if ((s = batched_shape(ctx, c, cfg, &bs)) != RTG_OK) return bail(s);
    if ((s = alloc_count_bufs(ctx, c, bs, p)) != RTG_OK) return bail(s);
    cudaError_t e;
    if ((e = cudaEventCreate(&p->k0)) != cudaSuccess ||
        (e = cudaEventCreate(&p->k1)) != cudaSuccess ||
        (e = cudaEventCreate(&p->c0)) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "event", __FILE__, __LINE__));
    if ((s = plan_items(ctx, c, bs, p)) != RTG_OK) return bail(s);
    if (p->core_ranks != bs.core_max) {  // the buffers shrink to the core the pick chose
        dev_free(p->core_m);
        dev_free(p->core_span);
        p->core_m = nullptr;
        p->core_span = nullptr;
        if ((s = core_shape(ctx, p->core_ranks, &bs)) != RTG_OK) return bail(s);
        if (bs.core_max &&
            ((s = dev_alloc(ctx, (void **)&p->core_m, bs.core_m_words() * 4)) != RTG_OK ||
             (s = dev_alloc(ctx, (void **)&p->core_span, (uint64_t)bs.core_max * 8)) != RTG_OK))
            return bail(s);
    }
    if ((e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
        return bail(cuda_fail(ctx, e, "capture", __FILE__, __LINE__));
    enqueue_count(ctx->stream, c, bs, plan_bufs(p), p->c0, p->k0, p->k1, true);
    e = cudaStreamEndCapture(ctx->stream, &p->graph);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "end capture", __FILE__, __LINE__));
    if ((e = cudaGraphInstantiate(&p->exec, p->graph, 0)) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "instantiate", __FILE__, __LINE__));
    size_t nn = 0;
    cudaGraphGetNodes(p->graph, nullptr, &nn);
    std::vector<cudaGraphNode_t> nodes(nn);
    cudaGraphGetNodes(p->graph, nodes.data(), &nn);
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(nd, &t);
        if (t == cudaGraphNodeTypeKernel) p->graph_kernels++;
    }
    g->plan_batched = p;
    *out = p;
    return RTG_OK;
}

rtg_status count_batched(rtg_ctx *ctx, rtg_graph *g, uint64_t *total, rtg_timing *t) {
    TcPlan *p = nullptr;
    RTG_TRY(batched_plan(ctx, g, &p));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    RTG_CUDA(ctx, cudaGraphLaunch(p->exec, ctx->stream));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
    ctx->launches += p->graph_kernels;
    unsigned long long h = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&h, p->acc, 8, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
    RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[2]));
    RTG_TRY(check_status_word(ctx));
    *total = h;
    float ms = 0, kms = 0, dms = 0, cms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&kms, p->k0, p->k1);
    cudaEventElapsedTime(&cms, p->c0, p->k0);
    cudaEventElapsedTime(&dms, ctx->ev[1], ctx->ev[2]);
    t->count_ms = ms;
    t->main_kernel_ms = kms;
    t->core_ms = p->core_ranks ? cms : 0.0;
    t->core_ranks = p->core_ranks;
    t->d2h_ms += dms;
    t->kernel_launches += p->graph_kernels;
    return RTG_OK;
}

rtg_status count_plain(rtg_ctx *ctx, rtg_graph *g, uint64_t *total, rtg_timing *t) {
    const Csr &c = g->ori;
    TcPlan *p = g->plan_plain;
    if (!p) {
        p = new TcPlan();
        p->mode = RTG_TC_PLAIN;
        rtg_status s = dev_alloc(ctx, (void **)&p->bucket, std::max<uint64_t>(c.m, 1));
        if (s == RTG_OK) s = dev_alloc(ctx, (void **)&p->lists, std::max<uint64_t>(c.m, 1) * 4);
        if (s == RTG_OK)
            s = dev_alloc(ctx, (void **)&p->acc, (1 + 3 * kPlainBuckets) * sizeof(unsigned long long));
        for (auto &ev : p->bev)
            if (s == RTG_OK && cudaEventCreate(&ev) != cudaSuccess)
                s = cuda_fail(ctx, cudaGetLastError(), "event", __FILE__, __LINE__);
        if (s != RTG_OK) {
            tc_plan_free(p);
            return s;
        }
        g->plan_plain = p;
    }
    uint64_t l0 = ctx->launches;
    unsigned long long *d_total = p->acc, *d_counts = p->acc + 1, *d_base = d_counts + kPlainBuckets,
                       *d_cursor = d_base + kPlainBuckets;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((c.m + 255) / 256,
                                                                    ctx->sm_count * 16ull));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    RTG_CUDA(ctx, cudaMemsetAsync(p->acc, 0, (1 + 3 * kPlainBuckets) * 8, ctx->stream));
    if (c.m) {
        k_plain_classify<<<grid, 256, 0, ctx->stream>>>(c.off, c.adj, c.src, c.m, p->bucket,
                                                        d_counts);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
    }
    unsigned long long hc[kPlainBuckets] = {0};
    RTG_CUDA(ctx, cudaMemcpyAsync(hc, d_counts, sizeof hc, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    unsigned long long hb[kPlainBuckets], run = 0;
    for (int i = 0; i < kPlainBuckets; ++i) {
        hb[i] = run;
        run += hc[i];
    }
    float kms_sum = 0;
    if (run) {
        RTG_CUDA(ctx, cudaMemcpyAsync(d_base, hb, sizeof hb, cudaMemcpyHostToDevice, ctx->stream));
        k_plain_scatter<<<grid, 256, 0, ctx->stream>>>(p->bucket, c.m, d_base, d_cursor, p->lists);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        for (int i = 0; i < kPlainBuckets; ++i) {
            if (!hc[i]) continue;
            uint64_t blocks = (hc[i] + 7) / 8;
            int gb = (int)std::min<uint64_t>(blocks, 65535);
            RTG_CUDA(ctx, cudaEventRecord(p->bev[2 * i], ctx->stream));
            if (i < 3)
                k_plain_edges<false><<<gb, 256, 0, ctx->stream>>>(c.off, c.adj, c.src,
                                                                  p->lists + hb[i], hc[i], d_total);
            else
                k_plain_edges<true><<<gb, 256, 0, ctx->stream>>>(c.off, c.adj, c.src,
                                                                 p->lists + hb[i], hc[i], d_total);
            ctx->launches++;
            RTG_CUDA(ctx, cudaGetLastError());
            RTG_CUDA(ctx, cudaEventRecord(p->bev[2 * i + 1], ctx->stream));
        }
    }
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
    unsigned long long h = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&h, d_total, 8, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
    RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[2]));
    *total = h;
    for (int i = 0; i < kPlainBuckets && run; ++i) {
        if (!hc[i]) continue;
        float bms = 0;
        cudaEventElapsedTime(&bms, p->bev[2 * i], p->bev[2 * i + 1]);
        kms_sum += bms;
    }
    float ms = 0, dms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&dms, ctx->ev[1], ctx->ev[2]);
    t->count_ms = ms;
    t->main_kernel_ms = kms_sum;
    t->d2h_ms += dms;
    t->kernel_launches += ctx->launches - l0;
    return RTG_OK;
}

// The counting-form kernel without persistence or graph, with the library's default
// schedule: work items built on every call, sorted into size buckets, one launch per
// non-empty bucket with one warp per item (grid = items / warps per block).
rtg_status count_bucketed(rtg_ctx *ctx, rtg_graph *g, uint64_t *total, rtg_timing *t) {
    const CountCsr &c = g->cnt;
    if (!c.built) return fail(ctx, RTG_ERR_STATE, "counting form of the CSR is missing");
    rtg_config dcfg{};
    dcfg.tc_item_edges = c.m >= kLargeItemsFrom ? kLargeItemEdges : kDefaultItemEdges;
    dcfg.tc_block_warps = kDefaultBlockWarps;
    dcfg.tc_region_words = kDefaultRegionWords;
    dcfg.tc_core_ranks = ctx->cfg.tc_core_ranks;  // the core is the algorithm's, not the schedule's
    BatchedShape bs{};
    RTG_TRY(batched_shape(ctx, c, dcfg, &bs));
    TcPlan *p = g->plan_bucketed;
    if (p && !same_tc_config(p->cfg, dcfg)) {  // buffers sized for another core setting
        tc_plan_free(p);
        p = g->plan_bucketed = nullptr;
    }
    if (!p) {
        p = new TcPlan();
        p->mode = RTG_TC_BUCKETED;
        p->cfg = dcfg;
        rtg_status s = alloc_count_bufs(ctx, c, bs, p);
        if (s == RTG_OK) s = dev_alloc(ctx, (void **)&p->bitems, bs.item_cap * 8 * kItemBuckets);
        if (s != RTG_OK) {
            tc_plan_free(p);
            return s;
        }
        g->plan_bucketed = p;
    }
    RTG_CUDA(ctx, cudaFuncSetAttribute(k_tc_warp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bs.smem));
    const uint64_t l0 = ctx->launches;
    const CountBufs b = plan_bufs(p);
    unsigned long long *acc = p->acc, *bcnt = p->acc + 3;
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    enqueue_items(ctx->stream, c, bs, b);  // zeroes acc
    ctx->launches += kItemKernels;
    const int gb = (int)std::max<uint64_t>(1, std::min<uint64_t>((bs.item_cap + 255) / 256,
                                                                  ctx->sm_count * 16ull));
    k_item_bucket<<<gb, 256, 0, ctx->stream>>>(p->items, acc + 2, p->sdeg, bs.pc.E, bs.item_cap,
                                               p->bitems, bcnt);
    ctx->launches++;
    RTG_CUDA(ctx, cudaGetLastError());
    float cms = 0;
    if (bs.core_max) {
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
        enqueue_core(ctx->stream, c, bs, b, ctx->d_status);
        ctx->launches += kCoreKernels;
        RTG_CUDA(ctx, cudaGetLastError());
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
    }
    // bucket counts (acc[3..5]) and the core's size (acc[8])
    unsigned long long hc[kAccCoreK - 2] = {0};
    RTG_CUDA(ctx, cudaMemcpyAsync(hc, bcnt, sizeof hc, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (bs.core_max) cudaEventElapsedTime(&cms, ctx->ev[4], ctx->ev[5]);
    t->core_ranks = (uint32_t)hc[kAccCoreK - 3];
    t->core_ms = t->core_ranks ? cms : 0.0;
    float kms_sum = 0;
    for (int r = 0; r < kItemBuckets; ++r) {
        if (!hc[r]) continue;
        WarpCfg pc = bs.pc;
        pc.first = 0;
        pc.last = (uint32_t)hc[r];
        const uint64_t blocks = (hc[r] + bs.W - 1) / bs.W;
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
        k_tc_warp<false><<<(unsigned)blocks, bs.W * 32, bs.smem, ctx->stream>>>(
            c.off, c.adj, c.in_off, c.in_rng, p->sdeg, p->bitems + r * bs.item_cap, acc, pc);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
        RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[5]));
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
        kms_sum += ms;
    }
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
    unsigned long long h = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&h, acc, 8, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
    RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[2]));
    *total = h;
    float ms = 0, dms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&dms, ctx->ev[1], ctx->ev[2]);
    t->count_ms = ms;
    t->main_kernel_ms = kms_sum;
    t->d2h_ms += dms;
    t->kernel_launches += ctx->launches - l0;
    return RTG_OK;
}

}  // namespace

uint32_t core_auto_host(const uint64_t *off, uint32_t n, uint64_t m) { return auto_core(off, n, m); }

void enqueue_core_auto(cudaStream_t st, const CountCsr &cc, unsigned long long *out) {
    k_core_auto<<<1, 32, 0, st>>>(cc.off, cc.n, cc.m, out);
}

void enqueue_core_choice(cudaStream_t st, const CountCsr &cc, uint32_t setting,
                         unsigned long long *out) {
    k_core_choice<<<1, 32, 0, st>>>(cc.off, cc.n, cc.m, setting, out);
}

uint64_t tc_plan_estimate_bytes(const rtg_ctx *ctx, const rtg_graph *g) {
    const CountCsr &c = g->cnt;
    const rtg_config cfg = effective_config(ctx, c.m);
    const uint32_t K = core_max_ranks(cfg.tc_core_ranks, c);
    // items + vertex counts and their scan + sdeg + scan temporary (bounded by one word per
    // vertex) + totals and alignment + core matrix and spans
    return (c.m / cfg.tc_item_edges + c.n + 1) * 8 + (c.n + 1ull) * 8 + (c.n + 1ull) * 4 +
           (c.n + 1ull) * 4 + 4096 + (uint64_t)K * core_row_words(K) * 4 + (uint64_t)K * 8;
}

rtg_status tc_launch_direct(rtg_ctx *ctx, rtg_graph *g, void *scratch, uint64_t scratch_bytes,
                            unsigned long long *h_total) {
    const CountCsr &c = g->cnt;
    if (!c.built) return fail(ctx, RTG_ERR_STATE, "counting form of the CSR is missing");
    if (c.n > 0x7FFFFFFFu || c.m >= (1ull << 32))
        return fail(ctx, RTG_ERR_INVALID_ARG, "graph too large for 32-bit edge ids");
    if (c.m == 0) {
        *h_total = 0;
        return RTG_OK;
    }
    if (tc_plan_estimate_bytes(ctx, g) > scratch_bytes)
        return fail(ctx, RTG_ERR_INVALID_ARG, "scratch too small for the count");
    if (kChecked) RTG_TRY(check_count_form(ctx, c));
    BatchedShape bs{};
    RTG_TRY(batched_shape(ctx, c, effective_config(ctx, c.m), &bs));
    // scratch: acc | core matrix | core spans | items | vertex counts and their scan | sdeg |
    // scan temporary (the matrix and the scan temporary 256-byte aligned)
    auto up = [](uintptr_t x) { return (x + 255) & ~(uintptr_t)255; };
    const uintptr_t p0 = reinterpret_cast<uintptr_t>(scratch);
    CountBufs b{};
    b.acc = reinterpret_cast<unsigned long long *>(p0);
    b.core_m = reinterpret_cast<uint32_t *>(up(p0 + kAccWords * 8));
    b.core_span = reinterpret_cast<uint2 *>(b.core_m + bs.core_m_words());
    b.items = reinterpret_cast<uint64_t *>(b.core_span + bs.core_max);
    b.vcnt = reinterpret_cast<uint32_t *>(b.items + bs.item_cap);
    b.sdeg = b.vcnt + 2 * (c.n + 1ull);
    b.cub_tmp = reinterpret_cast<void *>(up(reinterpret_cast<uintptr_t>(b.sdeg + (c.n + 1ull))));
    if ((uint64_t)(reinterpret_cast<uintptr_t>(b.cub_tmp) - p0) + bs.cub_bytes > scratch_bytes)
        return fail(ctx, RTG_ERR_INVALID_ARG, "scratch too small for the count");
    enqueue_batched(ctx->stream, c, bs, b);
    RTG_CUDA(ctx, cudaGetLastError());
    ctx->launches += kItemKernels + count_kernels(bs);
    RTG_CUDA(ctx, cudaMemcpyAsync(h_total, b.acc, 8, cudaMemcpyDeviceToHost, ctx->stream));
    return RTG_OK;
}

rtg_status tc_launch_async(rtg_ctx *ctx, rtg_graph *g, unsigned long long *h_total) {
    const CountCsr &c = g->cnt;
    if (!c.built) return fail(ctx, RTG_ERR_STATE, "counting form of the CSR is missing");
    if (c.n > 0x7FFFFFFFu || c.m >= (1ull << 32))
        return fail(ctx, RTG_ERR_INVALID_ARG, "graph too large for 32-bit edge ids");
    if (c.m == 0) {
        *h_total = 0;
        return RTG_OK;
    }
    if (kChecked) RTG_TRY(check_count_form(ctx, c));
    TcPlan *p = nullptr;
    RTG_TRY(batched_plan(ctx, g, &p));
    RTG_CUDA(ctx, cudaGraphLaunch(p->exec, ctx->stream));
    ctx->launches += p->graph_kernels;
    RTG_CUDA(ctx, cudaMemcpyAsync(h_total, p->acc, 8, cudaMemcpyDeviceToHost, ctx->stream));
    return RTG_OK;
}

void tc_plan_release(rtg_graph *g) {
    tc_plan_free(g->plan_batched);
    g->plan_batched = nullptr;
}

rtg_status tc_count(rtg_ctx *ctx, rtg_graph *g, rtg_tc_mode mode, uint64_t *total,
                    rtg_timing *t) {
    const Csr &c = g->ori;
    const CountCsr &cc = g->cnt;
    // a graph read from a cache file may hold its counting form alone
    const bool form_only = !c.built && cc.built;
    const uint32_t n = form_only ? cc.n : c.n;
    const uint64_t m = form_only ? cc.m : c.m;
    if (n > 0x7FFFFFFFu || m >= (1ull << 32))
        return fail(ctx, RTG_ERR_INVALID_ARG, "graph too large for 32-bit edge ids");
    t->algo_bytes = 4 * c.work_elems + 8 * c.m;
    if (m == 0) {
        *total = 0;
        return RTG_OK;
    }
    if (mode == RTG_TC_PLAIN) {
        if (!c.built) return fail(ctx, RTG_ERR_STATE, "oriented CSR not built");
        if (kChecked) RTG_TRY(check_csr(ctx, c, false));
        return count_plain(ctx, g, total, t);
    }
    if (kChecked) RTG_TRY(check_count_form(ctx, cc));
    if (mode == RTG_TC_BUCKETED) return count_bucketed(ctx, g, total, t);
    return count_batched(ctx, g, total, t);
}

// ------------------------------------------------------ allocation-free entry point
//
// For callers that must not allocate device memory: code running while another component
// owns the device heap (a framework's caching allocator, a memory pool handed out by the
// host application), code on a path where an allocation's implicit device synchronisation
// is not allowed, or code that may not grow the process's GPU footprint after start-up.
// The PLAIN count runs with its per-edge scratch (edge sources, bucket ids, bucket lists)
// and its counters placed in one file-scope device array instead of cudaMalloc'd buffers.

namespace {

constexpr uint64_t kNoAllocMaxEdges = RTG_NOALLOC_MAX_EDGES;
constexpr size_t kNoAllocCounterBytes = 256;  // total, status, bucket counts/bases/cursors
constexpr size_t kNoAllocScratchBytes =
    kNoAllocCounterBytes + kNoAllocMaxEdges * (4 /*src*/ + 4 /*lists*/ + 1 /*bucket*/);

// Shared by every call on a device and kept between calls; held by every GPU that loads
// the library until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[256] = {};

__global__ void k_noalloc_check(const uint64_t *__restrict__ off, const uint32_t *__restrict__ adj,
                                uint32_t n, uint64_t m, uint32_t *status) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v <= n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t o = off[v];
        if (o > m || (v == 0 && o != 0) || (v == n && o != m) || (v < n && off[v + 1] < o))
            atomicExch(status, 1u);
    }
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < m;
         e += (uint64_t)gridDim.x * blockDim.x)
        if (adj[e] >= n) atomicExch(status, 1u);
}

__global__ void k_noalloc_src(const uint64_t *__restrict__ off, uint32_t n, uint32_t *src) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x)
        for (uint64_t e = off[v]; e < off[v + 1]; ++e) src[e] = (uint32_t)v;
}

}  // namespace

}  // namespace rtg

using namespace rtg;

extern "C" rtg_status rtg_tc_count_device_csr_noalloc(const uint64_t *d_offsets,
                                                       const uint32_t *d_adj, uint32_t n,
                                                       uint64_t m, uint64_t *out_total,
                                                       void *stream) {
    if (!out_total || (n && !d_offsets) || (m && !d_adj)) return RTG_ERR_INVALID_ARG;
    if (m > kNoAllocMaxEdges || n > 0x7FFFFFFEu) return RTG_ERR_INVALID_ARG;
    *out_total = 0;
    if (m == 0 || n == 0) return RTG_OK;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
        cudaGetLastError();
        return RTG_ERR_DEVICE;
    }
    void *base = nullptr;
    {
        // set-up, once per device, with that device current: the array's device address
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
                cudaGetLastError();
                return RTG_ERR_DEVICE;
            }
            g_noalloc_addr[dev] = p;
        }
        base = g_noalloc_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;
    unsigned char *b = (unsigned char *)base;
    unsigned long long *d_total = (unsigned long long *)b;
    uint32_t *d_status = (uint32_t *)(b + 8);
    unsigned long long *d_counts = (unsigned long long *)(b + 16);
    unsigned long long *d_base = d_counts + kPlainBuckets;
    unsigned long long *d_cursor = d_base + kPlainBuckets;
    uint32_t *d_src = (uint32_t *)(b + kNoAllocCounterBytes);
    uint32_t *d_lists = d_src + kNoAllocMaxEdges;
    uint8_t *d_bucket = (uint8_t *)(d_lists + kNoAllocMaxEdges);
    auto cuda_ok = [](cudaError_t e) {
        if (e == cudaSuccess) return true;
        cudaGetLastError();
        return false;
    };
    int sms = 0;
    if (!cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))) return RTG_ERR_DEVICE;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((m + n + 255) / 256, sms * 16ull));
    // counters start at zero on every call (the array keeps the previous call's contents)
    if (!cuda_ok(cudaMemsetAsync(b, 0, kNoAllocCounterBytes, st))) return RTG_ERR_DEVICE;
    k_noalloc_check<<<grid, 256, 0, st>>>(d_offsets, d_adj, n, m, d_status);
    uint32_t bad = 0;
    if (!cuda_ok(cudaGetLastError()) ||
        !cuda_ok(cudaMemcpyAsync(&bad, d_status, 4, cudaMemcpyDeviceToHost, st)) ||
        !cuda_ok(cudaStreamSynchronize(st)))
        return RTG_ERR_DEVICE;
    if (bad) return RTG_ERR_INVALID_ARG;  // offsets not a CSR of m edges, or ids >= n
    k_noalloc_src<<<grid, 256, 0, st>>>(d_offsets, n, d_src);
    k_plain_classify<<<grid, 256, 0, st>>>(d_offsets, d_adj, d_src, m, d_bucket, d_counts);
    unsigned long long hc[kPlainBuckets] = {0};
    if (!cuda_ok(cudaGetLastError()) ||
        !cuda_ok(cudaMemcpyAsync(hc, d_counts, sizeof hc, cudaMemcpyDeviceToHost, st)) ||
        !cuda_ok(cudaStreamSynchronize(st)))
        return RTG_ERR_DEVICE;
    unsigned long long hb[kPlainBuckets], run = 0;
    for (int i = 0; i < kPlainBuckets; ++i) {
        hb[i] = run;
        run += hc[i];
    }
    if (run) {
        if (!cuda_ok(cudaMemcpyAsync(d_base, hb, sizeof hb, cudaMemcpyHostToDevice, st)))
            return RTG_ERR_DEVICE;
        k_plain_scatter<<<grid, 256, 0, st>>>(d_bucket, m, d_base, d_cursor, d_lists);
        for (int i = 0; i < kPlainBuckets; ++i) {
            if (!hc[i]) continue;
            const int gb = (int)std::min<uint64_t>((hc[i] + 7) / 8, 65535);
            if (i < 3)
                k_plain_edges<false><<<gb, 256, 0, st>>>(d_offsets, d_adj, d_src, d_lists + hb[i],
                                                         hc[i], d_total);
            else
                k_plain_edges<true><<<gb, 256, 0, st>>>(d_offsets, d_adj, d_src, d_lists + hb[i],
                                                        hc[i], d_total);
        }
    }
    unsigned long long h = 0;
    if (!cuda_ok(cudaGetLastError()) ||
        !cuda_ok(cudaMemcpyAsync(&h, d_total, 8, cudaMemcpyDeviceToHost, st)) ||
        !cuda_ok(cudaStreamSynchronize(st)))
        return RTG_ERR_DEVICE;
    *out_total = h;
    return RTG_OK;
}
