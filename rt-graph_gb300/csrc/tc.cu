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
//           push-order work on power-law graphs. The items are built once per (graph,
//           schedule); the count (counter resets + the persistent kernel) is one CUDA graph,
//           captured once and replayed. uint64 totals: lane partials -> warp shuffle sum ->
//           block sum -> one atomicAdd per block.
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

// items per vertex v: ceil(indeg(v) / E) when v has out-neighbours and in-neighbours
__global__ void k_item_counts(const uint64_t *__restrict__ off,
                              const uint64_t *__restrict__ in_off, uint32_t n, uint32_t E,
                              uint32_t *cnt) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v <= n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t c = 0;
        if (v < n) {
            uint32_t b = (uint32_t)(off[v + 1] - off[v]);
            uint32_t indeg = (uint32_t)(in_off[v + 1] - in_off[v]);
            c = (b >= 1 && indeg >= 1) ? (indeg + E - 1) / E : 0u;
        }
        cnt[v] = c;
    }
}

__global__ void k_item_fill(const uint64_t *__restrict__ off, const uint64_t *__restrict__ in_off,
                            uint32_t n, uint32_t E, const uint32_t *__restrict__ base,
                            uint64_t *items, unsigned long long *acc) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t b = (uint32_t)(off[v + 1] - off[v]);
        uint32_t indeg = (uint32_t)(in_off[v + 1] - in_off[v]);
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
                              const uint64_t *__restrict__ in_off, uint32_t E, uint64_t cap,
                              uint64_t *out, unsigned long long *cnt) {
    const unsigned long long ni = *nitems;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < ni;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t it = items[i];
        const uint32_t v = (uint32_t)(it >> 32), k0 = (uint32_t)it;
        const uint32_t ne = min(E, (uint32_t)(in_off[v + 1] - in_off[v]) - k0);
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

// acc[0] = total, acc[1] = item queue head, acc[2] = number of items
//
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
        const uint32_t k1 = min(k0 + p.E, (uint32_t)(in_off[v + 1] - kin));
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

}  // namespace

struct TcPlan {
    rtg_tc_mode mode = RTG_TC_BATCHED;
    rtg_config cfg{};
    // batched
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t *items = nullptr;
    uint32_t *vcnt = nullptr;
    void *cub_tmp = nullptr;
    unsigned long long *acc = nullptr;
    cudaEvent_t k0 = nullptr, k1 = nullptr;
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
    dev_free(p->cub_tmp);
    dev_free(p->acc);
    dev_free(p->bucket);
    dev_free(p->lists);
    dev_free(p->bitems);
    if (p->k0) cudaEventDestroy(p->k0);
    if (p->k1) cudaEventDestroy(p->k1);
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
           a.tc_block_warps == b.tc_block_warps && a.tc_blocks_per_sm == b.tc_blocks_per_sm;
}

// Launch shape of the batched count of one graph under one schedule.
struct BatchedShape {
    WarpCfg pc;
    uint32_t W;
    size_t smem;
    int grid, g1;
    uint64_t item_cap;
    size_t cub_bytes;
};

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
    return RTG_OK;
}

// reset -> item counts -> scan -> item fill (acc[2] = number of items)
void enqueue_items(cudaStream_t st, const CountCsr &c, const BatchedShape &bs, uint64_t *items,
                   uint32_t *vcnt, void *cub_tmp, unsigned long long *acc) {
    uint32_t *vbase = vcnt + (c.n + 1ull);
    size_t cub_bytes = bs.cub_bytes;
    cudaMemsetAsync(acc, 0, 8 * sizeof(unsigned long long), st);
    k_item_counts<<<bs.g1, 256, 0, st>>>(c.off, c.in_off, c.n, bs.pc.E, vcnt);
    cub::DeviceScan::ExclusiveSum(cub_tmp, cub_bytes, vcnt, vbase, (int64_t)c.n + 1, st);
    k_item_fill<<<bs.g1, 256, 0, st>>>(c.off, c.in_off, c.n, bs.pc.E, vbase, items, acc);
}

// reset of the total and the queue head (acc[2], the item count, stays) -> [k0] persistent
// count [k1]
void enqueue_count(cudaStream_t st, const CountCsr &c, const BatchedShape &bs,
                   const uint64_t *items, unsigned long long *acc, cudaEvent_t k0, cudaEvent_t k1,
                   bool external_events) {
    cudaMemsetAsync(acc, 0, 2 * sizeof(unsigned long long), st);
    if (k0) {
        if (external_events) cudaEventRecordWithFlags(k0, st, cudaEventRecordExternal);
        else cudaEventRecord(k0, st);
    }
    k_tc_warp<true><<<bs.grid, bs.W * 32, bs.smem, st>>>(c.off, c.adj, c.in_off, c.in_rng, items, acc,
                                                   bs.pc);
    if (k1) {
        if (external_events) cudaEventRecordWithFlags(k1, st, cudaEventRecordExternal);
        else cudaEventRecord(k1, st);
    }
}

constexpr uint64_t kBatchedKernels = 5;  // item counts, scan (init + sweep), item fill, count

void enqueue_batched(cudaStream_t st, const CountCsr &c, const BatchedShape &bs, uint64_t *items,
                     uint32_t *vcnt, void *cub_tmp, unsigned long long *acc) {
    enqueue_items(st, c, bs, items, vcnt, cub_tmp, acc);
    enqueue_count(st, c, bs, items, acc, nullptr, nullptr, false);
}

// A plan's items, built once when the plan is made (the counting form does not change while
// the plan exists), so that a replay launches only the count. Ordering them heaviest first
// by an estimated cost (elements streamed per item) was tried: 2.76 ms on R-MAT-21 against
// 2.72 ms for descending rank order, which keeps the items of one vertex together.
rtg_status plan_items(rtg_ctx *ctx, const CountCsr &c, const BatchedShape &bs, TcPlan *p) {
    enqueue_items(ctx->stream, c, bs, p->items, p->vcnt, p->cub_tmp, p->acc);
    ctx->launches += kBatchedKernels - 1;
    RTG_CUDA(ctx, cudaGetLastError());
    // the plan may be replayed on another context's stream (the serving engine's runs
    // share a graph's plan): the items must be complete before the plan is handed out
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
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
    if ((s = dev_alloc(ctx, (void **)&p->items, bs.item_cap * 8)) != RTG_OK) return bail(s);
    if ((s = dev_alloc(ctx, (void **)&p->vcnt, (c.n + 1ull) * 4 * 2)) != RTG_OK) return bail(s);
    if ((s = dev_alloc(ctx, (void **)&p->acc, 8 * sizeof(unsigned long long))) != RTG_OK)
        return bail(s);
    if ((s = dev_alloc(ctx, &p->cub_tmp, bs.cub_bytes)) != RTG_OK) return bail(s);
    cudaError_t e;
    if ((e = cudaEventCreate(&p->k0)) != cudaSuccess ||
        (e = cudaEventCreate(&p->k1)) != cudaSuccess)
        return bail(cuda_fail(ctx, e, "event", __FILE__, __LINE__));
    if ((s = plan_items(ctx, c, bs, p)) != RTG_OK) return bail(s);
    if ((e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal)) !=
        cudaSuccess)
        return bail(cuda_fail(ctx, e, "capture", __FILE__, __LINE__));
    enqueue_count(ctx->stream, c, bs, p->items, p->acc, p->k0, p->k1, true);
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
    float ms = 0, kms = 0, dms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&kms, p->k0, p->k1);
    cudaEventElapsedTime(&dms, ctx->ev[1], ctx->ev[2]);
    t->count_ms = ms;
    t->main_kernel_ms = kms;
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
    BatchedShape bs{};
    RTG_TRY(batched_shape(ctx, c, dcfg, &bs));
    TcPlan *p = g->plan_bucketed;
    if (!p) {
        p = new TcPlan();
        p->mode = RTG_TC_BUCKETED;
        rtg_status s = dev_alloc(ctx, (void **)&p->items, bs.item_cap * 8);
        if (s == RTG_OK) s = dev_alloc(ctx, (void **)&p->bitems, bs.item_cap * 8 * kItemBuckets);
        if (s == RTG_OK) s = dev_alloc(ctx, (void **)&p->vcnt, (c.n + 1ull) * 4 * 2);
        if (s == RTG_OK) s = dev_alloc(ctx, (void **)&p->acc, 8 * sizeof(unsigned long long));
        if (s == RTG_OK) s = dev_alloc(ctx, &p->cub_tmp, bs.cub_bytes);
        if (s != RTG_OK) {
            tc_plan_free(p);
            return s;
        }
        g->plan_bucketed = p;
    }
    RTG_CUDA(ctx, cudaFuncSetAttribute(k_tc_warp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)bs.smem));
    const uint64_t l0 = ctx->launches;
    unsigned long long *acc = p->acc, *bcnt = p->acc + 3;
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    enqueue_items(ctx->stream, c, bs, p->items, p->vcnt, p->cub_tmp, acc);  // zeroes acc[0..7]
    ctx->launches += kBatchedKernels - 1;
    const int gb = (int)std::max<uint64_t>(1, std::min<uint64_t>((bs.item_cap + 255) / 256,
                                                                  ctx->sm_count * 16ull));
    k_item_bucket<<<gb, 256, 0, ctx->stream>>>(p->items, acc + 2, c.in_off, bs.pc.E, bs.item_cap,
                                               p->bitems, bcnt);
    ctx->launches++;
    RTG_CUDA(ctx, cudaGetLastError());
    unsigned long long hc[kItemBuckets] = {0};
    RTG_CUDA(ctx, cudaMemcpyAsync(hc, bcnt, sizeof hc, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    float kms_sum = 0;
    for (int r = 0; r < kItemBuckets; ++r) {
        if (!hc[r]) continue;
        WarpCfg pc = bs.pc;
        pc.first = 0;
        pc.last = (uint32_t)hc[r];
        const uint64_t blocks = (hc[r] + bs.W - 1) / bs.W;
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
        k_tc_warp<false><<<(unsigned)blocks, bs.W * 32, bs.smem, ctx->stream>>>(
            c.off, c.adj, c.in_off, c.in_rng, p->bitems + r * bs.item_cap, acc, pc);
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

uint64_t tc_plan_estimate_bytes(const rtg_ctx *ctx, const rtg_graph *g) {
    const CountCsr &c = g->cnt;
    const rtg_config cfg = effective_config(ctx, c.m);
    // items + vertex counts + scan temporary (bounded by one word per vertex) + totals
    return (c.m / cfg.tc_item_edges + c.n + 1) * 8 + (c.n + 1ull) * 8 + (c.n + 1ull) * 4 + 4096;
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
    // scratch: acc (64 B) | items | vertex counts and offsets | scan temporary
    char *p = static_cast<char *>(scratch);
    unsigned long long *acc = reinterpret_cast<unsigned long long *>(p);
    uint64_t *items = reinterpret_cast<uint64_t *>(p + 64);
    uint32_t *vcnt = reinterpret_cast<uint32_t *>(items + bs.item_cap);
    void *tmp = reinterpret_cast<void *>(
        (reinterpret_cast<uintptr_t>(vcnt + 2 * (c.n + 1ull)) + 255) & ~(uintptr_t)255);
    if ((uint64_t)(static_cast<char *>(tmp) - p) + bs.cub_bytes > scratch_bytes)
        return fail(ctx, RTG_ERR_INVALID_ARG, "scratch too small for the count");
    enqueue_batched(ctx->stream, c, bs, items, vcnt, tmp, acc);
    RTG_CUDA(ctx, cudaGetLastError());
    ctx->launches += kBatchedKernels;
    RTG_CUDA(ctx, cudaMemcpyAsync(h_total, acc, 8, cudaMemcpyDeviceToHost, ctx->stream));
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
