// Batched pairwise set intersection.
//
// BATCHED (RTG_SI_AUTO): one persistent kernel streams every pair through a per-warp ring of
// shared-memory slots filled by 1-D bulk copies (cp.async.bulk, one mbarrier per slot).
// Warps take 32 pairs at a time from an atomic queue and sort each pair into one of:
//   packed – the pair's two lists fit one slot: consecutive such pairs share a slot (up to
//            kMaxSeg of them), every lane issuing the copies of its own pair;
//   chunked – a balanced pair longer than a slot: cut into K chunks of each list
//            (K = ceil((|A|+|B|) / slot capacity)); its jobs are the chunk pairs (p, q)
//            whose value ranges overlap, visited in merge order from the chunk maxima, so
//            every common element lies in exactly one job;
//   skewed – longer than a slot with |B| > ratio * |A|: the warp binary-searches the short
//            list's elements in the long list straight from global memory.
// Inside a slot the merged sequence of all its segments is split evenly over the 32 lanes
// (merge-path split point by binary search); each lane merges its share serially and counts
// an element of B when it equals the A element consumed just before it, adding the count of
// every segment it touched into a per-warp shared counter. Lists are read once from HBM in
// large asynchronous copies, several slots in flight per warp.
//
// Per-family kernel (PLAIN and the forced families): warps take 32 pairs at a time from an
// atomic queue; lane i loads the ids and list bounds of pair i, then the warp intersects
// the pairs one after another straight from global memory:
//   MERGE  – warp tile merge, both lists streamed (balanced lengths),
//   SEARCH – short-list elements binary-searched in the long list (skewed lengths),
//   HASH   – short list hashed into the warp's shared-memory table, long list streamed
//            through it (the block-bitmap / hash-table baselines' formulation).
// PLAIN picks SEARCH when |long| > ratio * |short|, MERGE otherwise.
//
// Counts are exact set-intersection sizes: what the reference's kernels accumulate per
// (A_i, B_j) with atomics (set_intersection/baseline/bs.cu:138-209, hi.cu:134-181,
// ip.cu:138-287, bi_dynamic.cu:134-169) and what its Check compares against the
// generator's known overlap (set_intersection/utils/util.cpp:39-51).
#include <cub/cub.cuh>

#include <algorithm>

#include "internal.h"
#include "intersect.cuh"
#include "tma.cuh"

namespace rtg {

namespace {

constexpr uint32_t kDefaultSiWarps = 8;
constexpr uint32_t kDefaultSearchRatio = 32;  // PLAIN: per-pair MERGE / SEARCH choice
constexpr uint32_t kDefaultStreamRatio = 8;   // batched: search a pair longer than a slot
constexpr uint32_t kSiHashSlots = 2048;
constexpr uint32_t kDefaultStreamWarps = 8;
constexpr uint32_t kDefaultStageSlots = 2;
constexpr uint32_t kDefaultStageBytes = 4096;

struct SiArgs {
    const uint64_t *off;
    const uint32_t *elems;
    uint64_t nsets;
    const uint32_t *pa;
    const uint32_t *pb;
    uint64_t np;
    uint32_t dense_nb, a_begin, b_begin;
    // several collections in one launch: pair k reads collection pg[k] of gtab
    const uint32_t *pg;
    const SetRef *gtab;
    uint32_t ngraphs;
};

__device__ __forceinline__ bool pair_ids(const SiArgs &s, uint64_t k, uint32_t &x, uint32_t &y) {
    if (s.dense_nb) {
        x = s.a_begin + (uint32_t)(k / s.dense_nb);
        y = s.b_begin + (uint32_t)(k % s.dense_nb);
    } else {
        x = __ldg(s.pa + k);
        y = __ldg(s.pb + k);
    }
    return x < s.nsets && y < s.nsets;
}

// Per-lane prefetch of one pair: list pointers and lengths, short list first.
struct PairRef {
    const uint32_t *A, *B;
    uint32_t a, b;
    bool valid;
};

__device__ __forceinline__ PairRef load_pair(const SiArgs &s, uint64_t k, bool in_range) {
    PairRef r{nullptr, nullptr, 0, 0, false};
    if (!in_range) return r;
    uint32_t x, y;
    const uint64_t *off = s.off;
    const uint32_t *el = s.elems;
    if (s.gtab) {
        const uint32_t g = __ldg(s.pg + k);
        if (g >= s.ngraphs) return r;
        const SetRef gr = s.gtab[g];
        x = __ldg(s.pa + k);
        y = __ldg(s.pb + k);
        if (x >= gr.nsets || y >= gr.nsets) return r;
        off = gr.off;
        el = gr.elems;
    } else if (!pair_ids(s, k, x, y)) {
        return r;
    }
    const uint64_t ox = __ldg(off + x), oy = __ldg(off + y);
    const uint32_t lx = (uint32_t)(__ldg(off + x + 1) - ox), ly = (uint32_t)(__ldg(off + y + 1) - oy);
    if (lx <= ly) {
        r.A = el + ox; r.a = lx; r.B = el + oy; r.b = ly;
    } else {
        r.A = el + oy; r.a = ly; r.B = el + ox; r.b = lx;
    }
    r.valid = true;
    return r;
}

__device__ __forceinline__ const uint32_t *shfl_ptr(const uint32_t *p, int src) {
    return reinterpret_cast<const uint32_t *>(
        __shfl_sync(kFull, (unsigned long long)reinterpret_cast<uintptr_t>(p), src));
}

__device__ __forceinline__ uint32_t intersect_family(const uint32_t *A, uint32_t a,
                                                     const uint32_t *B, uint32_t b,
                                                     uint32_t family, uint32_t ratio,
                                                     uint32_t *tab, uint32_t H, int lane) {
    if (a == 0) return 0;
    uint32_t f = family;
    if (f == RTG_SI_PLAIN) f = ((uint64_t)b > (uint64_t)ratio * a) ? RTG_SI_FORCE_SEARCH : RTG_SI_FORCE_MERGE;
    if (f == RTG_SI_FORCE_SEARCH) return warp_search_count(A, a, B, b, lane);
    if (f == RTG_SI_FORCE_BITMAP && a <= H / 2) {
        uint32_t lg = hash_lg_for(a);
        warp_hash_build(tab, lg, A, a, lane);
        uint32_t c = warp_hash_stream(tab, lg, B, b, lane);
        __syncwarp();
        return c;
    }
    return warp_merge_count(A, a, B, b, lane);
}

__global__ void k_si_count(SiArgs s, uint32_t *out, unsigned long long *head, uint32_t family,
                           uint32_t ratio, uint32_t H, uint32_t *status) {
    extern __shared__ __align__(16) uint32_t smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *tab = smem + warp * H;
    while (true) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(head, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= s.np) break;
        const uint64_t k = base + lane;
        const bool in_range = k < s.np;
        PairRef r = load_pair(s, k, in_range);
        if (in_range && !r.valid) {
            atomicExch(status, kStatusBadInput);
            out[k] = 0;
        }
        unsigned vmask = __ballot_sync(kFull, r.valid);
        uint32_t mine = 0;
        while (vmask) {
            const int e = __ffs(vmask) - 1;
            vmask &= vmask - 1;
            const uint32_t *A = shfl_ptr(r.A, e), *B = shfl_ptr(r.B, e);
            const uint32_t a = __shfl_sync(kFull, r.a, e), b = __shfl_sync(kFull, r.b, e);
            uint32_t c = intersect_family(A, a, B, b, family, ratio, tab, H, lane);
            c = __reduce_add_sync(kFull, c);
            if (lane == e) mine = c;
        }
        if (r.valid) out[k] = mine;
    }
}

// ---------------------------------------------------------------- batched form

struct StreamCfg {
    uint32_t S;           // staging slots per warp
    uint32_t slot_words;  // 32-bit words per slot
    uint32_t meta_off;    // byte offsets of the shared-memory regions
    uint32_t cnt_off;
    uint32_t ring_off;
    uint32_t ratio;       // a pair longer than a slot is searched when |B| > ratio * |A|
    uint32_t skew_pa;     // skewed pairs whose short list has at most this many elements
                          // are staged and streamed (skew jobs); longer ones are searched
    uint32_t probe_polls;  // test hook (0 in normal use): see the start of k_si_stream
    uint32_t probe_tx;
};

// Per-slot job description in shared memory (32-bit words):
//   [0] segments, [1] job kind, [2..3] output index of segment 0's pair (u64), [4] total
//   merged length L of the merged segments, [5] total short-list length LS of the searched
//   segments, [kP + s] first diagonal of segment s among the merged ones (kP + nseg holds
//   L), [kS + s] first short-list element of segment s among the searched ones (kS + nseg
//   holds LS), [kOffA + s] / [kLenA + s] / [kOffB + s] / [kLenB + s] word offset in the slot
//   and length of the segment's two lists, [kOut + s] output index of segment s relative
//   to [2..3]. A segment is merged or searched, never both (its other length is 0).
constexpr uint32_t kMaxSeg = 16;
constexpr uint32_t kP = 8, kS = 25, kOffA = 48, kLenA = 64, kOffB = 80, kLenB = 96, kOut = 112;
constexpr uint32_t kMetaWords = 128;

// Number of elements of the sorted list B (nb >= 1, B[nb] = kEmpty) below x: branch-free
// lower bound over shared memory.
__device__ __forceinline__ uint32_t smem_lower_bound(const uint32_t *B, uint32_t nb, uint32_t x) {
    const uint32_t *first = B;
    uint32_t len = nb;
    while (len > 1) {
        const uint32_t half = len >> 1;
        first = (first[half - 1] < x) ? first + half : first;
        len -= half;
    }
    return (uint32_t)(first - B) + ((*first < x) ? 1u : 0u);
}
enum : uint32_t { kJobPacked = 0, kJobChunk = 1, kJobChunkLast = 2, kJobSkew = 3 };
// Meta words of a skew job (its other fields stay 0): short list length and word offset in
// the slot, long list address (two words) and length, hash table word offset and log2 size.
constexpr uint32_t kSkA = 6, kSkOffA = 7, kSkB = 42, kSkLenB = 44, kSkTab = 45, kSkLg = 46;

// |A ∩ B| for the short list A staged in a slot and the long list B read from global
// memory: A goes into an open-addressing table in the same slot (2^lg words, kEmpty marks
// an empty slot, load at most 1/4), then B streams from HBM in coalesced 16-byte loads (its
// first and last few elements off the 16-byte grid as single words), every element probed
// in the table. Lane-local partial count.
__device__ __forceinline__ uint32_t skew_probe(const uint32_t *tab, uint32_t lg, uint32_t w) {
    const uint32_t mask = (1u << lg) - 1;
    uint32_t sl = hash_slot(w, lg);
    uint32_t x = tab[sl];
    while (x != w && x != kEmpty) {
        sl = (sl + 1) & mask;
        x = tab[sl];
    }
    return x == w ? 1u : 0u;
}

__device__ __forceinline__ uint32_t skew_stream_count(const uint32_t *As, uint32_t na,
                                                      uint32_t *tab, uint32_t lg,
                                                      const uint32_t *__restrict__ B, uint32_t nb,
                                                      int lane) {
    const uint32_t cap = 1u << lg;
    for (uint32_t q = lane; q < cap; q += 32) tab[q] = kEmpty;
    __syncwarp();
    for (uint32_t q = lane; q < na; q += 32) {
        const uint32_t w = As[q];
        uint32_t sl = hash_slot(w, lg);
        while (atomicCAS(&tab[sl], kEmpty, w) != kEmpty) sl = (sl + 1) & (cap - 1);
    }
    __syncwarp();
    uint32_t c = 0;
    const uint32_t head = min(nb, (uint32_t)((16u - (reinterpret_cast<uintptr_t>(B) & 15u)) & 15u) >> 2);
    if ((uint32_t)lane < head) c += skew_probe(tab, lg, __ldg(B + lane));
    const uint4 *B4 = reinterpret_cast<const uint4 *>(B + head);
    const uint32_t n4 = (nb - head) >> 2;
    for (uint32_t i = lane; i < n4; i += 64) {
        const uint4 v = __ldg(B4 + i);
        const bool two = i + 32 < n4;
        uint4 u = make_uint4(0u, 0u, 0u, 0u);
        if (two) u = __ldg(B4 + i + 32);
        c += skew_probe(tab, lg, v.x) + skew_probe(tab, lg, v.y) + skew_probe(tab, lg, v.z) +
             skew_probe(tab, lg, v.w);
        if (two)
            c += skew_probe(tab, lg, u.x) + skew_probe(tab, lg, u.y) +
                 skew_probe(tab, lg, u.z) + skew_probe(tab, lg, u.w);
    }
    const uint32_t t0 = head + 4 * n4;
    if (t0 + lane < nb) c += skew_probe(tab, lg, __ldg(B + t0 + lane));
    return c;
}
enum : uint32_t { kPairZero = 0, kPairPacked = 1, kPairChunked = 2, kPairSkewed = 3 };

// Count the common elements met on diagonals [x0, x1) of the merge of two sorted unique
// lists in shared memory, each followed by a kEmpty sentinel (elements are below kEmpty, so
// an exhausted list never wins a comparison). Ties take A first; a common element is
// counted at the step that consumes its A copy, where both heads are equal. The step is
// branch-free with one shared load.
__device__ __forceinline__ uint32_t merge_range_count(const uint32_t *A, uint32_t na,
                                                      const uint32_t *B, uint32_t nb,
                                                      uint32_t x0, uint32_t x1) {
    uint32_t lo = x0 > nb ? x0 - nb : 0u, hi = min(x0, na);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (A[mid] <= B[x0 - 1 - mid]) lo = mid + 1;
        else hi = mid;
    }
    const uint32_t *pa = A + lo, *pb = B + (x0 - lo);
    uint32_t ai = *pa, bj = *pb, c = 0;
    for (uint32_t d = x0; d < x1; ++d) {
        const bool ta = ai <= bj;
        c += (ai == bj) ? 1u : 0u;
        pa += ta ? 1 : 0;
        pb += ta ? 0 : 1;
        const uint32_t v = *(ta ? pa : pb);
        ai = ta ? v : ai;
        bj = ta ? bj : v;
    }
    return c;
}

// |A ∩ B| for a short list A against a long list B in global memory. The 32 bucket maxima
// of B (one per lane, b/32 elements per bucket) locate each A element's bucket with five
// register shuffles; the element is then binary-searched inside its bucket. Each lane
// searches kSkewIlp A elements in lockstep so their dependent loads overlap (two keep the
// kernel at 80 registers, three resident blocks per SM).
constexpr int kSkewIlp = 2;

__device__ __forceinline__ uint32_t skew_search_count(const uint32_t *__restrict__ A, uint32_t a,
                                                      const uint32_t *__restrict__ B, uint32_t b,
                                                      int lane) {
    const uint32_t step = (b + 31) / 32;
    const uint32_t first = (uint32_t)lane * step;
    const uint32_t smp = first < b ? __ldg(B + min(first + step, b) - 1) : kEmpty;
    const uint32_t iters = 33 - __clz(step);  // lower_bound over step elements converges
    uint32_t c = 0;
    for (uint32_t i0 = 0; i0 < a; i0 += 32 * kSkewIlp) {
        uint32_t x[kSkewIlp], lo[kSkewIlp], hi[kSkewIlp];
#pragma unroll
        for (int k = 0; k < kSkewIlp; ++k) {
            const uint32_t idx = i0 + 32 * k + lane;
            x[k] = idx < a ? __ldg(A + idx) : kEmpty;
            uint32_t pos = 0;  // number of bucket maxima below x (at most 31)
#pragma unroll
            for (uint32_t st = 16; st; st >>= 1)
                if (__shfl_sync(kFull, smp, pos + st - 1) < x[k]) pos += st;
            lo[k] = pos * step;
            hi[k] = idx < a ? min(lo[k] + step, b) : lo[k];
        }
        for (uint32_t it = 0; it < iters; ++it) {
#pragma unroll
            for (int k = 0; k < kSkewIlp; ++k) {
                if (lo[k] < hi[k]) {
                    const uint32_t mid = (lo[k] + hi[k]) >> 1;
                    if (__ldg(B + mid) < x[k]) lo[k] = mid + 1;
                    else hi[k] = mid;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kSkewIlp; ++k)
            c += (i0 + 32 * k + lane < a && lo[k] < b && __ldg(B + lo[k]) == x[k]) ? 1u : 0u;
    }
    return c;
}

__global__ void __maxnreg__(80) k_si_stream(SiArgs s, uint32_t *out, unsigned long long *head, StreamCfg p,
                            uint32_t *status) {
    extern __shared__ __align__(128) unsigned char stage_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t *bars = reinterpret_cast<uint64_t *>(stage_smem) + (size_t)warp * p.S;
    uint32_t *meta =
        reinterpret_cast<uint32_t *>(stage_smem + p.meta_off) + (size_t)warp * p.S * kMetaWords;
    uint32_t *cnt = reinterpret_cast<uint32_t *>(stage_smem + p.cnt_off) + (size_t)warp * kMaxSeg;
    uint32_t *ring =
        reinterpret_cast<uint32_t *>(stage_smem + p.ring_off) + (size_t)warp * p.S * p.slot_words;
    if ((uint32_t)lane < p.S) mbar_init(bars + lane, 1);
    if ((uint32_t)lane < kMaxSeg) cnt[lane] = 0;
    fence_mbar_init();
    __syncwarp();
    const uint32_t CAPE = p.slot_words - 16;  // list elements per chunk job (room for alignment)
    if (p.probe_tx && blockIdx.x == 0 && warp == 0) {
        // test hook: this warp arms its first slot for probe_tx bytes that no copy brings,
        // so the phase never completes and the wait (bounded at probe_polls) runs out; the
        // warp records the timeout and leaves before taking any pairs (the other warps count
        // them all), with nothing in flight
        if (lane == 0) mbar_arrive_expect_tx(bars, p.probe_tx);
        __syncwarp();
        if (!mbar_wait(bars, 0u, p.probe_polls) && lane == 0) atomicExch(status, kStatusTimeout);
        return;
    }

    // One batch of 32 pairs, lane e holding pair base + e: its lists, its kind, the words
    // its widened lists take in a slot and inclusive warp scans of those words, of the
    // merged lengths of packed pairs that are merged and of the short-list lengths of
    // packed pairs that are searched (|B| > ratio * |A|: binary search in the slot).
    struct Batch {
        unsigned long long base;
        PairRef r;
        uint32_t kind, w, sw, sl, ss;
    };
    auto fetch = [&](Batch &bt) {
        unsigned long long b0 = 0;
        if (lane == 0) b0 = atomicAdd(head, 32ull);
        bt.base = __shfl_sync(kFull, b0, 0);
        const uint64_t k = bt.base + lane;
        const bool in = k < s.np;
        bt.r = load_pair(s, k, in);
        if (in && !bt.r.valid) {
            atomicExch(status, kStatusBadInput);
            out[k] = 0;
        }
        bt.kind = kPairZero;
        bt.w = 0;
        uint32_t len = 0, slen = 0;
        if (bt.r.valid && bt.r.a > 0) {
            // words reserved in a slot: each widened list plus one word for its sentinel
            const uint32_t hA = (uint32_t)(reinterpret_cast<uintptr_t>(bt.r.A) & 15u) >> 2;
            const uint32_t hB = (uint32_t)(reinterpret_cast<uintptr_t>(bt.r.B) & 15u) >> 2;
            const uint64_t ww = (((uint64_t)hA + bt.r.a + 4) & ~3ull) + (((uint64_t)hB + bt.r.b + 4) & ~3ull);
            const bool skew = (uint64_t)bt.r.b > (uint64_t)p.ratio * bt.r.a;
            if (ww <= p.slot_words) {
                bt.kind = kPairPacked;
                bt.w = (uint32_t)ww;
                if (skew) slen = bt.r.a;
                else len = bt.r.a + bt.r.b;
            } else if (skew) {
                bt.kind = kPairSkewed;
            } else {
                bt.kind = kPairChunked;
            }
        }
        bt.sw = bt.w;
        bt.sl = len;
        bt.ss = slen;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(kFull, bt.sw, o), y = __shfl_up_sync(kFull, bt.sl, o);
            const uint32_t z = __shfl_up_sync(kFull, bt.ss, o);
            if (lane >= o) {
                bt.sw += x;
                bt.sl += y;
                bt.ss += z;
            }
        }
    };
    Batch cur, nxt;
    fetch(cur);
    fetch(nxt);
    uint32_t e = 0;
    // the chunked pair being cut into jobs (warp-uniform)
    bool open = false;
    const uint32_t *LA = nullptr, *LB = nullptr;  // the pair's short and long list
    uint64_t pk = 0;
    uint32_t a = 0, b = 0, CA = 0, CB = 0, KA = 0, KB = 0, pA = 0, qB = 0, wA = 0, wB = 0;
    uint32_t mxA = kEmpty, mxB = kEmpty;  // lane t: largest element of chunk wA+t / wB+t
    auto chunk_max = [&](uint32_t w, uint32_t K, uint32_t C, const uint32_t *L, uint32_t len) {
        const uint32_t t = w + lane;
        return t < K ? __ldg(L + min((t + 1) * C, len) - 1) : kEmpty;
    };

    // Fill slot `slot` (meta `mt`, barrier `bar`) with the next job; false when none is left.
    auto issue_job = [&](uint32_t *slot, uint32_t *mt, uint64_t *bar) -> bool {
        while (!open) {
            if (cur.base >= s.np) return false;
            const uint32_t nbat = (s.np - cur.base < 32ull) ? (uint32_t)(s.np - cur.base) : 32u;
            if (e >= nbat) {
                cur = nxt;
                e = 0;
                if (cur.base < s.np) fetch(nxt);
                continue;
            }
            const uint32_t kind = __shfl_sync(kFull, cur.kind, e);
            if (kind == kPairZero || kind == kPairPacked) {
                // consecutive packed (and empty) pairs e .. e1-1 that fit one slot together
                const uint32_t baseW = e ? __shfl_sync(kFull, cur.sw, e - 1) : 0u;
                const uint32_t baseL = e ? __shfl_sync(kFull, cur.sl, e - 1) : 0u;
                const uint32_t baseS = e ? __shfl_sync(kFull, cur.ss, e - 1) : 0u;
                const uint32_t me = (uint32_t)lane;
                const bool brk = me > e && (me >= nbat || cur.kind == kPairChunked ||
                                            cur.kind == kPairSkewed || cur.sw - baseW > p.slot_words ||
                                            me >= e + kMaxSeg);
                const unsigned bm = __ballot_sync(kFull, brk);
                const uint32_t e1 = bm ? (uint32_t)(__ffs(bm) - 1) : 32u;
                const uint32_t nseg = e1 - e;
                const uint32_t L = __shfl_sync(kFull, cur.sl, e1 - 1) - baseL;
                const uint32_t LS = __shfl_sync(kFull, cur.ss, e1 - 1) - baseS;
                const bool mine = me >= e && me < e1;
                const bool copies = mine && cur.kind == kPairPacked;
                uint32_t dst = 0, hA = 0, hB = 0, wa = 0, ca = 0, cb = 0;
                if (mine) {
                    const uint32_t sg = me - e;
                    const bool srch = copies && (uint64_t)cur.r.b > (uint64_t)p.ratio * cur.r.a;
                    dst = cur.sw - cur.w - baseW;
                    hA = (uint32_t)(reinterpret_cast<uintptr_t>(cur.r.A) & 15u) >> 2;
                    hB = (uint32_t)(reinterpret_cast<uintptr_t>(cur.r.B) & 15u) >> 2;
                    wa = (hA + cur.r.a + 4) & ~3u;  // A's words + sentinel, 16-byte multiple
                    ca = copies ? (hA + cur.r.a + 3) & ~3u : 0u;  // words copied
                    cb = copies ? (hB + cur.r.b + 3) & ~3u : 0u;
                    mt[kP + sg] = cur.sl - (copies && !srch ? cur.r.a + cur.r.b : 0u) - baseL;
                    mt[kS + sg] = cur.ss - (srch ? cur.r.a : 0u) - baseS;
                    mt[kOffA + sg] = dst + hA;
                    mt[kLenA + sg] = copies ? cur.r.a : 0u;
                    mt[kOffB + sg] = dst + wa + hB;
                    mt[kLenB + sg] = copies ? cur.r.b : 0u;
                    mt[kOut + sg] = me;
                }
                const uint32_t tx = __reduce_add_sync(kFull, (ca + cb) * 4u);
                if (lane == 0) {
                    mt[0] = nseg;
                    mt[1] = kJobPacked;
                    mt[2] = (uint32_t)cur.base;
                    mt[3] = (uint32_t)(cur.base >> 32);
                    mt[4] = L;
                    mt[5] = LS;
                    mt[kP + nseg] = L;
                    mt[kS + nseg] = LS;
                    mbar_arrive_expect_tx(bar, tx);
                }
                __syncwarp();
                if (copies) {
                    const uintptr_t gaa = reinterpret_cast<uintptr_t>(cur.r.A) & ~(uintptr_t)15;
                    const uintptr_t gbb = reinterpret_cast<uintptr_t>(cur.r.B) & ~(uintptr_t)15;
                    bulk_copy_g2s(slot + dst, reinterpret_cast<const void *>(gaa), ca * 4u, bar);
                    bulk_copy_g2s(slot + dst + wa, reinterpret_cast<const void *>(gbb), cb * 4u,
                                  bar);
                }
                e = e1;
                return true;
            }
            LA = shfl_ptr(cur.r.A, e);
            LB = shfl_ptr(cur.r.B, e);
            a = __shfl_sync(kFull, cur.r.a, e);
            b = __shfl_sync(kFull, cur.r.b, e);
            pk = cur.base + e;
            ++e;
            // skewed: stream the long list when that reads fewer sectors than searching it
            // (about b / 8 sectors against about one sector per search step, a x (log2 b - 4)
            // of them after the bucket maxima), else search it from global memory
            if (kind == kPairSkewed && a <= p.skew_pa && b < 8u * a * (27u - __clz(b))) {
                // short list staged in the slot by a bulk copy; the long list is streamed
                // by the consumer (skew_stream_count)
                if (lane == 0) {
                    const uintptr_t ga = reinterpret_cast<uintptr_t>(LA);
                    const uintptr_t gaa = ga & ~(uintptr_t)15;
                    const uint32_t hA = (uint32_t)(ga - gaa) >> 2;
                    const uint32_t bytesA = ((hA + a) * 4u + 15u) & ~15u;
                    uint32_t lg = 5;
                    while ((1u << lg) < 4 * a) ++lg;
                    mt[0] = 0;
                    mt[1] = kJobSkew;
                    mt[2] = (uint32_t)pk;
                    mt[3] = (uint32_t)(pk >> 32);
                    mt[4] = 0;
                    mt[5] = 0;
                    mt[kSkA] = a;
                    mt[kSkOffA] = hA;
                    mt[kSkB] = (uint32_t)reinterpret_cast<uintptr_t>(LB);
                    mt[kSkB + 1] = (uint32_t)(reinterpret_cast<uintptr_t>(LB) >> 32);
                    mt[kSkLenB] = b;
                    mt[kSkTab] = p.skew_pa + 4;
                    mt[kSkLg] = lg;
                    mbar_arrive_expect_tx(bar, bytesA);
                    bulk_copy_g2s(slot, reinterpret_cast<const void *>(gaa), bytesA, bar);
                }
                return true;
            }
            if (kind == kPairSkewed) {
                uint32_t c = skew_search_count(LA, a, LB, b, lane);
                c = __reduce_add_sync(kFull, c);
                if (lane == 0) out[pk] = c;
                continue;
            }
            const uint32_t K = (uint32_t)(((uint64_t)a + b + CAPE - 1) / CAPE);
            CA = (a + K - 1) / K;
            CB = (b + K - 1) / K;
            KA = (a + CA - 1) / CA;
            KB = (b + CB - 1) / CB;
            mxA = chunk_max(0, KA, CA, LA, a);
            mxB = chunk_max(0, KB, CB, LB, b);
            pA = qB = wA = wB = 0;
            open = true;
        }
        // next chunk pair of the open pair, in merge order of the chunk maxima
        const uint32_t a0 = pA * CA, na = min(CA, a - a0);
        const uint32_t b0 = qB * CB, nbb = min(CB, b - b0);
        const uint32_t ma = __shfl_sync(kFull, mxA, pA - wA), mb = __shfl_sync(kFull, mxB, qB - wB);
        if (ma <= mb) ++pA;
        if (mb <= ma) ++qB;
        const bool last = pA >= KA || qB >= KB;
        if (last) {
            open = false;
        } else {
            if (pA - wA >= 32) {
                wA += 32;
                mxA = chunk_max(wA, KA, CA, LA, a);
            }
            if (qB - wB >= 32) {
                wB += 32;
                mxB = chunk_max(wB, KB, CB, LB, b);
            }
        }
        if (lane == 0) {
            const uintptr_t ga = reinterpret_cast<uintptr_t>(LA + a0);
            const uintptr_t gb = reinterpret_cast<uintptr_t>(LB + b0);
            const uintptr_t gaa = ga & ~(uintptr_t)15, gbb = gb & ~(uintptr_t)15;
            const uint32_t hA = (uint32_t)(ga - gaa) >> 2, hB = (uint32_t)(gb - gbb) >> 2;
            const uint32_t bytesA = ((hA + na) * 4u + 15u) & ~15u;
            const uint32_t resA = ((hA + na + 1) * 4u + 15u) & ~15u;  // + sentinel word
            const uint32_t bytesB = ((hB + nbb) * 4u + 15u) & ~15u;
            mt[0] = 1;
            mt[1] = last ? kJobChunkLast : kJobChunk;
            mt[2] = (uint32_t)pk;
            mt[3] = (uint32_t)(pk >> 32);
            mt[4] = na + nbb;
            mt[5] = 0;
            mt[kP] = 0;
            mt[kP + 1] = na + nbb;
            mt[kS] = 0;
            mt[kS + 1] = 0;
            mt[kOffA] = hA;
            mt[kLenA] = na;
            mt[kOffB] = resA / 4 + hB;
            mt[kLenB] = nbb;
            mt[kOut] = 0;
            mbar_arrive_expect_tx(bar, bytesA + bytesB);
            bulk_copy_g2s(slot, reinterpret_cast<const void *>(gaa), bytesA, bar);
            bulk_copy_g2s(slot + resA / 4, reinterpret_cast<const void *>(gbb), bytesB, bar);
        }
        return true;
    };

    uint32_t inflight = 0, sw = 0, sr = 0, phase = 0, acc = 0;
    bool jobs = true;
    while (true) {
        while (inflight < p.S && jobs) {
            if (!issue_job(ring + (size_t)sw * p.slot_words, meta + sw * kMetaWords, bars + sw)) {
                jobs = false;
                break;
            }
            sw = (sw + 1 == p.S) ? 0 : sw + 1;
            ++inflight;
        }
        if (inflight == 0) break;
        __syncwarp();
        if (!mbar_wait(bars + sr, (phase >> sr) & 1u)) {
            if (lane == 0) atomicExch(status, kStatusTimeout);
            for (uint32_t q = 1; q < inflight; ++q) {  // bounded drain of the others
                const uint32_t s2 = (sr + q) % p.S;
                mbar_wait(bars + s2, (phase >> s2) & 1u);
            }
            break;
        }
        phase ^= 1u << sr;
        const uint32_t *mt = meta + sr * kMetaWords;
        uint32_t *slot = ring + (size_t)sr * p.slot_words;
        const uint32_t nseg = mt[0], kind = mt[1], L = mt[4];
        // a sentinel after every list of the slot (its reserved word; copies have landed)
        if ((uint32_t)lane < nseg && mt[kLenA + lane]) {
            slot[mt[kOffA + lane] + mt[kLenA + lane]] = kEmpty;
            slot[mt[kOffB + lane] + mt[kLenB + lane]] = kEmpty;
        }
        __syncwarp();
        uint32_t d0 = (uint32_t)(((uint64_t)L * (uint32_t)lane) >> 5);
        const uint32_t d1 = (uint32_t)(((uint64_t)L * (uint32_t)(lane + 1)) >> 5);
        if (d0 < d1) {
            // last segment starting at or before d0 (P is non-decreasing, P[nseg] = L > d0)
            uint32_t sg = 0;
#pragma unroll
            for (uint32_t st = kMaxSeg / 2; st; st >>= 1)
                if (sg + st < nseg && mt[kP + sg + st] <= d0) sg += st;
            while (d0 < d1) {
                const uint32_t ps = mt[kP + sg], pe = mt[kP + sg + 1];
                const uint32_t x1 = min(d1, pe) - ps;
                const uint32_t c = merge_range_count(slot + mt[kOffA + sg], mt[kLenA + sg],
                                                     slot + mt[kOffB + sg], mt[kLenB + sg],
                                                     d0 - ps, x1);
                if (c) atomicAdd(cnt + sg, c);
                d0 = ps + x1;
                ++sg;
                while (d0 < d1 && mt[kP + sg + 1] <= d0) ++sg;  // skip empty segments
            }
        }
        // searched segments: lane t takes short-list elements t, t + 32, ... of all of them
        // and finds each in its long list (both lists in the slot, long one sentinel-ended)
        const uint32_t LS = mt[5];
        for (uint32_t t = (uint32_t)lane; t < LS; t += 32) {
            uint32_t sg = 0;  // last segment whose first searched element is at or before t
#pragma unroll
            for (uint32_t st = kMaxSeg / 2; st; st >>= 1)
                if (sg + st < nseg && mt[kS + sg + st] <= t) sg += st;
            const uint32_t x = slot[mt[kOffA + sg] + (t - mt[kS + sg])];
            const uint32_t *B = slot + mt[kOffB + sg];
            if (B[smem_lower_bound(B, mt[kLenB + sg], x)] == x) atomicAdd(cnt + sg, 1u);
        }
        __syncwarp();
        const uint64_t obase = (uint64_t)mt[2] | ((uint64_t)mt[3] << 32);
        if (kind == kJobSkew) {
            const uint32_t *LBp = reinterpret_cast<const uint32_t *>(
                (uint64_t)mt[kSkB] | ((uint64_t)mt[kSkB + 1] << 32));
            uint32_t c = skew_stream_count(slot + mt[kSkOffA], mt[kSkA], slot + mt[kSkTab],
                                           mt[kSkLg], LBp, mt[kSkLenB], lane);
            c = __reduce_add_sync(kFull, c);
            if (lane == 0) out[obase] = c;
        } else if (kind == kJobPacked) {
            if ((uint32_t)lane < nseg) {
                out[obase + mt[kOut + lane]] = cnt[lane];
                cnt[lane] = 0;
            }
        } else if (lane == 0) {
            acc += cnt[0];
            cnt[0] = 0;
            if (kind == kJobChunkLast) {
                out[obase] = acc;
                acc = 0;
            }
        }
        __syncwarp();
        fence_proxy_async_smem();
        sr = (sr + 1 == p.S) ? 0 : sr + 1;
        --inflight;
    }
}

__global__ void k_si_write(SiArgs s, const uint64_t *__restrict__ out_off, uint32_t *out_elems) {
    const int lane = threadIdx.x & 31;
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t k = warp; k < s.np; k += nwarps) {
        uint32_t x, y;
        if (!pair_ids(s, k, x, y)) continue;
        uint64_t ox = s.off[x], oy = s.off[y];
        uint32_t lx = (uint32_t)(s.off[x + 1] - ox), ly = (uint32_t)(s.off[y + 1] - oy);
        warp_merge_write(s.elems + ox, lx, s.elems + oy, ly, out_elems + out_off[k], lane);
    }
}

__global__ void k_widen(const uint32_t *__restrict__ in, uint64_t n, uint64_t *out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

SiArgs make_args(const PairSpec &ps) {
    SiArgs a;
    a.off = ps.off;
    a.elems = ps.elems;
    a.nsets = ps.nsets;
    a.pa = ps.pa;
    a.pb = ps.pb;
    a.np = ps.npairs;
    a.dense_nb = ps.dense_nb;
    a.a_begin = ps.a_begin;
    a.b_begin = ps.b_begin;
    a.pg = ps.pg;
    a.gtab = ps.gtab;
    a.ngraphs = ps.ngraphs;
    return a;
}

}  // namespace

rtg_status si_count_device(rtg_ctx *ctx, const PairSpec &ps, uint32_t *d_out, uint32_t family,
                           float *kernel_ms, uint64_t *launches) {
    if (ps.npairs == 0) {
        if (kernel_ms) *kernel_ms = 0;
        return RTG_OK;
    }
    const rtg_config &cf = ctx->cfg;
    const uint32_t ratio = cf.si_search_ratio ? cf.si_search_ratio : kDefaultSearchRatio;
    if (family == RTG_SI_AUTO) {
        const uint32_t W = cf.si_block_warps ? cf.si_block_warps : kDefaultStreamWarps;
        StreamCfg sc{};
        sc.S = cf.si_stage_slots ? cf.si_stage_slots : kDefaultStageSlots;
        const uint32_t slot_bytes = cf.si_stage_bytes ? cf.si_stage_bytes : kDefaultStageBytes;
        sc.slot_words = slot_bytes / 4;
        sc.ratio = cf.si_search_ratio ? cf.si_search_ratio : kDefaultStreamRatio;
        // a skew job holds the short list (at most skew_pa elements, widened) and a table
        // of 4 x skew_pa words after it: the largest power of two with 5 x + 20 <= slot words
        sc.skew_pa = 0;
        if (cf.si_skew_stream) {
            sc.skew_pa = 16;
            while (5 * (2 * sc.skew_pa) + 20 <= sc.slot_words) sc.skew_pa *= 2;
        }
        // the test hook of rtg_debug_si_wait_limit applies to one launch
        sc.probe_polls = ctx->dbg_wait_polls ? ctx->dbg_wait_polls : kMaxWaitIters;
        sc.probe_tx = ctx->dbg_extra_tx;
        ctx->dbg_wait_polls = ctx->dbg_extra_tx = 0;
        sc.meta_off = ((W * sc.S * 8) + 127u) & ~127u;
        sc.cnt_off = (sc.meta_off + W * sc.S * kMetaWords * 4 + 127u) & ~127u;
        sc.ring_off = (sc.cnt_off + W * kMaxSeg * 4 + 127u) & ~127u;
        const size_t smem = (size_t)sc.ring_off + (size_t)W * sc.S * slot_bytes;
        if ((int)smem > ctx->smem_optin)
            return fail(ctx, RTG_ERR_INVALID_ARG, "SI schedule needs %zu B of shared memory", smem);
        RTG_CUDA(ctx, cudaFuncSetAttribute(k_si_stream, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
        int per_sm = 0;
        RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_si_stream, W * 32, smem));
        if (cf.si_blocks_per_sm) per_sm = std::min<int>(per_sm, (int)cf.si_blocks_per_sm);
        per_sm = std::max(per_sm, 1);
        const uint64_t need = (ps.npairs + 32ull * W - 1) / (32ull * W);
        const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)ctx->sm_count * per_sm));
        unsigned long long *head = ctx->d_scalars + 8;
        // one CUDA graph per context: the queue-head reset and the persistent kernel, captured
        // on the first launch; later launches set the kernel node's grid, shared memory and
        // arguments (pairs, outputs, schedule) and replay it
        SiArgs args = make_args(ps);
        uint32_t *status = ctx->d_status;
        if (!ctx->si_exec) {
            cudaGraph_t gr = nullptr;
            RTG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            cudaMemsetAsync(head, 0, 8, ctx->stream);
            k_si_stream<<<grid, W * 32, smem, ctx->stream>>>(args, d_out, head, sc, status);
            const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &gr);
            if (ce != cudaSuccess) return cuda_fail(ctx, ce, "SI graph capture", __FILE__, __LINE__);
            cudaGraphExec_t ex = nullptr;
            const cudaError_t ie = cudaGraphInstantiate(&ex, gr, 0);
            if (ie != cudaSuccess) {
                cudaGraphDestroy(gr);
                return cuda_fail(ctx, ie, "SI graph instantiate", __FILE__, __LINE__);
            }
            size_t nn = 0;
            cudaGraphGetNodes(gr, nullptr, &nn);
            std::vector<cudaGraphNode_t> nodes(nn);
            cudaGraphGetNodes(gr, nodes.data(), &nn);
            for (auto nd : nodes) {
                cudaGraphNodeType t;
                if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel)
                    ctx->si_knode = nd;
            }
            ctx->si_graph = gr;
            ctx->si_exec = ex;
            if (!ctx->si_knode) return fail(ctx, RTG_ERR_DEVICE, "SI graph has no kernel node");
        } else {
            void *kargs[] = {&args, &d_out, &head, &sc, &status};
            cudaKernelNodeParams kp{};
            kp.func = reinterpret_cast<void *>(k_si_stream);
            kp.gridDim = dim3((unsigned)grid);
            kp.blockDim = dim3(W * 32);
            kp.sharedMemBytes = (unsigned)smem;
            kp.kernelParams = kargs;
            RTG_CUDA(ctx, cudaGraphExecKernelNodeSetParams(ctx->si_exec, ctx->si_knode, &kp));
        }
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
        RTG_CUDA(ctx, cudaGraphLaunch(ctx->si_exec, ctx->stream));
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
        (*launches)++;
        if (kernel_ms) {
            RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[7]));
            cudaEventElapsedTime(kernel_ms, ctx->ev[6], ctx->ev[7]);
        }
        return RTG_OK;
    }
    const uint32_t W = cf.si_block_warps ? cf.si_block_warps : kDefaultSiWarps;
    const uint32_t H = (family == RTG_SI_FORCE_BITMAP) ? kSiHashSlots : 0;
    const size_t smem = (size_t)W * H * 4;
    if ((int)smem > ctx->smem_optin)
        return fail(ctx, RTG_ERR_INVALID_ARG, "SI schedule needs %zu B of shared memory", smem);
    RTG_CUDA(ctx, cudaFuncSetAttribute(k_si_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)std::max<size_t>(smem, 0)));
    int per_sm = 0;
    RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_si_count, W * 32, smem));
    per_sm = std::max(per_sm, 1);
    uint64_t need_blocks = (ps.npairs + 32 * W - 1) / (32 * W);
    int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(need_blocks, (uint64_t)ctx->sm_count * per_sm));
    unsigned long long *head = ctx->d_scalars + 8;
    RTG_CUDA(ctx, cudaMemsetAsync(head, 0, 8, ctx->stream));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
    k_si_count<<<grid, W * 32, smem, ctx->stream>>>(make_args(ps), d_out, head, family, ratio, H,
                                                    ctx->d_status);
    RTG_CUDA(ctx, cudaGetLastError());
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
    (*launches)++;
    if (kernel_ms) {
        RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[7]));
        cudaEventElapsedTime(kernel_ms, ctx->ev[6], ctx->ev[7]);
    }
    return RTG_OK;
}

rtg_status si_materialize_device(rtg_ctx *ctx, const PairSpec &ps, uint64_t *d_out_off,
                                 uint32_t *d_out_elems, uint64_t capacity, uint64_t *needed,
                                 uint64_t *launches) {
    const uint64_t np = ps.npairs;
    *needed = 0;
    // per-pair counts, widened to uint64, exclusive scan -> output offsets
    void *p = nullptr;
    RTG_TRY(scratch(ctx, 1, (np + 1) * 12 + 16, &p));
    uint32_t *cnt = (uint32_t *)p;
    uint64_t *wide = (uint64_t *)(((uintptr_t)(cnt + np + 1) + 15) & ~(uintptr_t)15);
    RTG_CUDA(ctx, cudaMemsetAsync(cnt, 0, (np + 1) * 4, ctx->stream));
    RTG_TRY(si_count_device(ctx, ps, cnt, RTG_SI_AUTO, nullptr, launches));
    k_widen<<<(int)std::max<uint64_t>(1, std::min<uint64_t>((np + 256) / 256, ctx->sm_count * 16ull)),
              256, 0, ctx->stream>>>(cnt, np + 1, wide);
    RTG_CUDA(ctx, cudaGetLastError());
    (*launches)++;
    size_t bytes = 0;
    RTG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, bytes, wide, d_out_off, (int64_t)np + 1,
                                                ctx->stream));
    void *tmp = nullptr;
    RTG_TRY(scratch(ctx, 0, bytes, &tmp));
    RTG_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, bytes, wide, d_out_off, (int64_t)np + 1,
                                                ctx->stream));
    (*launches) += 2;
    uint64_t total = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&total, d_out_off + np, 8, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *needed = total;
    if (total > capacity) return RTG_ERR_INVALID_ARG;
    if (np && total) {
        int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((np + 7) / 8, ctx->sm_count * 32ull));
        k_si_write<<<grid, 256, 0, ctx->stream>>>(make_args(ps), d_out_off, d_out_elems);
        RTG_CUDA(ctx, cudaGetLastError());
        (*launches)++;
    }
    return RTG_OK;
}

}  // namespace rtg
