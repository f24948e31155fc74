// Batched pairwise set intersection.
//
// BATCHED (RTG_SI_AUTO): one persistent kernel streams every pair through rings of
// shared-memory slots filled by 1-D bulk copies (cp.async.bulk, one mbarrier per slot), in
// one of two forms (si_form): producer/consumer (k_si_pc, the default: one warp per block
// forms the jobs and issues their copies into a ring shared by the block's merging warps)
// or per-warp rings (k_si_stream: every warp forms its own jobs and merges them). Pairs
// are taken 32 at a time from an atomic queue and sorted into one of:
//   packed – the pair's two lists fit one slot: consecutive such pairs share a slot (up to
//            kMaxSeg of them), every lane issuing the copies of its own pair;
//   chunked – a balanced pair longer than a slot: cut into K chunks of each list
//            (K = ceil((|A|+|B|) / slot capacity)); its jobs are the chunk pairs (p, q)
//            whose value ranges overlap, visited in merge order from the chunk maxima, so
//            every common element lies in exactly one job;
//   skewed – longer than a slot with |B| > ratio * |A|: a warp binary-searches the short
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
constexpr uint32_t kDefaultSiForm = 2;         // batched form (si_form): producer/consumer
constexpr uint32_t kDefaultPcWarps = 3;        // producer/consumer: merging warps per block
constexpr uint32_t kDefaultPcSlots = 5;        // producer/consumer: ring slots per block
constexpr uint32_t kDefaultPcSlotBytes = 8192; // producer/consumer: bytes per ring slot

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

// The ids of pair k as stored (pair arrays, dense A x B, or collection + pair arrays): the
// first, independent loads of a pair, which a caller may issue well ahead of resolve_pair.
struct PairIds {
    uint32_t x, y, g;
};

__device__ __forceinline__ PairIds load_ids(const SiArgs &s, uint64_t k, bool in_range) {
    PairIds id{0u, 0u, 0u};
    if (!in_range) return id;
    if (s.dense_nb) {
        id.x = s.a_begin + (uint32_t)(k / s.dense_nb);
        id.y = s.b_begin + (uint32_t)(k % s.dense_nb);
    } else {
        id.x = __ldg(s.pa + k);
        id.y = __ldg(s.pb + k);
        if (s.gtab) id.g = __ldg(s.pg + k);
    }
    return id;
}

// The pair's lists from its ids (validated against the collection): offsets loaded, short
// list first.
__device__ __forceinline__ PairRef resolve_pair(const SiArgs &s, bool in_range, PairIds id) {
    PairRef r{nullptr, nullptr, 0, 0, false};
    if (!in_range) return r;
    const uint32_t x = id.x, y = id.y;
    const uint64_t *off = s.off;
    const uint32_t *el = s.elems;
    if (s.gtab) {
        if (id.g >= s.ngraphs) return r;
        const SetRef gr = s.gtab[id.g];
        if (x >= gr.nsets || y >= gr.nsets) return r;
        off = gr.off;
        el = gr.elems;
    } else if (x >= s.nsets || y >= s.nsets) {
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

__device__ __forceinline__ PairRef load_pair(const SiArgs &s, uint64_t k, bool in_range) {
    return resolve_pair(s, in_range, load_ids(s, k, in_range));
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

// Per-slot job description in shared memory (32-bit words), written by the job's producer:
//   [0] segments, [1] job kind, [2..3] output index of segment 0's pair (u64; segment s
//   is pair [2..3] + s), [kOffA + s] / [kLenA + s] / [kOffB + s] / [kLenB + s] word offset
//   in the slot and length of the segment's two lists;
// and by its consumer before the merge: [kP + s] first diagonal of segment s among the
// merged ones (kP + nseg holds their total L), [kS + s] first short-list element of segment
// s among the searched ones (kS + nseg holds their total LS). A segment is searched when
// |B| > ratio * |A| (binary search of A's elements in B inside the slot), else merged.
constexpr uint32_t kMaxSeg = 16;
constexpr uint32_t kP = 8, kS = 25, kOffA = 48, kLenA = 64, kOffB = 80, kLenB = 96;
constexpr uint32_t kMetaWords = 112;

// Number of elements of the sorted list B (nb >= 1, B[nb] = kEmpty) below x: branch-free
// lower bound over shared memory.
__device__ __forceinline__ uint32_t smem_lower_bound(const uint32_t *B, uint32_t nb, uint32_t x) {
    const uint32_t b0 = smem_u32(B);
    uint32_t first = b0, len = nb;
    while (len > 1) {
        const uint32_t half = len >> 1;
        first = (lds_u32(first + 4 * (half - 1)) < x) ? first + 4 * half : first;
        len -= half;
    }
    return (first - b0) / 4 + ((lds_u32(first) < x) ? 1u : 0u);
}
enum : uint32_t { kJobPacked = 0, kJobChunk = 1, kJobChunkLast = 2, kJobSkew = 3 };
// meta word of a chunk job holding its accumulator entry (producer/consumer form)
constexpr uint32_t kCkEnt = 6;
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
    // 32-bit shared-memory byte addresses throughout (2 % faster than generic pointers)
    const uint32_t sA = smem_u32(A), sB = smem_u32(B);
    uint32_t lo = x0 > nb ? x0 - nb : 0u, hi = min(x0, na);
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (lds_u32(sA + 4 * mid) <= lds_u32(sB + 4 * (x0 - 1 - mid))) lo = mid + 1;
        else hi = mid;
    }
    uint32_t ia = sA + 4 * lo, ib = sB + 4 * (x0 - lo);
    uint32_t ai = lds_u32(ia), bj = lds_u32(ib), c = 0;
    for (uint32_t n = x1 - x0; n; --n) {
        const bool ta = ai <= bj;
        c += (ai == bj) ? 1u : 0u;
        const uint32_t inc = ta ? 4u : 0u;
        ia += inc;
        ib += 4u - inc;
        const uint32_t v = lds_u32(ta ? ia : ib);
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

template <int kIlp = kSkewIlp>
__device__ __forceinline__ uint32_t skew_search_count(const uint32_t *__restrict__ A, uint32_t a,
                                                      const uint32_t *__restrict__ B, uint32_t b,
                                                      int lane) {
    const uint32_t step = (b + 31) / 32;
    const uint32_t first = (uint32_t)lane * step;
    const uint32_t smp = first < b ? __ldg(B + min(first + step, b) - 1) : kEmpty;
    const uint32_t iters = 33 - __clz(step);  // lower_bound over step elements converges
    uint32_t c = 0;
    for (uint32_t i0 = 0; i0 < a; i0 += 32 * kIlp) {
        uint32_t x[kIlp], lo[kIlp], hi[kIlp];
#pragma unroll
        for (int k = 0; k < kIlp; ++k) {
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
            for (int k = 0; k < kIlp; ++k) {
                if (lo[k] < hi[k]) {
                    const uint32_t mid = (lo[k] + hi[k]) >> 1;
                    if (__ldg(B + mid) < x[k]) lo[k] = mid + 1;
                    else hi[k] = mid;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kIlp; ++k)
            c += (i0 + 32 * k + lane < a && lo[k] < b && __ldg(B + lo[k]) == x[k]) ? 1u : 0u;
    }
    return c;
}

// One batch of 32 pairs taken from the queue, lane e holding pair base + e: its lists, its
// kind, the words its widened lists take in a slot and the inclusive warp scan of those
// words.
struct Batch {
    unsigned long long base;
    PairRef r;
    uint32_t kind, w, sw;
};

// Batch from its base and its pairs' ids (loaded ahead with load_ids).
__device__ __forceinline__ void batch_from_ids(Batch &bt, unsigned long long base, PairIds id,
                                               const SiArgs &s, uint32_t *out, uint32_t *status,
                                               uint32_t slot_words, uint32_t ratio, int lane) {
    bt.base = base;
    const uint64_t k = bt.base + lane;
    const bool in = k < s.np;
    bt.r = resolve_pair(s, in, id);
    if (in && !bt.r.valid) {
        atomicExch(status, kStatusBadInput);
        out[k] = 0;
    }
    bt.kind = kPairZero;
    bt.w = 0;
    if (bt.r.valid && bt.r.a > 0) {
        // words reserved in a slot: each widened list plus one word for its sentinel
        const uint32_t hA = (uint32_t)(reinterpret_cast<uintptr_t>(bt.r.A) & 15u) >> 2;
        const uint32_t hB = (uint32_t)(reinterpret_cast<uintptr_t>(bt.r.B) & 15u) >> 2;
        const uint64_t ww =
            (((uint64_t)hA + bt.r.a + 4) & ~3ull) + (((uint64_t)hB + bt.r.b + 4) & ~3ull);
        const bool skew = (uint64_t)bt.r.b > (uint64_t)ratio * bt.r.a;
        if (ww <= slot_words) {
            bt.kind = kPairPacked;
            bt.w = (uint32_t)ww;
        } else if (skew) {
            bt.kind = kPairSkewed;
        } else {
            bt.kind = kPairChunked;
        }
    }
    bt.sw = bt.w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(kFull, bt.sw, o);
        if (lane >= o) bt.sw += x;
    }
}

__device__ __forceinline__ void fetch_batch(Batch &bt, const SiArgs &s, uint32_t *out,
                                            unsigned long long *head, uint32_t *status,
                                            uint32_t slot_words, uint32_t ratio, int lane) {
    unsigned long long b0 = 0;
    if (lane == 0) b0 = atomicAdd(head, 32ull);
    b0 = __shfl_sync(kFull, b0, 0);
    batch_from_ids(bt, b0, load_ids(s, b0 + lane, b0 + lane < s.np), s, out, status, slot_words,
                   ratio, lane);
}

// A packed job into `slot` (meta `mt`, barrier `bar`): the consecutive packed (and empty)
// pairs e .. e1-1 of the batch that fit one slot together, at most kMaxSeg of them, every
// lane issuing the copies of its own pair at a warp-scanned offset. Returns e1.
__device__ __forceinline__ uint32_t form_packed(const Batch &cur, uint32_t e, uint32_t nbat,
                                                uint32_t slot_words, uint32_t *slot, uint32_t *mt,
                                                uint64_t *bar, int lane) {
    const uint32_t baseW = e ? __shfl_sync(kFull, cur.sw, e - 1) : 0u;
    const uint32_t me = (uint32_t)lane;
    const bool brk = me > e && (me >= nbat || cur.kind == kPairChunked ||
                                cur.kind == kPairSkewed || cur.sw - baseW > slot_words ||
                                me >= e + kMaxSeg);
    const unsigned bm = __ballot_sync(kFull, brk);
    const uint32_t e1 = bm ? (uint32_t)(__ffs(bm) - 1) : 32u;
    const bool mine = me >= e && me < e1;
    const bool copies = mine && cur.kind == kPairPacked;
    uint32_t dst = 0, wa = 0, ca = 0, cb = 0;
    if (mine) {
        const uint32_t sg = me - e;
        dst = cur.sw - cur.w - baseW;
        const uint32_t hA = (uint32_t)(reinterpret_cast<uintptr_t>(cur.r.A) & 15u) >> 2;
        const uint32_t hB = (uint32_t)(reinterpret_cast<uintptr_t>(cur.r.B) & 15u) >> 2;
        wa = (hA + cur.r.a + 4) & ~3u;  // A's words + sentinel, 16-byte multiple
        ca = copies ? (hA + cur.r.a + 3) & ~3u : 0u;  // words copied
        cb = copies ? (hB + cur.r.b + 3) & ~3u : 0u;
        mt[kOffA + sg] = dst + hA;
        mt[kLenA + sg] = copies ? cur.r.a : 0u;
        mt[kOffB + sg] = dst + wa + hB;
        mt[kLenB + sg] = copies ? cur.r.b : 0u;
    }
    const uint32_t tx = __reduce_add_sync(kFull, (ca + cb) * 4u);
    __syncwarp();  // every lane's meta words before lane 0's arrival publishes the job
    if (lane == 0) {
        const unsigned long long ob = cur.base + e;
        mt[0] = e1 - e;
        mt[1] = kJobPacked;
        mt[2] = (uint32_t)ob;
        mt[3] = (uint32_t)(ob >> 32);
        mbar_arrive_expect_tx(bar, tx);
    }
    __syncwarp();
    if (copies) {
        const uintptr_t gaa = reinterpret_cast<uintptr_t>(cur.r.A) & ~(uintptr_t)15;
        const uintptr_t gbb = reinterpret_cast<uintptr_t>(cur.r.B) & ~(uintptr_t)15;
        bulk_copy_g2s(slot + dst, reinterpret_cast<const void *>(gaa), ca * 4u, bar);
        bulk_copy_g2s(slot + dst + wa, reinterpret_cast<const void *>(gbb), cb * 4u, bar);
    }
    return e1;
}

// A skewed pair staged for streaming: its short list (at most skew_pa elements) bulk-copied
// into the slot with room for an open-addressing table after it; the long list is streamed
// from global memory by the consumer (skew_stream_count).
__device__ __forceinline__ void form_skew_stream(const uint32_t *LA, uint32_t a, const uint32_t *LB,
                                                 uint32_t b, uint64_t pk, uint32_t skew_pa,
                                                 uint32_t *slot, uint32_t *mt, uint64_t *bar,
                                                 int lane) {
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
        mt[kSkA] = a;
        mt[kSkOffA] = hA;
        mt[kSkB] = (uint32_t)reinterpret_cast<uintptr_t>(LB);
        mt[kSkB + 1] = (uint32_t)(reinterpret_cast<uintptr_t>(LB) >> 32);
        mt[kSkLenB] = b;
        mt[kSkTab] = skew_pa + 4;
        mt[kSkLg] = lg;
        mbar_arrive_expect_tx(bar, bytesA);
        bulk_copy_g2s(slot, reinterpret_cast<const void *>(gaa), bytesA, bar);
    }
}

// The chunk jobs of one balanced pair longer than a slot (warp-uniform state): K chunks of
// each list (K = ceil((|A| + |B|) / chunk capacity)); the jobs are the chunk pairs (p, q)
// whose value ranges overlap, visited in merge order of the chunk maxima, so every common
// element lies in exactly one job.
struct ChunkCut {
    bool open = false;
    const uint32_t *LA = nullptr, *LB = nullptr;  // the pair's short and long list
    uint64_t pk = 0;
    uint32_t a = 0, b = 0, CA = 0, CB = 0, KA = 0, KB = 0, pA = 0, qB = 0, wA = 0, wB = 0;
    uint32_t mxA = kEmpty, mxB = kEmpty;  // lane t: largest element of chunk wA+t / wB+t

    __device__ __forceinline__ static uint32_t chunk_max(uint32_t w, uint32_t K, uint32_t C,
                                                         const uint32_t *L, uint32_t len,
                                                         int lane) {
        const uint32_t t = w + lane;
        return t < K ? __ldg(L + min((t + 1) * C, len) - 1) : kEmpty;
    }

    __device__ __forceinline__ void start(const uint32_t *la, uint32_t na, const uint32_t *lb,
                                          uint32_t nb, uint64_t k, uint32_t cape, int lane) {
        LA = la;
        LB = lb;
        a = na;
        b = nb;
        pk = k;
        const uint32_t K = (uint32_t)(((uint64_t)a + b + cape - 1) / cape);
        CA = (a + K - 1) / K;
        CB = (b + K - 1) / K;
        KA = (a + CA - 1) / CA;
        KB = (b + CB - 1) / CB;
        mxA = chunk_max(0, KA, CA, LA, a, lane);
        mxB = chunk_max(0, KB, CB, LB, b, lane);
        pA = qB = wA = wB = 0;
        open = true;
    }

    // Issue the next chunk job into `slot` (meta `mt`, barrier `bar`); with `ent` set, lane 0
    // first records entry index `ei` in the meta and adds one pending job to *ent. Returns
    // true for the pair's last job (the cut is then closed).
    __device__ __forceinline__ bool next(uint32_t *slot, uint32_t *mt, uint64_t *bar, int lane,
                                         unsigned long long *ent, uint32_t ei) {
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
                mxA = chunk_max(wA, KA, CA, LA, a, lane);
            }
            if (qB - wB >= 32) {
                wB += 32;
                mxB = chunk_max(wB, KB, CB, LB, b, lane);
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
            mt[kOffA] = hA;
            mt[kLenA] = na;
            mt[kOffB] = resA / 4 + hB;
            mt[kLenB] = nbb;
            if (ent) {
                mt[kCkEnt] = ei;
                atomicAdd(ent, 1ull);
            }
            mbar_arrive_expect_tx(bar, bytesA + bytesB);
            bulk_copy_g2s(slot, reinterpret_cast<const void *>(gaa), bytesA, bar);
            bulk_copy_g2s(slot + resA / 4, reinterpret_cast<const void *>(gbb), bytesB, bar);
        }
        return last;
    }
};

// skewed pairs: stream the long list when that reads fewer sectors than searching it (about
// b / 8 sectors against about one sector per search step, a x (log2 b - 4) of them after the
// bucket maxima), else search it from global memory
__device__ __forceinline__ bool skew_streams(uint32_t a, uint32_t b, uint32_t skew_pa) {
    return a <= skew_pa && b < 8u * a * (27u - __clz(b));
}

// |A ∩ B| of a skew job (short list staged in the slot, long list in global memory).
__device__ __forceinline__ uint32_t consume_skew(const uint32_t *mt, uint32_t *slot, int lane) {
    const uint32_t *LBp = reinterpret_cast<const uint32_t *>(
        (uint64_t)mt[kSkB] | ((uint64_t)mt[kSkB + 1] << 32));
    uint32_t c = skew_stream_count(slot + mt[kSkOffA], mt[kSkA], slot + mt[kSkTab], mt[kSkLg],
                                   LBp, mt[kSkLenB], lane);
    return __reduce_add_sync(kFull, c);
}

// The merge and search work of a staged packed or chunk job (`mt` its meta words, `slot`
// its landed copies): per-segment counts accumulate into cnt[segment] (per-warp shared
// counters). Jobs of other kinds have no segments and pass through.
__device__ __forceinline__ void consume_slot(uint32_t *mt, uint32_t *slot, uint32_t *cnt,
                                             uint32_t ratio, uint32_t slot_words,
                                             uint32_t *status, int lane) {
    const uint32_t nseg = mt[0];
    // per segment: a sentinel after each list (its reserved word; copies have landed) and
    // its merged or searched length, scanned into the segments' first diagonal / element
    uint32_t m = 0, sv = 0;
    if ((uint32_t)lane < nseg) {
        uint32_t la = mt[kLenA + lane], lb = mt[kLenB + lane];
        if (kChecked && (mt[kOffA + lane] + la >= slot_words || mt[kOffB + lane] + lb >= slot_words)) {
            atomicExch(status, kStatusBadInput);  // a segment past its slot: dropped
            la = lb = 0;
            mt[kLenA + lane] = mt[kLenB + lane] = 0;
        }
        if (la) {
            slot[mt[kOffA + lane] + la] = kEmpty;
            slot[mt[kOffB + lane] + lb] = kEmpty;
        }
        const bool srch = (uint64_t)lb > (uint64_t)ratio * la;
        m = srch ? 0u : la + lb;
        sv = srch ? la : 0u;
    }
    uint32_t im = m, is = sv;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(kFull, im, o), y = __shfl_up_sync(kFull, is, o);
        if (lane >= o) {
            im += x;
            is += y;
        }
    }
    if ((uint32_t)lane < nseg) {
        mt[kP + lane] = im - m;
        mt[kS + lane] = is - sv;
    }
    const uint32_t L = __shfl_sync(kFull, im, 31), LS = __shfl_sync(kFull, is, 31);
    if (lane == 0) {
        mt[kP + nseg] = L;
        mt[kS + nseg] = LS;
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
}

// Per-warp ring form: every warp forms its own jobs and merges them (S slots per warp).
__global__ void __maxnreg__(80) k_si_stream(SiArgs s, uint32_t *out, unsigned long long *head,
                                            StreamCfg p, uint32_t *status) {
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

    Batch cur, nxt;
    fetch_batch(cur, s, out, head, status, p.slot_words, p.ratio, lane);
    fetch_batch(nxt, s, out, head, status, p.slot_words, p.ratio, lane);
    uint32_t e = 0;
    ChunkCut ck;  // the chunked pair being cut into jobs

    // Fill slot `slot` (meta `mt`, barrier `bar`) with the next job; false when none is left.
    auto issue_job = [&](uint32_t *slot, uint32_t *mt, uint64_t *bar) -> bool {
        while (!ck.open) {
            if (cur.base >= s.np) return false;
            const uint32_t nbat = (s.np - cur.base < 32ull) ? (uint32_t)(s.np - cur.base) : 32u;
            if (e >= nbat) {
                cur = nxt;
                e = 0;
                if (cur.base < s.np) fetch_batch(nxt, s, out, head, status, p.slot_words, p.ratio, lane);
                continue;
            }
            const uint32_t kind = __shfl_sync(kFull, cur.kind, e);
            if (kind == kPairZero || kind == kPairPacked) {
                e = form_packed(cur, e, nbat, p.slot_words, slot, mt, bar, lane);
                return true;
            }
            const uint32_t *LA = shfl_ptr(cur.r.A, e), *LB = shfl_ptr(cur.r.B, e);
            const uint32_t a = __shfl_sync(kFull, cur.r.a, e), b = __shfl_sync(kFull, cur.r.b, e);
            const uint64_t pk = cur.base + e;
            ++e;
            if (kind == kPairSkewed && skew_streams(a, b, p.skew_pa)) {
                form_skew_stream(LA, a, LB, b, pk, p.skew_pa, slot, mt, bar, lane);
                return true;
            }
            if (kind == kPairSkewed) {
                uint32_t c = skew_search_count(LA, a, LB, b, lane);
                c = __reduce_add_sync(kFull, c);
                if (lane == 0) out[pk] = c;
                continue;
            }
            ck.start(LA, a, LB, b, pk, CAPE, lane);
        }
        ck.next(slot, mt, bar, lane, nullptr, 0);
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
        uint32_t *mt = meta + sr * kMetaWords;
        uint32_t *slot = ring + (size_t)sr * p.slot_words;
        const uint32_t nseg = mt[0], kind = mt[1];
        consume_slot(mt, slot, cnt, p.ratio, p.slot_words, status, lane);
        const uint64_t obase = (uint64_t)mt[2] | ((uint64_t)mt[3] << 32);
        if (kind == kJobSkew) {
            const uint32_t c = consume_skew(mt, slot, lane);
            if (lane == 0) out[obase] = c;
        } else if (kind == kJobPacked) {
            if ((uint32_t)lane < nseg) {
                out[obase + lane] = cnt[lane];
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

// ------------------------------------------------ producer / consumer form
// One producer warp per block (warp 0) forms the jobs of the pairs it takes from the queue
// and issues their bulk copies into a ring of R slots shared by the block; W consumer warps
// take the jobs in order by tickets (job t lives in slot t mod R) and only merge / search.
// The producer runs up to R jobs ahead, so copies stay in flight while the consumers merge,
// and job formation leaves the consumers' path:
//   full[r]  – completes when slot r's job is posted and its copies have landed
//              (one arrival by the producer + the copies' bytes);
//   empty[r] – completes when the consumer of slot r's job is done with it (one arrival);
//              the producer waits on it before reusing the slot;
//   acquired – jobs whose slot the producer has taken. Tickets may run more than a round
//              of the ring ahead of the slots, and an mbarrier parity wait is exact only
//              within one phase, so a consumer first waits for acquired > t (the slot's
//              previous job is then released) and only then waits on full[t mod R].
// Search jobs (skewed pairs searched in global memory) carry no data: their consumer frees
// the slot at once. Chunk jobs of one pair may go to different consumers: their counts add
// into one of kPcEnt 64-bit accumulators (count << 32 | pending jobs, the producer holding
// one reference until the pair's last job is posted); whoever drops the pending count to
// zero writes the pair's total. After the last job the producer posts one end marker per
// consumer (released like any job, as there may be more consumers than slots). Every wait is bounded and also ends when a warp of the block raised the abort
// flag after a timeout; before leaving, the producer waits (bounded) for the copies of the
// last R jobs it posted.
struct PcCfg {
    uint32_t R;           // ring slots per block
    uint32_t slot_words;  // 32-bit words per slot
    uint32_t W;           // consumer warps per block (the block has W + 1 warps)
    uint32_t ent_off;     // byte offsets of the shared-memory regions
    uint32_t cnt_off;
    uint32_t meta_off;
    uint32_t ring_off;
    uint32_t ratio;
    uint32_t skew_pa;
    uint32_t probe_polls;  // test hook (0 in normal use): see the producer's start
    uint32_t probe_tx;
};
constexpr uint32_t kPcEnt = 16;
constexpr int kPcSkewIlp = 4;  // skewed searches per lane in lockstep (merging warps)
enum : uint32_t { kJobSearch = 4, kJobEnd = 5 };
// meta words of a search job: short and long list lengths and addresses (two words each)
constexpr uint32_t kSrA = 6, kSrB = 7, kSrLA = 8, kSrLB = 10;

__device__ __forceinline__ bool pc_wait(uint64_t *bar, uint32_t parity,
                                        const volatile uint32_t *abort_flag, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 31u) == 31u && *abort_flag) return false;
    }
    return false;
}

__global__ void __maxnreg__(96)
    k_si_pc(SiArgs s, uint32_t *out, unsigned long long *head, PcCfg p, uint32_t *status) {
    extern __shared__ __align__(128) unsigned char pc_smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t *full = reinterpret_cast<uint64_t *>(pc_smem);
    uint64_t *empty = full + p.R;
    // control words: consumer ticket, abort flag, jobs acquired by the producer, probe barrier
    uint32_t *ctl = reinterpret_cast<uint32_t *>(empty + p.R);
    uint64_t *probe_bar = reinterpret_cast<uint64_t *>(ctl + 4);
    unsigned long long *ent = reinterpret_cast<unsigned long long *>(pc_smem + p.ent_off);
    uint32_t *meta = reinterpret_cast<uint32_t *>(pc_smem + p.meta_off);
    uint32_t *ring = reinterpret_cast<uint32_t *>(pc_smem + p.ring_off);
    volatile uint32_t *abort_flag = ctl + 1;
    volatile uint32_t *acquired = ctl + 2;
    if (warp == 0) {
        for (uint32_t q = lane; q < p.R; q += 32) {
            mbar_init(full + q, 1);
            mbar_init(empty + q, 1);
        }
        if (lane == 0) {
            ctl[0] = ctl[1] = ctl[2] = ctl[3] = 0;
            mbar_init(probe_bar, 1);
        }
        if ((uint32_t)lane < kPcEnt) ent[lane] = 0ull;
        fence_mbar_init();
    }
    {
        uint32_t *cnt_all = reinterpret_cast<uint32_t *>(pc_smem + p.cnt_off);
        for (uint32_t q = threadIdx.x; q < p.W * kMaxSeg; q += blockDim.x) cnt_all[q] = 0;
    }
    __syncthreads();

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (p.probe_tx && blockIdx.x == 0) {
            // test hook: arm a barrier of its own for probe_tx bytes that no copy brings, so
            // the wait (bounded at probe_polls) runs out; record the timeout and go on (no
            // copy is in flight on that barrier)
            if (lane == 0) mbar_arrive_expect_tx(probe_bar, p.probe_tx);
            __syncwarp();
            const bool ok = mbar_wait(probe_bar, 0u, p.probe_polls);
            if (!__all_sync(kFull, ok) && lane == 0) atomicExch(status, kStatusTimeout);
        }
        const uint32_t CAPE = p.slot_words - 16;
        Batch cur, nxt;
        fetch_batch(cur, s, out, head, status, p.slot_words, p.ratio, lane);
        fetch_batch(nxt, s, out, head, status, p.slot_words, p.ratio, lane);
        // a lone producer would wait out three dependent round trips per batch (queue
        // position, pair ids, list offsets): the batch after nxt has its ids in flight and
        // the one after that its queue position, so only the offset loads are waited for
        unsigned long long b2 = 0, b3 = 0;
        if (lane == 0) b2 = atomicAdd(head, 32ull);
        b2 = __shfl_sync(kFull, b2, 0);
        PairIds id2 = load_ids(s, b2 + lane, b2 + lane < s.np);
        if (lane == 0) b3 = atomicAdd(head, 32ull);
        uint32_t e = 0, j = 0, next_ent = 0, ei = 0;
        ChunkCut ck;
        bool ok = true;
        // take slot sl for job j: wait for the release of its previous job (j - R; exact,
        // since job j - R was posted only after job j - 2R had been released), then tell the
        // consumers that job j's slot is taken
        auto acquire = [&](uint32_t sl) -> bool {
            if (j >= p.R && !__all_sync(kFull, pc_wait(empty + sl, ((j / p.R) - 1u) & 1u,
                                                       abort_flag, kMaxWaitIters)))
                return false;
            if (lane == 0 && *acquired < j + 1) *acquired = j + 1;
            return true;
        };
        while (true) {
            const uint32_t sl = j % p.R;
            if (!acquire(sl)) {
                ok = false;
                break;
            }
            uint32_t *slot = ring + (size_t)sl * p.slot_words;
            uint32_t *mt = meta + (size_t)sl * kMetaWords;
            uint64_t *bar = full + sl;
            bool posted = false;
            while (!ck.open) {
                if (cur.base >= s.np) break;
                const uint32_t nbat = (s.np - cur.base < 32ull) ? (uint32_t)(s.np - cur.base) : 32u;
                if (e >= nbat) {
                    cur = nxt;
                    e = 0;
                    if (cur.base < s.np) {
                        batch_from_ids(nxt, b2, id2, s, out, status, p.slot_words, p.ratio, lane);
                        b2 = __shfl_sync(kFull, b3, 0);
                        id2 = load_ids(s, b2 + lane, b2 + lane < s.np);
                        if (lane == 0) b3 = atomicAdd(head, 32ull);
                    }
                    continue;
                }
                const uint32_t kind = __shfl_sync(kFull, cur.kind, e);
                if (kind == kPairZero || kind == kPairPacked) {
                    e = form_packed(cur, e, nbat, p.slot_words, slot, mt, bar, lane);
                    posted = true;
                    break;
                }
                const uint32_t *LA = shfl_ptr(cur.r.A, e), *LB = shfl_ptr(cur.r.B, e);
                const uint32_t a = __shfl_sync(kFull, cur.r.a, e);
                const uint32_t b = __shfl_sync(kFull, cur.r.b, e);
                const uint64_t pk = cur.base + e;
                ++e;
                if (kind == kPairSkewed && skew_streams(a, b, p.skew_pa)) {
                    form_skew_stream(LA, a, LB, b, pk, p.skew_pa, slot, mt, bar, lane);
                    posted = true;
                    break;
                }
                if (kind == kPairSkewed) {
                    if (lane == 0) {
                        mt[0] = 0;
                        mt[1] = kJobSearch;
                        mt[2] = (uint32_t)pk;
                        mt[3] = (uint32_t)(pk >> 32);
                        mt[kSrA] = a;
                        mt[kSrB] = b;
                        mt[kSrLA] = (uint32_t)reinterpret_cast<uintptr_t>(LA);
                        mt[kSrLA + 1] = (uint32_t)(reinterpret_cast<uintptr_t>(LA) >> 32);
                        mt[kSrLB] = (uint32_t)reinterpret_cast<uintptr_t>(LB);
                        mt[kSrLB + 1] = (uint32_t)(reinterpret_cast<uintptr_t>(LB) >> 32);
                        mbar_arrive_expect_tx(bar, 0u);
                    }
                    posted = true;
                    break;
                }
                // a chunked pair: take the next accumulator (free when nothing is pending)
                ei = next_ent;
                next_ent = (next_ent + 1 == kPcEnt) ? 0u : next_ent + 1;
                bool freed = false;
                if (lane == 0) {
                    const volatile unsigned long long *ve = ent + ei;
                    for (uint32_t it = 0; it < kMaxWaitIters && !freed; ++it) {
                        if ((uint32_t)*ve == 0u) freed = true;
                        else if ((it & 31u) == 31u && *abort_flag) break;
                    }
                    if (freed) ent[ei] = 1ull;  // count 0, one reference (the producer's)
                }
                if (!__shfl_sync(kFull, freed, 0)) {
                    ok = false;
                    break;
                }
                ck.start(LA, a, LB, b, pk, CAPE, lane);
            }
            if (!ok) break;
            if (!posted) {
                if (!ck.open) break;  // no pairs left: slot sl takes the first end marker
                if (ck.next(slot, mt, bar, lane, ent + ei, ei) && lane == 0) {
                    // drop the producer's reference; the last one out writes the total
                    const unsigned long long old = atomicAdd(ent + ei, ~0ull);
                    if ((uint32_t)old == 1u) out[ck.pk] = (uint32_t)(old >> 32);
                }
            }
            ++j;
        }
        // one end marker per consumer (a consumer leaves at the first one it takes)
        for (uint32_t c = 0; ok && c < p.W; ++c) {
            const uint32_t sl = j % p.R;
            if (!acquire(sl)) {
                ok = false;
                break;
            }
            if (lane == 0) {
                meta[(size_t)sl * kMetaWords + 1] = kJobEnd;
                mbar_arrive_expect_tx(full + sl, 0u);
            }
            ++j;
        }
        if (!ok && lane == 0) {
            atomicExch(status, kStatusTimeout);
            *abort_flag = 1u;
        }
        // the copies of the last jobs posted have landed before the block can retire
        const uint32_t nd = min(j, p.R);
        for (uint32_t q = 0; q < nd; ++q) {
            const uint32_t jj = j - 1 - q;
            mbar_wait(full + jj % p.R, (jj / p.R) & 1u);
        }
        return;
    }

    // -------------------------------------------------------------- consumers
    uint32_t *cnt = reinterpret_cast<uint32_t *>(pc_smem + p.cnt_off) + (size_t)(warp - 1) * kMaxSeg;
    while (true) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(ctl, 1u);
        t = __shfl_sync(kFull, t, 0);
        const uint32_t sl = t % p.R, round = t / p.R;
        // Wait for the job of ticket t. Tickets can run ahead of the ring by more than one
        // round, and a parity wait is exact only within one phase, so first wait until the
        // producer has taken slot sl for job t (acquired > t): the slot's previous job has
        // then been released, and full[sl] is at job t's phase.
        bool ok = false;
        if (lane == 0) {
            for (uint32_t it = 0; it < kMaxWaitIters; ++it) {
                if (*acquired > t) {
                    ok = true;
                    break;
                }
                if (*abort_flag) break;
                __nanosleep(64);
            }
        }
        ok = __shfl_sync(kFull, ok, 0);
        if (ok) ok = pc_wait(full + sl, round & 1u, abort_flag, kMaxWaitIters);
        if (!__all_sync(kFull, ok)) {
            if (lane == 0) {
                atomicExch(status, kStatusTimeout);
                *abort_flag = 1u;
            }
            break;
        }
        uint32_t *mt = meta + (size_t)sl * kMetaWords;
        uint32_t *slot = ring + (size_t)sl * p.slot_words;
        const uint32_t kind = mt[1];
        if (kind == kJobEnd) {  // release the slot too: there may be more markers than slots
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + sl);
            break;
        }
        const uint64_t obase = (uint64_t)mt[2] | ((uint64_t)mt[3] << 32);
        if (kind == kJobSearch) {
            const uint32_t a = mt[kSrA], b = mt[kSrB];
            const uint32_t *LA = reinterpret_cast<const uint32_t *>(
                (uint64_t)mt[kSrLA] | ((uint64_t)mt[kSrLA + 1] << 32));
            const uint32_t *LB = reinterpret_cast<const uint32_t *>(
                (uint64_t)mt[kSrLB] | ((uint64_t)mt[kSrLB + 1] << 32));
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + sl);  // no data in the slot: free it now
            uint32_t c = skew_search_count<kPcSkewIlp>(LA, a, LB, b, lane);
            c = __reduce_add_sync(kFull, c);
            if (lane == 0) out[obase] = c;
            continue;
        }
        const uint32_t nseg = mt[0];
        consume_slot(mt, slot, cnt, p.ratio, p.slot_words, status, lane);
        if (kind == kJobSkew) {
            const uint32_t c = consume_skew(mt, slot, lane);
            if (lane == 0) out[obase] = c;
        } else if (kind == kJobPacked) {
            if ((uint32_t)lane < nseg) {
                out[obase + lane] = cnt[lane];
                cnt[lane] = 0;
            }
        } else if (lane == 0) {
            // a chunk job: add the count and drop one pending job in one 64-bit atomic
            const uint32_t c = cnt[0];
            cnt[0] = 0;
            const unsigned long long old =
                atomicAdd(ent + mt[kCkEnt], ((unsigned long long)c << 32) - 1ull);
            if ((uint32_t)old == 1u) out[obase] = (uint32_t)(old >> 32) + c;
        }
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + sl);
    }
}

constexpr uint32_t kWriteSearchRatio = 16;  // long/short above this: search, not merge

__global__ void k_si_write(SiArgs s, const uint64_t *__restrict__ out_off, uint32_t *out_elems) {
    const int lane = threadIdx.x & 31;
    uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t k = warp; k < s.np; k += nwarps) {
        uint32_t x, y;
        if (!pair_ids(s, k, x, y)) continue;
        uint64_t ox = s.off[x], oy = s.off[y];
        uint32_t lx = (uint32_t)(s.off[x + 1] - ox), ly = (uint32_t)(s.off[y + 1] - oy);
        // skewed pairs: the short list searched in the long one (a merge would walk the
        // whole long list); the matches come out ascending either way
        if ((uint64_t)ly > (uint64_t)kWriteSearchRatio * lx)
            warp_search_write(s.elems + ox, lx, s.elems + oy, ly, out_elems + out_off[k], lane);
        else if ((uint64_t)lx > (uint64_t)kWriteSearchRatio * ly)
            warp_search_write(s.elems + oy, ly, s.elems + ox, lx, out_elems + out_off[k], lane);
        else
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

// One batched SI launch of kernel form `form` (`kern`, `threads` per block, `smem` bytes of
// shared memory per block): a persistent grid of as many blocks as fit on the SMs (capped by
// si_blocks_per_sm and by `need`, the blocks the pairs can keep busy), launched through the context's CUDA graph of that
// form. The first launch captures the queue-head reset and the kernel; later launches set
// the kernel node's grid, shared memory and arguments and replay it.
template <typename Cfg>
rtg_status launch_batched(rtg_ctx *ctx, int form,
                          void (*kern)(SiArgs, uint32_t *, unsigned long long *, Cfg, uint32_t *),
                          uint32_t threads, size_t smem, uint64_t need, SiArgs args,
                          uint32_t *d_out, unsigned long long *head, Cfg cfg, float *kernel_ms,
                          uint64_t *launches) {
    if ((int)smem > ctx->smem_optin)
        return fail(ctx, RTG_ERR_INVALID_ARG, "SI schedule needs %zu B of shared memory", smem);
    RTG_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    RTG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, (int)threads, smem));
    if (ctx->cfg.si_blocks_per_sm) per_sm = std::min<int>(per_sm, (int)ctx->cfg.si_blocks_per_sm);
    if (per_sm < 1) return fail(ctx, RTG_ERR_INVALID_ARG, "SI schedule does not fit on an SM");
    const int grid =
        (int)std::max<uint64_t>(1, std::min<uint64_t>(need, (uint64_t)ctx->sm_count * per_sm));
    uint32_t *status = ctx->d_status;
    auto &kg = ctx->si_graphs[form];
    if (!kg.exec) {
        cudaGraph_t gr = nullptr;
        RTG_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        cudaMemsetAsync(head, 0, 8, ctx->stream);
        kern<<<grid, threads, smem, ctx->stream>>>(args, d_out, head, cfg, status);
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
                kg.knode = nd;
        }
        kg.graph = gr;
        kg.exec = ex;
        if (!kg.knode) return fail(ctx, RTG_ERR_DEVICE, "SI graph has no kernel node");
    } else {
        void *kargs[] = {&args, &d_out, &head, &cfg, &status};
        cudaKernelNodeParams kp{};
        kp.func = reinterpret_cast<void *>(kern);
        kp.gridDim = dim3((unsigned)grid);
        kp.blockDim = dim3(threads);
        kp.sharedMemBytes = (unsigned)smem;
        kp.kernelParams = kargs;
        RTG_CUDA(ctx, cudaGraphExecKernelNodeSetParams(kg.exec, kg.knode, &kp));
    }
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
    RTG_CUDA(ctx, cudaGraphLaunch(kg.exec, ctx->stream));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
    (*launches)++;
    if (kernel_ms) {
        RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[7]));
        cudaEventElapsedTime(kernel_ms, ctx->ev[6], ctx->ev[7]);
    }
    return RTG_OK;
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
        const uint32_t form = cf.si_form ? cf.si_form : kDefaultSiForm;
        const uint32_t slot_bytes =
            cf.si_stage_bytes ? cf.si_stage_bytes
                              : (form == 2 ? kDefaultPcSlotBytes : kDefaultStageBytes);
        const uint32_t slot_words = slot_bytes / 4;
        const uint32_t sratio = cf.si_search_ratio ? cf.si_search_ratio : kDefaultStreamRatio;
        // a skew job holds the short list (at most skew_pa elements, widened) and a table
        // of 4 x skew_pa words after it: the largest power of two with 5 x + 20 <= slot words
        uint32_t skew_pa = 0;
        if (cf.si_skew_stream) {
            skew_pa = 16;
            while (5 * (2 * skew_pa) + 20 <= slot_words) skew_pa *= 2;
        }
        // the test hook of rtg_debug_si_wait_limit applies to one launch
        const uint32_t probe_polls = ctx->dbg_wait_polls ? ctx->dbg_wait_polls : kMaxWaitIters;
        const uint32_t probe_tx = ctx->dbg_extra_tx;
        ctx->dbg_wait_polls = ctx->dbg_extra_tx = 0;
        SiArgs args = make_args(ps);
        unsigned long long *head = ctx->d_scalars + 8;
        if (form == 2) {
            PcCfg pc{};
            pc.W = cf.si_block_warps ? cf.si_block_warps : kDefaultPcWarps;
            if (pc.W > 31) return fail(ctx, RTG_ERR_INVALID_ARG, "at most 31 merging warps per block");
            pc.R = cf.si_stage_slots ? cf.si_stage_slots : kDefaultPcSlots;
            pc.slot_words = slot_words;
            pc.ratio = sratio;
            pc.skew_pa = skew_pa;
            pc.probe_polls = probe_polls;
            pc.probe_tx = probe_tx;
            pc.ent_off = 16 * pc.R + 32;  // full and empty barriers, 4 control words, probe
            pc.cnt_off = pc.ent_off + kPcEnt * 8;
            pc.meta_off = (pc.cnt_off + pc.W * kMaxSeg * 4 + 15u) & ~15u;
            pc.ring_off = (pc.meta_off + pc.R * kMetaWords * 4 + 127u) & ~127u;
            const size_t smem = (size_t)pc.ring_off + (size_t)pc.R * slot_bytes;
            const uint64_t need = (ps.npairs + 32ull * pc.W - 1) / (32ull * pc.W);
            return launch_batched(ctx, 1, k_si_pc, (pc.W + 1) * 32, smem, need, args, d_out, head,
                                  pc, kernel_ms, launches);
        }
        const uint32_t W = cf.si_block_warps ? cf.si_block_warps : kDefaultStreamWarps;
        StreamCfg sc{};
        sc.S = cf.si_stage_slots ? cf.si_stage_slots : kDefaultStageSlots;
        sc.slot_words = slot_words;
        sc.ratio = sratio;
        sc.skew_pa = skew_pa;
        sc.probe_polls = probe_polls;
        sc.probe_tx = probe_tx;
        sc.meta_off = ((W * sc.S * 8) + 127u) & ~127u;
        sc.cnt_off = (sc.meta_off + W * sc.S * kMetaWords * 4 + 127u) & ~127u;
        sc.ring_off = (sc.cnt_off + W * kMaxSeg * 4 + 127u) & ~127u;
        const size_t smem = (size_t)sc.ring_off + (size_t)W * sc.S * slot_bytes;
        const uint64_t need = (ps.npairs + 32ull * W - 1) / (32ull * W);
        return launch_batched(ctx, 0, k_si_stream, W * 32, smem, need, args, d_out, head, sc,
                              kernel_ms, launches);
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
