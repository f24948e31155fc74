// Warp-level sorted-list intersection primitives shared by the TC and SI kernels.
//
// All lists are sorted ascending with unique elements; kEmpty (0xFFFFFFFF) never occurs
// as an element. Every primitive is called by all 32 lanes of a warp with warp-uniform
// arguments and returns a lane-local partial count (sum over the warp = |A ∩ B|).
#pragma once

#include <cstdint>

namespace rtg {

constexpr unsigned kFull = 0xffffffffu;

// Lower bound of x among the first nb lanes' values of r (sorted ascending across lanes;
// lanes >= nb act as +infinity). Returns a lane index in [0, 31].
__device__ __forceinline__ int warp_lower_bound(uint32_t r, uint32_t nb, uint32_t x) {
    int pos = 0;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        int probe = pos + s - 1;
        uint32_t v = __shfl_sync(kFull, r, probe);
        if ((uint32_t)probe < nb && v < x) pos += s;
    }
    return pos;
}

// Tile merge ("merge family", cf. the merge-path baseline set_intersection/baseline/ip.cu:
// 138-287): both lists advance 32 elements at a time; every A element of the tile is
// looked up among the B tile by a 5-step shuffle search; the tiles then advance past
// min(max A tile, max B tile). Each match is seen exactly once, in the iteration whose
// bound first covers its value.
__device__ __forceinline__ uint32_t warp_merge_count(const uint32_t *__restrict__ A, uint32_t a,
                                                     const uint32_t *__restrict__ B, uint32_t b,
                                                     int lane) {
    uint32_t i = 0, j = 0, cnt = 0;
    while (i < a && j < b) {
        uint32_t na = min(32u, a - i), nb = min(32u, b - j);
        uint32_t ra = (uint32_t)lane < na ? __ldg(A + i + lane) : kEmpty;
        uint32_t rb = (uint32_t)lane < nb ? __ldg(B + j + lane) : kEmpty;
        uint32_t amax = __shfl_sync(kFull, ra, na - 1);
        uint32_t bmax = __shfl_sync(kFull, rb, nb - 1);
        int pos = warp_lower_bound(rb, nb, ra);
        uint32_t at = __shfl_sync(kFull, rb, pos);
        cnt += ((uint32_t)lane < na && (uint32_t)pos < nb && at == ra) ? 1u : 0u;
        uint32_t x = min(amax, bmax);
        i += __popc(__ballot_sync(kFull, (uint32_t)lane < na && ra <= x));
        j += __popc(__ballot_sync(kFull, (uint32_t)lane < nb && rb <= x));
    }
    return cnt;
}

// Same walk, writing the matches: out receives the common elements in ascending order.
// Returns the number written (warp-uniform).
__device__ __forceinline__ uint32_t warp_merge_write(const uint32_t *__restrict__ A, uint32_t a,
                                                     const uint32_t *__restrict__ B, uint32_t b,
                                                     uint32_t *__restrict__ out, int lane) {
    uint32_t i = 0, j = 0, w = 0;
    const unsigned lt = (1u << lane) - 1u;
    while (i < a && j < b) {
        uint32_t na = min(32u, a - i), nb = min(32u, b - j);
        uint32_t ra = (uint32_t)lane < na ? __ldg(A + i + lane) : kEmpty;
        uint32_t rb = (uint32_t)lane < nb ? __ldg(B + j + lane) : kEmpty;
        uint32_t amax = __shfl_sync(kFull, ra, na - 1);
        uint32_t bmax = __shfl_sync(kFull, rb, nb - 1);
        int pos = warp_lower_bound(rb, nb, ra);
        uint32_t at = __shfl_sync(kFull, rb, pos);
        bool hit = (uint32_t)lane < na && (uint32_t)pos < nb && at == ra;
        unsigned hm = __ballot_sync(kFull, hit);
        if (hit) out[w + __popc(hm & lt)] = ra;
        w += __popc(hm);
        uint32_t x = min(amax, bmax);
        i += __popc(__ballot_sync(kFull, (uint32_t)lane < na && ra <= x));
        j += __popc(__ballot_sync(kFull, (uint32_t)lane < nb && rb <= x));
    }
    return w;
}

// Search family (cf. the binary-search baselines set_intersection/baseline/bs.cu:341-370 and
// tc/bs_tc/bs_tc.cu:14-25): each lane takes one element of the short list S and binary-
// searches it in the long list L. Rounds of 32 elements; the search window of a round
// starts where the previous round's last element landed (S is sorted).
__device__ __forceinline__ uint32_t warp_search_count(const uint32_t *__restrict__ S, uint32_t s,
                                                      const uint32_t *__restrict__ L, uint32_t l,
                                                      int lane) {
    uint32_t cnt = 0, base = 0;
    for (uint32_t i = 0; i < s && base < l; i += 32) {
        uint32_t k = i + lane;
        bool valid = k < s;
        uint32_t x = valid ? __ldg(S + k) : kEmpty;
        uint32_t lo = base, hi = l;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (__ldg(L + mid) < x) lo = mid + 1;
            else hi = mid;
        }
        cnt += (valid && lo < l && __ldg(L + lo) == x) ? 1u : 0u;
        uint32_t last = min(32u, s - i) - 1;
        base = __shfl_sync(kFull, lo, last);
    }
    return cnt;
}

// Same search, writing the matches: out receives the common elements in ascending order (S
// is sorted; each round's matches are written in lane order at their ballot rank). Returns
// the number written (warp-uniform).
__device__ __forceinline__ uint32_t warp_search_write(const uint32_t *__restrict__ S, uint32_t s,
                                                      const uint32_t *__restrict__ L, uint32_t l,
                                                      uint32_t *out, int lane) {
    uint32_t n = 0, base = 0;
    const uint32_t lt = (1u << lane) - 1u;
    for (uint32_t i = 0; i < s && base < l; i += 32) {
        uint32_t k = i + lane;
        bool valid = k < s;
        uint32_t x = valid ? __ldg(S + k) : kEmpty;
        uint32_t lo = base, hi = l;
        while (lo < hi) {
            uint32_t mid = (lo + hi) >> 1;
            if (__ldg(L + mid) < x) lo = mid + 1;
            else hi = mid;
        }
        const bool hit = valid && lo < l && __ldg(L + lo) == x;
        const unsigned hm = __ballot_sync(kFull, hit);
        if (hit) out[n + __popc(hm & lt)] = x;
        n += __popc(hm);
        uint32_t last = min(32u, s - i) - 1;
        base = __shfl_sync(kFull, lo, last);
    }
    return n;
}

// Open-addressing hash of a short list in shared memory (one table per warp). The table
// has cap = 2^lg slots with cap >= 2 * length, so every probe chain ends at an empty slot.
__device__ __forceinline__ uint32_t hash_slot(uint32_t w, uint32_t lg) {
    return (w * 0x9E3779B1u) >> (32 - lg);
}

__device__ __forceinline__ uint32_t hash_lg_for(uint32_t len) {
    uint32_t lg = 5;
    while ((1u << lg) < 2 * len) ++lg;
    return lg;
}

__device__ __forceinline__ void warp_hash_build(uint32_t *tab, uint32_t lg,
                                                const uint32_t *__restrict__ list, uint32_t len,
                                                int lane) {
    const uint32_t cap = 1u << lg, mask = cap - 1;
    uint4 *t4 = reinterpret_cast<uint4 *>(tab);
    const uint4 e4 = make_uint4(kEmpty, kEmpty, kEmpty, kEmpty);
    for (uint32_t s = lane; s < cap / 4; s += 32) t4[s] = e4;
    __syncwarp();
    for (uint32_t t = lane; t < len; t += 32) {
        uint32_t w = __ldg(list + t);
        uint32_t s = hash_slot(w, lg);
        while (atomicCAS(&tab[s], kEmpty, w) != kEmpty) s = (s + 1) & mask;
    }
    __syncwarp();
}

__device__ __forceinline__ uint32_t hash_probe(const uint32_t *tab, uint32_t lg, uint32_t w) {
    const uint32_t mask = (1u << lg) - 1;
    uint32_t s = hash_slot(w, lg);
    while (true) {
        uint32_t x = tab[s];
        if (x == w) return 1u;
        if (x == kEmpty) return 0u;
        s = (s + 1) & mask;
    }
}

// Stream the long list B through the hash of the short list (4 loads in flight per lane).
__device__ __forceinline__ uint32_t warp_hash_stream(const uint32_t *tab, uint32_t lg,
                                                     const uint32_t *__restrict__ B, uint32_t b,
                                                     int lane) {
    uint32_t cnt = 0, t = lane;
    for (; t + 96 < b; t += 128) {
        uint32_t w0 = __ldg(B + t), w1 = __ldg(B + t + 32), w2 = __ldg(B + t + 64),
                 w3 = __ldg(B + t + 96);
        cnt += hash_probe(tab, lg, w0) + hash_probe(tab, lg, w1) + hash_probe(tab, lg, w2) +
               hash_probe(tab, lg, w3);
    }
    for (; t < b; t += 32) cnt += hash_probe(tab, lg, __ldg(B + t));
    return cnt;
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

}  // namespace rtg
