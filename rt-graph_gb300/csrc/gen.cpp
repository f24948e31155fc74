// Seeded synthetic inputs: R-MAT, Barabasi-Albert, Holme-Kim graphs and the batched
// set-intersection pair workload. Integer-only random streams (splitmix64 / xoshiro256**)
// so the same seed gives the same edges on every host architecture.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "rtg.h"

namespace {

inline uint64_t splitmix64(uint64_t &x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Stateless 64-bit hash of (seed, a, b): the counter-based stream used by R-MAT.
inline uint64_t hash3(uint64_t seed, uint64_t a, uint64_t b) {
    uint64_t x = seed ^ (a * 0xD6E8FEB86659FD93ull) ^ (b * 0xA0761D6478BD642Full);
    return splitmix64(x);
}

struct Xoshiro {
    uint64_t s[4];
    explicit Xoshiro(uint64_t seed) {
        uint64_t x = seed;
        for (auto &w : s) w = splitmix64(x);
    }
    static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    inline uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    // uniform integer in [0, n) (Lemire's multiply-shift, unbiased with rejection)
    inline uint64_t below(uint64_t n) {
        unsigned __int128 m = (unsigned __int128)next() * n;
        uint64_t l = (uint64_t)m;
        if (l < n) {
            uint64_t t = (0 - n) % n;
            while (l < t) {
                m = (unsigned __int128)next() * n;
                l = (uint64_t)m;
            }
        }
        return (uint64_t)(m >> 64);
    }
    inline double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
};

inline uint32_t threshold32(double p) {
    if (p <= 0) return 0;
    if (p >= 1) return 0xFFFFFFFFu;
    return (uint32_t)std::floor(p * 4294967296.0);
}

}  // namespace

extern "C" {

rtg_status rtg_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                        uint64_t seed, uint32_t *src, uint32_t *dst) {
    if (!src || !dst || scale == 0 || scale > 31 || edge_factor == 0) return RTG_ERR_INVALID_ARG;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return RTG_ERR_INVALID_ARG;
    const uint64_t m = (uint64_t)edge_factor << scale;
    const uint32_t ta = threshold32(a), tb = threshold32(a + b), tc = threshold32(a + b + c);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)m; ++i) {
        uint32_t s = 0, d = 0;
        uint64_t r = 0;
        for (uint32_t l = 0; l < scale; ++l) {
            if ((l & 1) == 0) r = hash3(seed, (uint64_t)i, l >> 1);
            uint32_t u = (uint32_t)(r >> ((l & 1) ? 32 : 0));
            uint32_t sb, db;
            if (u < ta) { sb = 0; db = 0; }
            else if (u < tb) { sb = 0; db = 1; }
            else if (u < tc) { sb = 1; db = 0; }
            else { sb = 1; db = 1; }
            s = (s << 1) | sb;
            d = (d << 1) | db;
        }
        src[i] = s;
        dst[i] = d;
    }
    return RTG_OK;
}

rtg_status rtg_gen_ba(uint32_t n, uint32_t m, uint64_t seed, uint32_t *src, uint32_t *dst,
                      uint64_t *m_out) {
    if (!src || !dst || m == 0 || n <= m) return RTG_ERR_INVALID_ARG;
    Xoshiro rng(seed);
    std::vector<uint32_t> repeated;
    repeated.reserve(2ull * m * n);
    uint64_t e = 0;
    // seed graph: a star on m+1 vertices centred on 0
    for (uint32_t i = 1; i <= m; ++i) {
        src[e] = 0;
        dst[e] = i;
        ++e;
        repeated.push_back(0);
        repeated.push_back(i);
    }
    std::vector<uint32_t> targets;
    targets.reserve(m);
    for (uint32_t v = m + 1; v < n; ++v) {
        targets.clear();
        while (targets.size() < m) {
            uint32_t t = repeated[rng.below(repeated.size())];
            if (std::find(targets.begin(), targets.end(), t) == targets.end()) targets.push_back(t);
        }
        for (uint32_t t : targets) {
            src[e] = v;
            dst[e] = t;
            ++e;
            repeated.push_back(t);
            repeated.push_back(v);
        }
    }
    if (m_out) *m_out = e;
    return RTG_OK;
}

rtg_status rtg_gen_hk(uint32_t n, uint32_t m, double p, uint64_t seed, uint32_t *src,
                      uint32_t *dst, uint64_t *m_out) {
    if (!src || !dst || m == 0 || n <= m || p < 0 || p > 1) return RTG_ERR_INVALID_ARG;
    Xoshiro rng(seed);
    std::vector<std::vector<uint32_t>> adj(n);
    std::vector<uint32_t> repeated;
    repeated.reserve(2ull * m * n);
    for (uint32_t i = 0; i < m; ++i) repeated.push_back(i);
    uint64_t e = 0;
    std::vector<uint32_t> targets;
    auto adjacent = [&](uint32_t x, uint32_t y) {
        const auto &l = adj[x];
        return std::find(l.begin(), l.end(), y) != l.end();  // x is the new vertex: <= m entries
    };
    auto add = [&](uint32_t x, uint32_t y) {
        adj[x].push_back(y);
        adj[y].push_back(x);
        src[e] = x;
        dst[e] = y;
        ++e;
        repeated.push_back(y);
    };
    for (uint32_t v = m; v < n; ++v) {
        // m distinct preferential-attachment candidates
        targets.clear();
        while (targets.size() < m) {
            uint32_t t = repeated[rng.below(repeated.size())];
            if (std::find(targets.begin(), targets.end(), t) == targets.end()) targets.push_back(t);
        }
        uint32_t t = targets.back();
        targets.pop_back();
        add(v, t);
        uint32_t count = 1;
        while (count < m) {
            if (rng.uniform() < p) {
                // triad closure: a neighbour of t not yet adjacent to v
                const auto &nt = adj[t];
                uint32_t pick = 0xFFFFFFFFu;
                for (int tries = 0; tries < 8 && !nt.empty(); ++tries) {
                    uint32_t w = nt[rng.below(nt.size())];
                    if (w != v && !adjacent(v, w)) {
                        pick = w;
                        break;
                    }
                }
                if (pick == 0xFFFFFFFFu) {
                    std::vector<uint32_t> cand;
                    for (uint32_t w : nt)
                        if (w != v && !adjacent(v, w)) cand.push_back(w);
                    if (!cand.empty()) pick = cand[rng.below(cand.size())];
                }
                if (pick != 0xFFFFFFFFu) {
                    add(v, pick);
                    ++count;
                    continue;
                }
            }
            // preferential-attachment step: next candidate not already adjacent
            bool added = false;
            while (!targets.empty()) {
                t = targets.back();
                targets.pop_back();
                if (!adjacent(v, t)) {
                    add(v, t);
                    added = true;
                    break;
                }
            }
            if (!added) break;
            ++count;
        }
        for (uint32_t i = 0; i < m; ++i) repeated.push_back(v);
    }
    if (m_out) *m_out = e;
    return RTG_OK;
}

rtg_status rtg_gen_si_pairs(uint64_t npairs, double median, double sigma, uint32_t min_len,
                            uint32_t max_len, uint32_t universe_log2, double overlap_max,
                            uint64_t seed, uint32_t *len, uint64_t *total, uint64_t *offsets,
                            uint32_t *elems, uint32_t *expected) {
    if (!len || !total || median <= 0 || sigma < 0 || min_len == 0 || max_len < min_len ||
        universe_log2 == 0 || universe_log2 > 31 || overlap_max < 0 || overlap_max > 1)
        return RTG_ERR_INVALID_ARG;
    const uint64_t U = 1ull << universe_log2;
    if (2ull * max_len > U) return RTG_ERR_INVALID_ARG;
    if (!elems) {
        // phase 1: lengths (lognormal, clamped)
        const double mu = std::log(median);
        uint64_t tot = 0;
#pragma omp parallel for reduction(+ : tot) schedule(static)
        for (int64_t i = 0; i < (int64_t)(2 * npairs); ++i) {
            uint64_t r = hash3(seed, 0x5151u, (uint64_t)i);
            double u1 = ((double)(r >> 11) + 0.5) * 0x1.0p-53;
            uint64_t r2 = hash3(seed, 0x5152u, (uint64_t)i);
            double u2 = (double)(r2 >> 11) * 0x1.0p-53;
            double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
            double x = std::floor(std::exp(mu + sigma * z));
            uint32_t l = (x < (double)min_len) ? min_len : (x > (double)max_len ? max_len : (uint32_t)x);
            len[i] = l;
            tot += l;
        }
        *total = tot;
        return RTG_OK;
    }
    if (!offsets || !expected) return RTG_ERR_INVALID_ARG;
    offsets[0] = 0;
    for (uint64_t i = 0; i < 2 * npairs; ++i) offsets[i + 1] = offsets[i] + len[i];
    if (offsets[2 * npairs] != *total) return RTG_ERR_INVALID_ARG;
#pragma omp parallel
    {
        std::vector<uint32_t> buf, idx;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < (int64_t)npairs; ++i) {
            Xoshiro rng(hash3(seed, 0x5153u, (uint64_t)i));
            const uint64_t sa = 2 * i, sb = 2 * i + 1;
            const bool a_long = len[sa] >= len[sb];
            const uint64_t sl = a_long ? sa : sb, ss = a_long ? sb : sa;
            const uint32_t L = len[sl], S = len[ss];
            uint32_t *Lp = elems + offsets[sl], *Sp = elems + offsets[ss];
            // long list: L distinct uniform values, sorted
            buf.clear();
            while (buf.size() < L) {
                size_t need = L - buf.size();
                for (size_t k = 0; k < need; ++k) buf.push_back((uint32_t)rng.below(U));
                std::sort(buf.begin(), buf.end());
                buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
            }
            std::memcpy(Lp, buf.data(), L * 4ull);
            // short list: k elements of the long list, S-k from outside it
            const double f = rng.uniform() * overlap_max;
            const uint32_t k = (uint32_t)std::floor(f * S);
            idx.resize(L);
            for (uint32_t t = 0; t < L; ++t) idx[t] = t;
            buf.clear();
            for (uint32_t t = 0; t < k; ++t) {  // partial Fisher-Yates
                uint32_t r = t + (uint32_t)rng.below(L - t);
                std::swap(idx[t], idx[r]);
                buf.push_back(Lp[idx[t]]);
            }
            while (buf.size() < S) {
                size_t need = S - buf.size();
                for (size_t q = 0; q < need; ++q) {
                    uint32_t x = (uint32_t)rng.below(U);
                    if (!std::binary_search(Lp, Lp + L, x)) buf.push_back(x);
                }
                std::sort(buf.begin(), buf.end());
                buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
            }
            std::memcpy(Sp, buf.data(), S * 4ull);
            expected[i] = k;
        }
    }
    return RTG_OK;
}

}  // extern "C"
