/*
 * CPU oracle for the set-intersection path — TEST INFRASTRUCTURE ONLY (see rtg_oracle.h).
 * Each function restates one reference routine; the citation is beside it.
 */
#include "rtg_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdlib.h>
#include <string.h>

static void set_threads(int threads) {
    if (threads > 0) omp_set_num_threads(threads);
}

/* ------------------------------------------------------------ preprocessing */

int64_t orc_compact_ids(int32_t *pairs, int64_t m) {
    /* graph.cpp:40-62: mark used ids, prefix-sum, replace every id by (rank - 1). The
     * reference relies on malloc returning zeroed pages (its memset has swapped
     * arguments, graph.cpp:48); the array is zeroed explicitly here. */
    int32_t max_id = 0;
    for (int64_t i = 0; i < 2 * m; ++i)
        if (pairs[i] > max_id) max_id = pairs[i];
    if (m == 0) return 0;
    int32_t *before = (int32_t *)calloc((size_t)max_id + 1, sizeof(int32_t));
    if (!before) return -1;
    for (int64_t i = 0; i < 2 * m; ++i) before[pairs[i]] = 1;
    for (int32_t i = 1; i <= max_id; ++i) before[i] += before[i - 1];
    for (int64_t i = 0; i < 2 * m; ++i) pairs[i] = before[pairs[i]] - 1;
    int64_t nodes = before[max_id];
    free(before);
    return nodes;
}

static int cmp_pair(const void *x, const void *y) {
    const int32_t *a = (const int32_t *)x, *b = (const int32_t *)y;
    if (a[0] != b[0]) return a[0] < b[0] ? -1 : 1;
    if (a[1] != b[1]) return a[1] < b[1] ? -1 : 1;
    return 0;
}

int orc_tc_preprocess_ref(int32_t *pairs, int64_t m, int32_t nodes, int32_t *offsets,
                          int32_t *adjs, int32_t *out_nodes, int64_t *out_edges) {
    if (m == 0 || nodes <= 0) {
        *out_nodes = 0;
        *out_edges = 0;
        if (offsets) offsets[0] = 0;
        return 0;
    }
    int32_t *degree = (int32_t *)calloc((size_t)nodes, sizeof(int32_t));
    int32_t *removes = (int32_t *)malloc((size_t)nodes * sizeof(int32_t));
    if (!degree || !removes) return -1;
    /* graph.cpp:108-114: degree on the raw list (duplicates and self loops included) */
    for (int64_t i = 0; i < m; ++i) {
        degree[pairs[2 * i]] += 1;
        degree[pairs[2 * i + 1]] += 1;
    }
    /* graph.cpp:116-124: orient towards the higher degree, ties to the larger id */
    for (int64_t i = 0; i < m; ++i) {
        int32_t s = pairs[2 * i], d = pairs[2 * i + 1];
        if (degree[s] > degree[d] || (degree[s] == degree[d] && s > d)) {
            pairs[2 * i] = d;
            pairs[2 * i + 1] = s;
        }
    }
    /* graph.cpp:126-149: drop vertices of degree <= 1, shift ids down */
    removes[0] = degree[0] <= 1;
    for (int32_t i = 1; i < nodes; ++i) removes[i] = removes[i - 1] + (degree[i] <= 1);
    int64_t kept = 0;
    for (int64_t i = 0; i < m; ++i) {
        int32_t s = pairs[2 * i], d = pairs[2 * i + 1];
        if (degree[s] <= 1 || degree[d] <= 1) continue;
        pairs[2 * kept] = s - removes[s];
        pairs[2 * kept + 1] = d - removes[d];
        ++kept;
    }
    int32_t n2 = nodes - removes[nodes - 1];
    free(degree);
    free(removes);
    /* graph.cpp:157 (ThrustSortEdgesInBatch, thrust_helper.cu:16-42): lexicographic sort */
    qsort(pairs, (size_t)kept, 2 * sizeof(int32_t), cmp_pair);
    /* graph.cpp:160-173 and 71-102: drop self loops and repeats, build the CSR */
    for (int32_t v = 0; v <= n2; ++v) offsets[v] = 0;
    int64_t e = 0;
    int32_t ls = -1, ld = -1;
    for (int64_t i = 0; i < kept; ++i) {
        int32_t s = pairs[2 * i], d = pairs[2 * i + 1];
        int drop = (s == d) || (s == ls && d == ld);
        ls = s;
        ld = d;
        if (drop) continue;
        offsets[s + 1] += 1;
        adjs[e++] = d;
    }
    for (int32_t v = 0; v < n2; ++v) offsets[v + 1] += offsets[v];
    *out_nodes = n2;
    *out_edges = e;
    return 0;
}

static int cmp_u64(const void *x, const void *y) {
    uint64_t a = *(const uint64_t *)x, b = *(const uint64_t *)y;
    return a < b ? -1 : (a > b ? 1 : 0);
}

/* sorted unique canonical (min,max) keys without self loops; returns count */
static uint64_t simple_edges(const uint32_t *src, const uint32_t *dst, uint64_t m, uint64_t *k) {
    uint64_t c = 0;
    for (uint64_t i = 0; i < m; ++i) {
        uint32_t a = src[i], b = dst[i];
        if (a == b) continue;
        if (a > b) {
            uint32_t t = a;
            a = b;
            b = t;
        }
        k[c++] = ((uint64_t)a << 32) | b;
    }
    qsort(k, (size_t)c, sizeof(uint64_t), cmp_u64);
    uint64_t u = 0;
    for (uint64_t i = 0; i < c; ++i)
        if (u == 0 || k[u - 1] != k[i]) k[u++] = k[i];
    return u;
}

static void keys_to_csr(uint64_t *k, uint64_t mk, uint32_t n, uint64_t *off, uint32_t *adj) {
    qsort(k, (size_t)mk, sizeof(uint64_t), cmp_u64);
    for (uint64_t v = 0; v <= n; ++v) off[v] = 0;
    for (uint64_t i = 0; i < mk; ++i) {
        off[(k[i] >> 32) + 1] += 1;
        adj[i] = (uint32_t)k[i];
    }
    for (uint64_t v = 0; v < n; ++v) off[v + 1] += off[v];
}

int orc_csr_degree(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n,
                   uint64_t *offsets, uint32_t *adj, uint64_t *m_out) {
    uint64_t *k = (uint64_t *)malloc((m ? m : 1) * sizeof(uint64_t));
    uint32_t *deg = (uint32_t *)calloc((size_t)n + 1, sizeof(uint32_t));
    if (!k || !deg) return -1;
    uint64_t mu = simple_edges(src, dst, m, k);
    for (uint64_t i = 0; i < mu; ++i) {
        if ((k[i] >> 32) >= n || (uint32_t)k[i] >= n) {
            free(k);
            free(deg);
            return -1;
        }
        deg[k[i] >> 32]++;
        deg[(uint32_t)k[i]]++;
    }
    for (uint64_t i = 0; i < mu; ++i) {
        uint32_t a = (uint32_t)(k[i] >> 32), b = (uint32_t)k[i]; /* a < b */
        if (deg[a] > deg[b]) k[i] = ((uint64_t)b << 32) | a;
    }
    keys_to_csr(k, mu, n, offsets, adj);
    *m_out = mu;
    free(k);
    free(deg);
    return 0;
}

int orc_csr_symmetric(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n,
                      uint64_t *offsets, uint32_t *adj, uint64_t *m_out) {
    uint64_t *k = (uint64_t *)malloc((2 * m ? 2 * m : 1) * sizeof(uint64_t));
    if (!k) return -1;
    uint64_t mu = simple_edges(src, dst, m, k);
    for (uint64_t i = 0; i < mu; ++i)
        k[mu + i] = ((uint64_t)(uint32_t)k[i] << 32) | (k[i] >> 32);
    keys_to_csr(k, 2 * mu, n, offsets, adj);
    *m_out = 2 * mu;
    free(k);
    return 0;
}

/* ---------------------------------------------------------------- counting */

static int binary_check(const int32_t *data, int32_t l, int32_t r, int32_t val) {
    /* bs_tc.cu:14-25 */
    while (l <= r) {
        int32_t mid = (l + r) >> 1;
        if (data[mid] == val) return 1;
        if (data[mid] < val) l = mid + 1;
        else r = mid - 1;
    }
    return 0;
}

uint64_t orc_tc_bsearch_i32(const int32_t *offsets, const int32_t *adjs, int32_t nodes,
                            int threads) {
    set_threads(threads);
    uint64_t total = 0;
    /* bs_tc.cu:120-148: one iteration per oriented edge (u, w) */
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : total)
    for (int32_t u = 0; u < nodes; ++u) {
        for (int32_t e = offsets[u]; e < offsets[u + 1]; ++e) {
            int32_t w = adjs[e];
            uint64_t cnt = 0;
            for (int32_t i = offsets[u]; i < offsets[u + 1]; ++i) {
                int32_t v = adjs[i];
                int32_t len = offsets[v + 1] - offsets[v];
                if (len == 0) continue;
                cnt += binary_check(adjs + offsets[v], 0, len - 1, w);
            }
            total += cnt;
        }
    }
    return total;
}

uint64_t orc_tc_bsearch_rows(const int32_t *offsets, const int32_t *adjs, const int32_t *rows,
                             int64_t nrows, int threads) {
    set_threads(threads);
    uint64_t total = 0;
    /* bs_tc.cu:120-148 restricted to the oriented edges whose source is listed in rows */
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
    for (int64_t r = 0; r < nrows; ++r) {
        int32_t u = rows[r];
        for (int32_t e = offsets[u]; e < offsets[u + 1]; ++e) {
            int32_t w = adjs[e];
            for (int32_t i = offsets[u]; i < offsets[u + 1]; ++i) {
                int32_t v = adjs[i];
                int32_t len = offsets[v + 1] - offsets[v];
                if (len == 0) continue;
                total += binary_check(adjs + offsets[v], 0, len - 1, w);
            }
        }
    }
    return total;
}

static int cmp_i32(const void *x, const void *y) {
    int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
    return a < b ? -1 : (a > b ? 1 : 0);
}

uint64_t orc_tc_hashmap_i32(const int32_t *offsets, const int32_t *adjs, int32_t nodes,
                            int threads) {
    set_threads(threads);
    uint64_t total = 0;
#pragma omp parallel reduction(+ : total)
    {
        int32_t *two = NULL;
        int64_t cap = 0;
#pragma omp for schedule(dynamic, 64)
        for (int32_t u = 0; u < nodes; ++u) {
            /* bs_tc.cu:171-183: gather the out-lists of u's out-neighbours */
            int64_t len = 0;
            for (int32_t j = offsets[u]; j < offsets[u + 1]; ++j) {
                int32_t v = adjs[j];
                len += offsets[v + 1] - offsets[v];
            }
            if (len == 0) continue;
            if (len > cap) {
                free(two);
                cap = len;
                two = (int32_t *)malloc((size_t)cap * sizeof(int32_t));
            }
            int64_t p = 0;
            for (int32_t j = offsets[u]; j < offsets[u + 1]; ++j) {
                int32_t v = adjs[j];
                int32_t l = offsets[v + 1] - offsets[v];
                memcpy(two + p, adjs + offsets[v], (size_t)l * sizeof(int32_t));
                p += l;
            }
            /* bs_tc.cu:185-205: sort + run-length encode into (u, w, cnt) */
            qsort(two, (size_t)len, sizeof(int32_t), cmp_i32);
            int32_t du = offsets[u + 1] - offsets[u];
            for (int64_t i = 0; i < len;) {
                int64_t j = i;
                while (j < len && two[j] == two[i]) ++j;
                /* bs_tc.cu:213-229: the triple counts when w is an out-neighbour of u */
                if (du > 0 && binary_check(adjs + offsets[u], 0, du - 1, two[i]))
                    total += (uint64_t)(j - i);
                i = j;
            }
        }
        free(two);
    }
    return total;
}

static uint32_t merge_count(const uint32_t *a, uint32_t la, const uint32_t *b, uint32_t lb) {
    uint32_t i = 0, j = 0, c = 0;
    while (i < la && j < lb) {
        if (a[i] < b[j]) ++i;
        else if (a[i] > b[j]) ++j;
        else {
            ++c;
            ++i;
            ++j;
        }
    }
    return c;
}

uint64_t orc_tc_merge(const uint64_t *off, const uint32_t *adj, uint32_t n, int threads) {
    set_threads(threads);
    uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : total)
    for (int64_t u = 0; u < (int64_t)n; ++u) {
        const uint32_t *A = adj + off[u];
        uint32_t a = (uint32_t)(off[u + 1] - off[u]);
        for (uint32_t j = 0; j < a; ++j) {
            uint32_t v = A[j];
            total += merge_count(A, a, adj + off[v], (uint32_t)(off[v + 1] - off[v]));
        }
    }
    return total;
}

/* -------------------------------------------------------- set intersection */

uint32_t orc_si_merge(const uint32_t *a, uint32_t la, const uint32_t *b, uint32_t lb) {
    /* ip.cu:266-287 with a_begin = b_begin = 0 and vt = la + lb steps */
    uint32_t ab = 0, bb = 0, count = 0;
    uint64_t vt = (uint64_t)la + lb;
    for (uint64_t i = 0; i < vt; ++i) {
        int flag = 0;
        if (ab >= la) flag = 0;
        else if (bb >= lb) flag = 1;
        else {
            if (a[ab] < b[bb]) flag = 1;
            if (a[ab] == b[bb]) count += 1;
        }
        if (flag) ab += 1;
        else bb += 1;
    }
    return count;
}

uint32_t orc_si_bsearch(const uint32_t *a, uint32_t la, const uint32_t *b, uint32_t lb) {
    /* bs.cu:341-370: every element of a is searched in b */
    uint32_t count = 0;
    for (uint32_t k = 0; k < la; ++k) {
        uint32_t target = a[k];
        int64_t l = 0, r = (int64_t)lb - 1;
        while (l <= r) {
            int64_t mid = l + (r - l) / 2;
            if (b[mid] == target) {
                count += 1;
                break;
            } else if (b[mid] > target) r = mid - 1;
            else l = mid + 1;
        }
    }
    return count;
}

void orc_si_pairs(const uint64_t *off, const uint32_t *elems, const uint32_t *pa,
                  const uint32_t *pb, uint64_t np, uint32_t *out, int threads) {
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < (int64_t)np; ++i) {
        uint32_t x = pa[i], y = pb[i];
        out[i] = merge_count(elems + off[x], (uint32_t)(off[x + 1] - off[x]), elems + off[y],
                             (uint32_t)(off[y + 1] - off[y]));
    }
}

void orc_si_dense(const uint64_t *off, const uint32_t *elems, uint32_t a0, uint32_t a1,
                  uint32_t b0, uint32_t b1, uint32_t *out, int threads) {
    set_threads(threads);
    const uint64_t nb = b1 - b0;
#pragma omp parallel for schedule(dynamic, 16) collapse(2)
    for (int64_t x = a0; x < (int64_t)a1; ++x)
        for (int64_t y = b0; y < (int64_t)b1; ++y)
            out[(uint64_t)(x - a0) * nb + (uint64_t)(y - b0)] =
                orc_si_merge(elems + off[x], (uint32_t)(off[x + 1] - off[x]), elems + off[y],
                             (uint32_t)(off[y + 1] - off[y]));
}

uint64_t orc_si_materialize(const uint64_t *off, const uint32_t *elems, const uint32_t *pa,
                            const uint32_t *pb, uint64_t np, uint64_t *out_off,
                            uint32_t *out_elems, uint64_t cap) {
    uint64_t w = 0;
    for (uint64_t p = 0; p < np; ++p) {
        out_off[p] = w;
        const uint32_t *a = elems + off[pa[p]], *b = elems + off[pb[p]];
        uint32_t la = (uint32_t)(off[pa[p] + 1] - off[pa[p]]);
        uint32_t lb = (uint32_t)(off[pb[p] + 1] - off[pb[p]]);
        uint32_t i = 0, j = 0;
        while (i < la && j < lb) {
            if (a[i] < b[j]) ++i;
            else if (a[i] > b[j]) ++j;
            else {
                if (w < cap) out_elems[w] = a[i];
                ++w;
                ++i;
                ++j;
            }
        }
    }
    out_off[np] = w;
    return w;
}

/* ------------------------------------------------------------------ workload generators
 * Seeded synthetic inputs for the timed CPU reference arm, so that it generates its
 * workload without the library under test. Same streams as the library's generators
 * (rt-graph_gb300/csrc/gen.cpp); the tests check that both give identical arrays. */

static inline uint64_t orc_splitmix64(uint64_t *x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline uint64_t orc_hash3(uint64_t seed, uint64_t a, uint64_t b) {
    uint64_t x = seed ^ (a * 0xD6E8FEB86659FD93ull) ^ (b * 0xA0761D6478BD642Full);
    return orc_splitmix64(&x);
}

static uint32_t orc_threshold32(double p) {
    if (p <= 0) return 0;
    if (p >= 1) return 0xFFFFFFFFu;
    return (uint32_t)floor(p * 4294967296.0);
}

int orc_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                 uint64_t seed, uint32_t *src, uint32_t *dst, int threads) {
    if (!src || !dst || scale == 0 || scale > 31 || edge_factor == 0) return -1;
    set_threads(threads);
    const uint64_t m = (uint64_t)edge_factor << scale;
    const uint32_t ta = orc_threshold32(a), tb = orc_threshold32(a + b),
                   tc = orc_threshold32(a + b + c);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)m; ++i) {
        uint32_t s = 0, d = 0;
        uint64_t r = 0;
        for (uint32_t l = 0; l < scale; ++l) {
            /* one 64-bit draw per two levels: low half for even levels, high half for odd */
            if ((l & 1) == 0) r = orc_hash3(seed, (uint64_t)i, l >> 1);
            const uint32_t u = (uint32_t)(r >> ((l & 1) ? 32 : 0));
            const uint32_t sb = u >= tb, db = (u >= ta && u < tb) || u >= tc;
            s = (s << 1) | sb;
            d = (d << 1) | db;
        }
        src[i] = s;
        dst[i] = d;
    }
    return 0;
}

/* xoshiro256** seeded by splitmix64, and Lemire's unbiased bounded draw (as in gen.cpp) */
typedef struct {
    uint64_t s[4];
} orc_xoshiro;

static void orc_xo_seed(orc_xoshiro *g, uint64_t seed) {
    uint64_t x = seed;
    for (int k = 0; k < 4; ++k) g->s[k] = orc_splitmix64(&x);
}

static inline uint64_t orc_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t orc_xo_next(orc_xoshiro *g) {
    uint64_t *s = g->s;
    const uint64_t r = orc_rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = orc_rotl(s[3], 45);
    return r;
}

static inline uint64_t orc_xo_below(orc_xoshiro *g, uint64_t n) {
    unsigned __int128 m = (unsigned __int128)orc_xo_next(g) * n;
    uint64_t l = (uint64_t)m;
    if (l < n) {
        const uint64_t t = (0 - n) % n;
        while (l < t) {
            m = (unsigned __int128)orc_xo_next(g) * n;
            l = (uint64_t)m;
        }
    }
    return (uint64_t)(m >> 64);
}

static int orc_cmp_u32(const void *a, const void *b) {
    const uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

/* sort ascending and drop repeats; returns the new length */
static size_t orc_sort_unique(uint32_t *v, size_t n) {
    if (n < 2) return n;
    qsort(v, n, 4, orc_cmp_u32);
    size_t w = 1;
    for (size_t i = 1; i < n; ++i)
        if (v[i] != v[w - 1]) v[w++] = v[i];
    return w;
}

static int orc_contains(const uint32_t *v, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (v[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && v[lo] == x;
}

int orc_gen_si_lengths(uint64_t npairs, double median, double sigma, uint32_t min_len,
                       uint32_t max_len, uint64_t seed, uint32_t *len, uint64_t *total,
                       int threads) {
    if (!len || !total || median <= 0 || sigma < 0 || min_len == 0 || max_len < min_len)
        return -1;
    set_threads(threads);
    const double mu = log(median);
    uint64_t tot = 0;
#pragma omp parallel for reduction(+ : tot) schedule(static)
    for (int64_t i = 0; i < (int64_t)(2 * npairs); ++i) {
        /* lognormal length by Box-Muller on two hashed uniforms, floored and clamped */
        const uint64_t r = orc_hash3(seed, 0x5151u, (uint64_t)i);
        const double u1 = ((double)(r >> 11) + 0.5) * 0x1.0p-53;
        const uint64_t r2 = orc_hash3(seed, 0x5152u, (uint64_t)i);
        const double u2 = (double)(r2 >> 11) * 0x1.0p-53;
        const double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
        const double x = floor(exp(mu + sigma * z));
        const uint32_t l =
            (x < (double)min_len) ? min_len : (x > (double)max_len ? max_len : (uint32_t)x);
        len[i] = l;
        tot += l;
    }
    *total = tot;
    return 0;
}

int orc_gen_si_lists(uint64_t npairs, uint32_t universe_log2, double overlap_max, uint64_t seed,
                     const uint32_t *len, uint64_t *offsets, uint32_t *elems, uint32_t *expected,
                     int threads) {
    if (!len || !offsets || !elems || !expected || universe_log2 == 0 || universe_log2 > 31)
        return -1;
    set_threads(threads);
    const uint64_t U = 1ull << universe_log2;
    offsets[0] = 0;
    uint32_t maxl = 0;
    for (uint64_t i = 0; i < 2 * npairs; ++i) {
        offsets[i + 1] = offsets[i] + len[i];
        if (len[i] > maxl) maxl = len[i];
    }
    int bad = 0;
#pragma omp parallel
    {
        uint32_t *buf = (uint32_t *)malloc(sizeof(uint32_t) * (maxl ? 2 * (size_t)maxl : 1));
        uint32_t *idx = (uint32_t *)malloc(sizeof(uint32_t) * (maxl ? maxl : 1));
        if (!buf || !idx) {
#pragma omp atomic write
            bad = 1;
        }
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < (int64_t)npairs; ++i) {
            if (!buf || !idx) continue;
            orc_xoshiro g;
            orc_xo_seed(&g, orc_hash3(seed, 0x5153u, (uint64_t)i));
            const uint64_t sa = 2 * (uint64_t)i, sb = sa + 1;
            const int a_long = len[sa] >= len[sb];
            const uint64_t sl = a_long ? sa : sb, ss = a_long ? sb : sa;
            const uint32_t L = len[sl], S = len[ss];
            uint32_t *Lp = elems + offsets[sl], *Sp = elems + offsets[ss];
            /* long list: L distinct uniform values, topped up after each sort + unique */
            size_t nb = 0;
            while (nb < L) {
                const size_t need = L - nb;
                for (size_t k = 0; k < need; ++k) buf[nb++] = (uint32_t)orc_xo_below(&g, U);
                nb = orc_sort_unique(buf, nb);
            }
            memcpy(Lp, buf, (size_t)L * 4);
            /* short list: k elements of the long list (partial Fisher-Yates), the rest
             * distinct values outside it */
            const double f = (double)(orc_xo_next(&g) >> 11) * 0x1.0p-53 * overlap_max;
            const uint32_t k = (uint32_t)floor(f * S);
            for (uint32_t t = 0; t < L; ++t) idx[t] = t;
            nb = 0;
            for (uint32_t t = 0; t < k; ++t) {
                const uint32_t r = t + (uint32_t)orc_xo_below(&g, L - t);
                const uint32_t tmp = idx[t];
                idx[t] = idx[r];
                idx[r] = tmp;
                buf[nb++] = Lp[idx[t]];
            }
            while (nb < S) {
                const size_t need = S - nb;
                for (size_t q = 0; q < need; ++q) {
                    const uint32_t x = (uint32_t)orc_xo_below(&g, U);
                    if (!orc_contains(Lp, L, x)) buf[nb++] = x;
                }
                nb = orc_sort_unique(buf, nb);
            }
            memcpy(Sp, buf, (size_t)S * 4);
            expected[i] = k;
        }
        free(buf);
        free(idx);
    }
    return bad ? -1 : 0;
}
