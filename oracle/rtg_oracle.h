/*
 * CPU oracle for the set-intersection path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of RT-Graph's reference algorithms for triangle counting and set
 * intersection, used by the tests, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg as the checker. librtg never links, loads or calls it.
 *
 * Parity is pinned: tests/golden/ holds outputs of the reference's own code
 * (tc/graph/graph.cpp and the host preprocessing of tc/bs_tc/bs_tc.cu compiled here from
 * the reference sources by oracle/build_ref.sh, and .s_data files written by the
 * reference's set_intersection/data_generator/data.cpp) and the oracle is checked
 * against every one of them by tests/test_oracle_golden.py.
 */
#ifndef RTG_ORACLE_H
#define RTG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* tc/graph/graph.cpp:40-62 — ids compacted in place to dense ranks of the used ids;
 * returns the number of used ids (the reference's graph_info_.nodes). */
int64_t orc_compact_ids(int32_t *pairs, int64_t m);

/* tc/graph/graph.cpp:104-177 then 71-102 — the reference's TC preprocessing and CSR on
 * compacted pairs (modified in place). offsets: nodes+1 capacity, adjs: m capacity.
 * Returns 0, or -1 on bad input. */
int orc_tc_preprocess_ref(int32_t *pairs, int64_t m, int32_t nodes, int32_t *offsets,
                          int32_t *adjs, int32_t *out_nodes, int64_t *out_edges);

/* Simple graph oriented low -> high (degree, id), degree counted after removing self loops
 * and duplicates. n = number of vertices (ids < n). offsets: n+1, adj: m capacity. */
int orc_csr_degree(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n,
                   uint64_t *offsets, uint32_t *adj, uint64_t *m_out);

/* Simple undirected graph with both directions stored. adj capacity 2m. */
int orc_csr_symmetric(const uint32_t *src, const uint32_t *dst, uint64_t m, uint32_t n,
                      uint64_t *offsets, uint32_t *adj, uint64_t *m_out);

/* tc/bs_tc/bs_tc.cu:120-148 (ListIntersectionKernel) with BinaryCheck (:14-25): for every
 * oriented edge (u, w) and every v in N+(u), binary-search w in N+(v). uint64 total. */
uint64_t orc_tc_bsearch_i32(const int32_t *offsets, const int32_t *adjs, int32_t nodes,
                            int threads);

/* The same rule restricted to the oriented edges whose source vertex is in rows[0..nrows):
 * the bounded sample used as the timed CPU baseline. */
uint64_t orc_tc_bsearch_rows(const int32_t *offsets, const int32_t *adjs, const int32_t *rows,
                             int64_t nrows, int threads);

/* tc/bs_tc/bs_tc.cu:153-211 (Preprocessing: per-vertex two-hop aggregation into
 * (u, w, cnt) triples) and :213-229 (HashmapKernel: add cnt when w in N+(u)). */
uint64_t orc_tc_hashmap_i32(const int32_t *offsets, const int32_t *adjs, int32_t nodes,
                            int threads);

/* An independent second opinion: sum over oriented edges (u, v) of |N+(u) ∩ N+(v)| by a
 * sorted merge. */
uint64_t orc_tc_merge(const uint64_t *off, const uint32_t *adj, uint32_t n, int threads);

/* set_intersection/baseline/ip.cu:266-287 (SerialIntersection) walked over both whole
 * lists. */
uint32_t orc_si_merge(const uint32_t *a, uint32_t la, const uint32_t *b, uint32_t lb);

/* set_intersection/baseline/bs.cu:341-370 (per-element binary search of one list's
 * elements in the other). */
uint32_t orc_si_bsearch(const uint32_t *a, uint32_t la, const uint32_t *b, uint32_t lb);

/* Per-pair counts: out[i] = |S[pa[i]] ∩ S[pb[i]]|. */
void orc_si_pairs(const uint64_t *off, const uint32_t *elems, const uint32_t *pa,
                  const uint32_t *pb, uint64_t np, uint32_t *out, int threads);

/* Dense A x B in the reference's row-major order (bs.cu:93-96,148). */
void orc_si_dense(const uint64_t *off, const uint32_t *elems, uint32_t a0, uint32_t a1,
                  uint32_t b0, uint32_t b1, uint32_t *out, int threads);

/* Materialised intersections: out_off has np+1 entries; out_elems capacity cap.
 * Returns the total needed. */
uint64_t orc_si_materialize(const uint64_t *off, const uint32_t *elems, const uint32_t *pa,
                            const uint32_t *pb, uint64_t np, uint64_t *out_off,
                            uint32_t *out_elems, uint64_t cap);

#ifdef __cplusplus
}
#endif
#endif
