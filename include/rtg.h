/*
 * rtg.h — C ABI of librtg, the GB300 (sm_103a) implementation of RT-Graph's
 * sorted-adjacency set-intersection path: triangle counting (TC) and batched
 * pairwise set-intersection counting (SI).
 *
 * Every entry point is plain C: pointers, sizes and status codes, no C++ or torch
 * types. Every function returns an rtg_status and never calls exit(); the text of
 * the last error on a context is available from rtg_last_error().
 *
 * Reference interfaces replaced (paths are relative to the RT-Graph repository):
 *   - Graph::ReadBinaryEdges / TCPreprocessing / ConvertToCSR / Txt2Bin
 *       tc/graph/include/graph.h:13-20, tc/graph/graph.cpp:23-214
 *   - void CountOnGPU(int *adjs, int *offsets, int nodes, int edges, int device_id)
 *       tc/bs_tc/bs_tc.h:5, tc/bs_tc/bs_tc.cu:232-354
 *   - class RTTC { BuildBVHAndComputeRay; CountTriangles; total_triangles_ }
 *       tc/rt_tc/include/rt_tc.h:7-59
 *   - XxxBasedIntersection(const Dataset&, uint blocks, uint block_size, std::vector<uint>&)
 *       set_intersection/baseline/bs.cu:21-22, hi.cu:22-23, ip.cu:32-33,
 *       bi_naive.cu:26-27, bi_dynamic.cu:24-25
 *   - class RTInter { BuildBVHAndComputeRay(Dataset); CountIntersection(std::vector<uint>&) }
 *       set_intersection/rt/include/rt_intersection.h:7-29
 *   - ReadData / Check / struct Dataset
 *       set_intersection/utils/util.h:19-36, util.cpp:3-51
 *
 * Threading: one rtg_ctx per host thread; a context owns one CUDA stream and all
 * calls on it are ordered on that stream. Graphs and set collections belong to the
 * context that created them.
 */
#ifndef RTG_H
#define RTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RTG_ABI_VERSION 3

/* Status codes. The reference prints and calls exit(2) on any CUDA error
 * (tc/utils/common.h:13-32); librtg returns one of these instead. */
typedef enum rtg_status {
    RTG_OK = 0,
    RTG_ERR_INVALID_ARG = 1, /* null pointer, size out of range, unsorted list ... */
    RTG_ERR_OOM = 2,         /* device, pinned-host or host allocation failed      */
    RTG_ERR_IO = 3,          /* file could not be opened / read / written          */
    RTG_ERR_FORMAT = 4,      /* malformed input file                               */
    RTG_ERR_DEVICE = 5,      /* CUDA runtime error (text in rtg_last_error)        */
    RTG_ERR_TIMEOUT = 6,     /* a bounded device wait ran out (status word)        */
    RTG_ERR_CANCELLED = 7,   /* request cancelled before completion                */
    RTG_ERR_STATE = 8,       /* call out of order, e.g. count before rtg_csr_build */
    RTG_ERR_BUSY = 9         /* admission refused: no slot or memory budget left   */
} rtg_status;

typedef struct rtg_ctx rtg_ctx;
typedef struct rtg_graph rtg_graph;
typedef struct rtg_sets rtg_sets;

/* Input formats of rtg_graph_load.
 *  EDGE_BIN : int32 (src,dst) pairs back to back, the reference's binary edge list
 *             (tc/graph/graph.cpp:23-38).
 *  EDGE_TXT : "src dst" per line, as read by Graph::Txt2Bin (graph.cpp:179-214).
 *  MTX      : MatrixMarket coordinate file, 1-based (bfs/graph/graph.cpp:17-122). */
typedef enum rtg_format {
    RTG_FMT_EDGE_BIN = 0,
    RTG_FMT_EDGE_TXT = 1,
    RTG_FMT_MTX = 2,
    RTG_FMT_RTG_CSR = 3 /* CSR cache written by rtg_graph_save (rtg_graph_load only) */
} rtg_format;

/* CSR kinds built by rtg_csr_build.
 *  DEGREE          : simple undirected graph (self loops and duplicates removed), each
 *                    edge oriented from the endpoint of lower degree to the higher one,
 *                    ties to the smaller id. Vertex ids are kept.
 *  DEGREE_RAW_REF  : the reference's exact preprocessing, bit for bit: ids compacted to
 *                    dense ranks (graph.cpp:40-62), orientation by the degree counted on
 *                    the raw list including duplicates (graph.cpp:108-124), vertices of
 *                    raw degree <= 1 dropped and ids renumbered (graph.cpp:126-149),
 *                    then sort, duplicate and self-loop removal, CSR (graph.cpp:154-173,
 *                    71-102).
 *  SYMMETRIC       : unoriented simple graph, both directions stored (used for vertex-
 *                    pair queries). Held beside the oriented CSR, not in place of it. */
typedef enum rtg_orient {
    RTG_ORIENT_DEGREE = 0,
    RTG_ORIENT_DEGREE_RAW_REF = 1,
    RTG_ORIENT_SYMMETRIC = 2
} rtg_orient;

/* Triangle-count forms. PLAIN: the reference's per-edge formulation (one warp per oriented
 * edge, one launch per degree/ratio bucket). BATCHED: the counting form streamed by the
 * persistent kernel from a device queue, replayed from a CUDA graph, autotunable; edges
 * among the top ranks (the dense core, rtg_config.tc_core_ranks) are counted as word ANDs
 * of the core's adjacency bit matrix, the other in-edges are streamed. BUCKETED: the same
 * counting-form kernels without persistence or graph: work items built on every call, one
 * launch per item-size bucket with one warp per item, the library's default schedule and
 * the context's core setting (it separates what the algorithm and what the scheduling
 * contribute). */
typedef enum rtg_tc_mode { RTG_TC_PLAIN = 0, RTG_TC_BATCHED = 1, RTG_TC_BUCKETED = 2 } rtg_tc_mode;

/* Set-intersection execution forms (flags of rtg_si_count*).
 *  AUTO   : BATCHED form — one persistent launch; both lists of every pair (or of every
 *           chunk pair of a long pair) are staged into shared memory by bulk copies and
 *           merged there; by default one warp per block forms the jobs and issues their
 *           copies into a ring of slots that the block's other warps merge (si_form); a
 *           pair longer than a staging slot whose long list exceeds si_search_ratio
 *           (default 8) x the short one is binary-searched from global memory instead.
 *  PLAIN  : per-pair family from global memory: SEARCH when |long| > si_search_ratio
 *           (default 32) x |short|, MERGE otherwise.
 *  FORCE_*: one family for every pair; these back the reference's per-baseline CLIs. */
#define RTG_SI_AUTO 0u
#define RTG_SI_FORCE_MERGE 1u   /* warp merge path (ip.cu)                        */
#define RTG_SI_FORCE_SEARCH 2u  /* short list searched in the long list (bs.cu)   */
#define RTG_SI_FORCE_BITMAP 3u  /* block bitmap / hash probe (bi_dynamic.cu, hi.cu) */
#define RTG_SI_PLAIN 4u
#define RTG_SI_FAMILY_MASK 0xFu
#define RTG_PAIRS_DEVICE 0x100u /* pair arrays are device pointers                 */
#define RTG_OUT_DEVICE 0x200u   /* output array is a device pointer                */

/* Per-call timing and counters. All times in milliseconds. Device times come from CUDA
 * events on the context stream. */
typedef struct rtg_timing {
    double h2d_ms;            /* host -> device copies made by the call (0 when the
                                 kernel reads page-locked host memory itself)      */
    double build_ms;          /* CSR build / set upload stage                     */
    double count_ms;          /* counting stage (all kernels of the stage)        */
    double main_kernel_ms;    /* the dominant counting kernel alone               */
    double d2h_ms;            /* device -> host copies made by the call           */
    double total_ms;          /* host wall time of the call                       */
    uint64_t kernel_launches; /* librtg kernels launched by the call (graph nodes
                                 count one each)                                   */
    uint64_t algo_bytes;      /* algorithmic bytes of the counting stage          */
    uint64_t h2d_bytes;
    uint64_t d2h_bytes;
    double core_ms;           /* BATCHED / BUCKETED count: the dense-core stage (core
                                 matrix build + core count), part of count_ms        */
    uint32_t core_ranks;      /* ... and the top ranks it covered (0: no core)      */
    uint32_t reserved;
} rtg_timing;

typedef struct rtg_graph_info {
    uint32_t n;              /* vertices of the oriented CSR                      */
    uint64_t m_input;        /* input (raw) edges                                 */
    uint64_t m;              /* edges of the oriented CSR = undirected simple m   */
    uint32_t max_out_degree; /* max d+ of the oriented CSR                        */
    uint64_t work_elems;     /* sum over oriented (u,v) of d+(u)+d+(v)            */
    int32_t orient;          /* rtg_orient of the oriented CSR, -1 if not built   */
    int32_t has_symmetric;   /* 1 when the symmetric CSR is built                 */
    uint32_t n_sym;          /* vertices of the symmetric CSR                     */
    uint64_t m_sym;          /* directed entries of the symmetric CSR (= 2 m)     */
} rtg_graph_info;

/* Tunable schedule of the BATCHED triangle count and of the SI pair kernels. Zero in
 * any field means "library default". */
typedef struct rtg_config {
    uint32_t tc_block_warps;    /* warps per block of the persistent TC kernel        */
    uint32_t tc_item_edges;     /* in-edges of one vertex per work item (default: 1024
                                   from 2^23 oriented edges up, else 256)            */
    uint32_t tc_region_words;   /* 32-bit words of shared memory per warp for the
                                   out-list of the item's vertex: a bitmap of 32x that
                                   many ranks, or a hash table (power of two, 64..16384) */
    uint32_t tc_blocks_per_sm;  /* resident blocks per SM of the persistent kernel    */
    uint32_t si_block_warps;    /* warps per block of the SI kernels                  */
    uint32_t si_search_ratio;   /* long/short length ratio above which the forced-
                                   family-free PLAIN form uses SEARCH                 */
    uint32_t si_stage_slots;    /* bulk-copy staging slots per warp, or per block in the
                                   producer/consumer form (2..32)                     */
    uint32_t si_stage_bytes;    /* bytes per staging slot (multiple of 128, 512..32768) */
    uint32_t si_blocks_per_sm;  /* resident blocks per SM of the batched SI kernel    */
    uint32_t si_skew_stream;    /* 1: a skewed pair longer than a staging slot whose short
                                   list fits a slot's table is counted by staging the short
                                   list in shared memory (bulk copy) and streaming the long
                                   list from HBM in 16-byte loads, when that reads fewer
                                   sectors than searching it; 0 (default): always searched */
    uint32_t si_form;           /* batched SI kernel form: 1 = every warp forms its own jobs
                                   and merges them (si_stage_slots slots per warp); 2 =
                                   producer/consumer: one warp per block forms the jobs and
                                   issues their bulk copies into a ring of si_stage_slots
                                   slots shared by si_block_warps merging warps; 0 = library
                                   default                                            */
    uint32_t tc_core_ranks;     /* dense core of the BATCHED / BUCKETED triangle count: the
                                   top min(value, n) ranks (1..32768) have their
                                   adjacency held as a bit matrix, and their edges are
                                   counted by word AND + popcount; RTG_TC_CORE_NONE: no
                                   core; 0 = library choice (the largest of 32768, 24576,
                                   16384, 12288, 8192, 6144, 4096, 3072, 2048, 1536,
                                   1024 top ranks whose edge density is at least 2.5 %,
                                   none if no such core)                             */
} rtg_config;

#define RTG_TC_CORE_NONE 0xFFFFFFFFu
#define RTG_TC_CORE_MAX_RANKS 32768u

/* ---------------------------------------------------------------- context */
rtg_status rtg_init(int device, rtg_ctx **out);
/* Also releases every graph and set collection still attached to the context; their
 * handles are invalid afterwards. */
void rtg_destroy(rtg_ctx *ctx);
const char *rtg_last_error(const rtg_ctx *ctx);
const char *rtg_status_str(rtg_status s);
int rtg_abi_version(void);
rtg_status rtg_set_config(rtg_ctx *ctx, const rtg_config *cfg);
rtg_status rtg_get_config(const rtg_ctx *ctx, rtg_config *cfg);
/* 1 in the checked build (librtg_checked.so, compiled with RTG_CHECKED), 0 otherwise; no
 * counterpart in the reference, which has no checked build. The checked build validates
 * every CSR and counting form on the device before a count reads it (offsets, ids, row
 * order, suffix ranges) and checks the indexes the counting kernels derive from them; a
 * violation is reported as RTG_ERR_FORMAT through the device status word, never as a
 * fault. */
int rtg_checked_build(void);
/* Test hook of the checked build (RTG_ERR_STATE in any other build); no counterpart in the
 * reference. With on != 0, rtg_graph_load(RTG_FMT_RTG_CSR) checks a cache file's sizes and
 * checksum only, not its structure, so that a forged form reaches the device-side checks.
 * Process-wide. */
rtg_status rtg_debug_skip_file_checks(int on);
/* Cumulative number of librtg kernel launches on this context. */
uint64_t rtg_kernel_launches(const rtg_ctx *ctx);
rtg_status rtg_synchronize(rtg_ctx *ctx);
/* Overwrite a device buffer larger than L2 so the next call starts cold. */
rtg_status rtg_flush_l2(rtg_ctx *ctx);
/* Device properties used by schedules (SM count, shared memory per block). */
rtg_status rtg_device_info(const rtg_ctx *ctx, int *sm_count, int *smem_per_block_optin,
                           int *cc_major, int *cc_minor);
/* Pinned host memory for callers that want page-locked staging buffers. */
rtg_status rtg_host_alloc(rtg_ctx *ctx, size_t bytes, void **out);
void rtg_host_free(void *p);

/* ----------------------------------------------------------------- graphs */
/* Edges as two uint32 arrays (host). The arrays are copied; the caller keeps them. */
rtg_status rtg_graph_from_host_edges(rtg_ctx *ctx, const uint32_t *src, const uint32_t *dst,
                                     uint64_t m, rtg_graph **out);
/* Edges in the reference's edge_t layout: int32 {src,dst} pairs (tc/utils/model.h:16-29). */
rtg_status rtg_graph_from_host_pairs(rtg_ctx *ctx, const int32_t *pairs, uint64_t m,
                                     rtg_graph **out);
/* Edges already on the device (copied into the graph). */
rtg_status rtg_graph_from_device_edges(rtg_ctx *ctx, const uint32_t *d_src,
                                       const uint32_t *d_dst, uint64_t m, rtg_graph **out);
rtg_status rtg_graph_load(rtg_ctx *ctx, const char *path, rtg_format fmt, rtg_graph **out);
/* Build a CSR on the GPU (radix sort, dedup, self-loop removal, orientation). */
rtg_status rtg_csr_build(rtg_ctx *ctx, rtg_graph *g, rtg_orient orient);
/* A CSR given directly by the caller (host arrays, int32 like the reference's
 * Graph::adjs_/offsets_): rows must be sorted ascending and oriented (a DAG). */
rtg_status rtg_graph_from_host_csr(rtg_ctx *ctx, const int32_t *offsets, const int32_t *adjs,
                                   int32_t nodes, int64_t edges, rtg_graph **out);
rtg_status rtg_graph_info_get(const rtg_graph *g, rtg_graph_info *info);
/* Device pointers owned by the graph; valid until rtg_graph_destroy. */
rtg_status rtg_csr_view(const rtg_graph *g, int symmetric, const uint64_t **d_offsets,
                        const uint32_t **d_adj, uint32_t *n, uint64_t *m);
/* Copy a CSR to caller-allocated host arrays (offsets: n+1 entries, adj: m entries). */
rtg_status rtg_csr_to_host(rtg_ctx *ctx, const rtg_graph *g, int symmetric, uint64_t *offsets,
                           uint32_t *adj);
/* Free the raw edge buffer once the CSRs needed are built. */
rtg_status rtg_graph_release_edges(rtg_graph *g);
/* Device bytes currently held by the graph. */
uint64_t rtg_graph_device_bytes(const rtg_graph *g);
/* On-disk CSR cache: write every CSR the graph holds (oriented, counting form, symmetric)
 * to one file; rtg_graph_load(ctx, path, RTG_FMT_RTG_CSR, &g) reads it back without the
 * sort-based build (the graph then has no raw edges). A file whose checksum or structure
 * does not hold is refused with RTG_ERR_FORMAT. No reference counterpart: the reference
 * rebuilds its CSR (tc/graph/graph.cpp:71-102) on every run. */
rtg_status rtg_graph_save(rtg_ctx *ctx, const rtg_graph *g, const char *path);
/* The checks rtg_graph_load(RTG_FMT_RTG_CSR) runs before anything reaches the device, on
 * the host alone (no context, no GPU): RTG_OK for a file it would accept, RTG_ERR_FORMAT
 * for a damaged or forged one (checksum, sizes, offsets, ids below n, counting-form rows
 * ascending and above their vertex, every in-edge suffix range inside one row and holding
 * only ranks above its head), RTG_ERR_IO when it cannot be read. */
rtg_status rtg_graph_file_check(const char *path);
void rtg_graph_destroy(rtg_graph *g);

/* ------------------------------------------------------ triangle counting */
/* Exact uint64 triangle count of the oriented CSR of g (BATCHED and BUCKETED read its
 * counting form, which is all a graph read from a counting-form-only cache file holds). */
rtg_status rtg_tc_count(rtg_ctx *ctx, rtg_graph *g, rtg_tc_mode mode, uint64_t *out_total,
                        rtg_timing *timing);
/* End to end from host edges: copy in, build the CSR with `orient`, count, copy the
 * total out. The drop-in for the bs_tc / rt_tc pipelines. With RTG_ORIENT_DEGREE and
 * RTG_TC_BATCHED the edges, the counting form and the count's buffers are kept in the
 * context's grow-only scratch (about 21 bytes per edge, released by rtg_destroy), so
 * repeated calls allocate nothing once it has grown; that form takes at most 2^32 - 1
 * edges and vertex ids below 2^31 - 1 (RTG_ERR_INVALID_ARG otherwise, before anything is
 * sized by the ids). */
rtg_status rtg_tc_count_host_edges(rtg_ctx *ctx, const uint32_t *src, const uint32_t *dst,
                                   uint64_t m, rtg_orient orient, rtg_tc_mode mode,
                                   uint64_t *out_total, rtg_timing *timing);
/* Per-edge triangle lists on the oriented CSR of g (built with rtg_csr_build, or a host
 * CSR): for oriented edge e = (u -> v) in CSR order (u its row, v = adj[e]) the ids w of
 * N+(u) ∩ N+(v), ascending, in out_elems[out_offsets[e] .. out_offsets[e+1]). Every
 * triangle of the graph appears exactly once, as (u, v, w) for its edge e = (u -> v);
 * out_offsets[m] is the triangle count. The reference only counts (tc/bs_tc/bs_tc.cu:
 * 120-148); the lists are the same sum written out. out_offsets has m + 1 entries; when
 * out_capacity is too small the call fails with RTG_ERR_INVALID_ARG and out_offsets[m]
 * holds the number of entries needed. Host arrays. */
rtg_status rtg_tc_list(rtg_ctx *ctx, rtg_graph *g, uint64_t *out_offsets, uint32_t *out_elems,
                       uint64_t out_capacity, rtg_timing *timing);
/* Replaces CountOnGPU (tc/bs_tc/bs_tc.h:5): host int32 CSR in, count out (uint64
 * instead of the reference's uint32). Rows must be strictly ascending with ids in
 * [0, nodes) (RTG_ERR_INVALID_ARG otherwise). PLAIN counts the CSR as given (an acyclic
 * orientation with every edge once, as the reference's preprocessing writes it); BATCHED
 * counts the CSR's edges as a one-shot edge list (counting form built from them, direct
 * launches), BUCKETED through a graph handle. */
rtg_status rtg_tc_count_host_csr(rtg_ctx *ctx, const int32_t *offsets, const int32_t *adjs,
                                 int32_t nodes, int64_t edges, rtg_tc_mode mode,
                                 uint64_t *out_total, rtg_timing *timing);
/* Allocation-free triangle count. No counterpart in the reference: it exists for callers
 * that cannot let a library call cudaMalloc, for example code running inside an
 * application whose memory pool or framework allocator owns the device heap, or code on a
 * latency-critical path where the implicit device synchronisation of an allocation is not
 * allowed. It needs no rtg_ctx.
 *
 * Input: an oriented CSR already on the current device (d_offsets: n+1 entries, d_adj: m
 * entries, rows sorted ascending, every edge stored once). The orientation must be
 * acyclic (every edge from the lower to the higher vertex of one total order, by degree
 * rank or by id) and hold no self loops: a cyclically oriented triangle adds nothing and a
 * self loop adds spurious counts, and neither is detected. The library's own oriented CSR
 * (rtg_csr_view with symmetric = 0 after rtg_csr_build) is such an input. Output: the
 * exact uint64 triangle count written to the host word *out_total. Work is ordered on `stream`
 * (a cudaStream_t; NULL for the default stream) and the call returns when the count is
 * on the host. It uses the PLAIN kernels; their scratch lives in one fixed device array
 * inside the library (about 9 bytes per edge for RTG_NOALLOC_MAX_EDGES edges, reserved on
 * every GPU that loads the library until the process exits), so:
 *   - graphs with more than RTG_NOALLOC_MAX_EDGES edges are rejected with
 *     RTG_ERR_INVALID_ARG before any GPU work, as are offsets that do not describe a CSR of
 *     m edges with ids below n;
 *   - the first call on a device looks up the array's device address (once per device, with
 *     that device current). With lazy module loading (the CUDA default) the array itself is
 *     reserved when the library's code is first loaded on that device, which may be during
 *     that first call: make it at start-up, before another allocator takes over the device
 *     heap and before any stream capture;
 *   - the looked-up address is kept for the life of the process: do not use this entry
 *     point on a device after cudaDeviceReset (or any reset of its primary context);
 *   - every call on a device shares the one array, so calls that overlap on the GPU (other
 *     host threads, other streams) race and must be serialised by the caller.
 * Returns RTG_ERR_DEVICE on a CUDA error. It calls no cudaMalloc, cudaFree or other
 * allocating routine. */
#define RTG_NOALLOC_MAX_EDGES (1u << 19)
rtg_status rtg_tc_count_device_csr_noalloc(const uint64_t *d_offsets, const uint32_t *d_adj,
                                           uint32_t n, uint64_t m, uint64_t *out_total,
                                           void *stream);
/* |N(u) ∩ N(v)| on the symmetric CSR for each query pair (u[i], v[i]). */
rtg_status rtg_graph_pair_count(rtg_ctx *ctx, rtg_graph *g, const uint32_t *u,
                                const uint32_t *v, uint64_t npairs, uint32_t *out,
                                uint32_t flags, rtg_timing *timing);

/* --------------------------------------------------------- set collections */
/* nsets sorted, duplicate-free uint32 lists; offsets has nsets+1 entries. */
rtg_status rtg_sets_from_host(rtg_ctx *ctx, const uint64_t *offsets, uint64_t nsets,
                              const uint32_t *elems, rtg_sets **out);
/* The reference Dataset layout (uint32 offsets, set_intersection/utils/util.h:19-28). */
rtg_status rtg_sets_from_host_u32(rtg_ctx *ctx, const uint32_t *offsets, uint32_t nsets,
                                  const uint32_t *elems, rtg_sets **out);
uint64_t rtg_sets_count(const rtg_sets *s);
uint64_t rtg_sets_elems(const rtg_sets *s);
void rtg_sets_destroy(rtg_sets *s);

/* |S[pair_a[i]] ∩ S[pair_b[i]]| for i < npairs. flags: RTG_SI_* family, RTG_PAIRS_DEVICE,
 * RTG_OUT_DEVICE. Host pair and count arrays in page-locked memory (rtg_host_alloc,
 * cudaHostAlloc, cudaHostRegister) are read and written by the kernel itself over the
 * host link, with no staging copies (timing->h2d_bytes / d2h_bytes count the bytes moved,
 * h2d_ms / d2h_ms stay 0); pageable host arrays are copied through device memory. */
rtg_status rtg_si_count(rtg_ctx *ctx, const rtg_sets *s, const uint32_t *pair_a,
                        const uint32_t *pair_b, uint64_t npairs, uint32_t *out_counts,
                        uint32_t flags, rtg_timing *timing);
/* Test hook for the bounded device waits; no counterpart in the reference (whose CUDA
 * error path prints and exits, tc/utils/common.h:13-32). For the next batched
 * (RTG_SI_AUTO) launch on ctx only: one warp of the staging kernel arms its shared-memory
 * barrier for extra_tx_bytes (a multiple of 16, not 0) that no copy brings, so that phase
 * never completes and its wait, bounded at max_polls polls (the kernel's waits default to
 * 2^22), runs out. The warp records RTG_ERR_TIMEOUT in the status word (in the per-warp
 * form it then leaves before taking any pairs; in the producer/consumer form the producer
 * arms a barrier of its own and goes on), nothing stays in flight, and the call returns
 * RTG_ERR_TIMEOUT with the context still usable. */
rtg_status rtg_debug_si_wait_limit(rtg_ctx *ctx, uint32_t max_polls, uint32_t extra_tx_bytes);
/* Dense |A| x |B| in the reference's row-major order (bs.cu:93-96,148):
 * out[(a - a_begin) * (b_end - b_begin) + (b - b_begin)]. */
rtg_status rtg_si_count_dense(rtg_ctx *ctx, const rtg_sets *s, uint32_t a_begin,
                              uint32_t a_end, uint32_t b_begin, uint32_t b_end,
                              uint32_t *out_counts, uint32_t flags, rtg_timing *timing);
/* Materialised intersections: out_offsets (npairs+1 entries) and the elements of every
 * intersection back to back in out_elems (capacity out_capacity entries; when it is too
 * small the call fails with RTG_ERR_INVALID_ARG and out_offsets[npairs] holds the size
 * needed). Host arrays. */
rtg_status rtg_si_materialize(rtg_ctx *ctx, const rtg_sets *s, const uint32_t *pair_a,
                              const uint32_t *pair_b, uint64_t npairs, uint64_t *out_offsets,
                              uint32_t *out_elems, uint64_t out_capacity, rtg_timing *timing);

/* --------------------------------------------------------------- autotuning
 * Time a grid of schedules for the batched forms (after an L2 flush, median of three
 * runs each), keep the fastest whose result is bit-identical to the default schedule's,
 * and set it on the context. TC: tc_item_edges x tc_region_words x tc_block_warps. SI:
 * si_form x si_stage_bytes x si_stage_slots x si_block_warps x si_search_ratio, on the pairs given
 * (host arrays; a representative sample of the workload). With cache_path (a text file,
 * created if missing) the winner is stored under a key of the device and the workload's
 * size class, and a later call with the same key applies it without searching. */
typedef struct rtg_tune_result {
    rtg_config best;
    double best_ms;      /* median time of the winner                        */
    double default_ms;   /* median time of the library default               */
    uint32_t candidates; /* schedules tried                                   */
    uint32_t rejected;   /* did not fit the device or did not match the count */
    uint32_t from_cache; /* 1: taken from the cache, nothing was timed        */
    uint32_t reserved;
} rtg_tune_result;
rtg_status rtg_tune_tc(rtg_ctx *ctx, rtg_graph *g, const char *cache_path, rtg_tune_result *res);
rtg_status rtg_tune_si(rtg_ctx *ctx, const rtg_sets *s, const uint32_t *pair_a,
                       const uint32_t *pair_b, uint64_t npairs, const char *cache_path,
                       rtg_tune_result *res);

/* ----------------------------------------------------------------- serving
 * A request loop over many graphs resident in HBM. No counterpart in the reference,
 * whose mains run one graph or one dataset per process; it serves the reference's two
 * computations as requests: the triangle count of a graph (what CountOnGPU prints,
 * tc/bs_tc/bs_tc.cu:232-354) and intersection counts |N(u) ∩ N(v)| of vertex pairs on a
 * graph's symmetric adjacency (the per-pair count of the SI baselines).
 *
 * rtg_serve_start creates the server and its engine thread on one device. Graphs are
 * built on the GPU from host edges (the symmetric CSR for pair queries and the oriented
 * counting form for triangle counts) and stay resident until removed. Submissions are
 * thread-safe and return at once with a request id. The engine admits work against the
 * HBM budget; packs the pair requests waiting at each launch point, of any graphs and any
 * sizes, into one persistent set-intersection launch (up to si_slots launches in flight
 * on their own streams); runs triangle counts as CUDA-graph replays on another stream, so
 * both kinds overlap on the device; coalesces triangle-count requests of one graph that
 * wait together; and completes requests as their launches finish.
 *
 * Borrowed buffers: the pair arrays u, v and the output out_counts of
 * rtg_serve_submit_pairs are read and written by the engine after the call returns; they
 * must stay valid until the request is reported complete (rtg_serve_poll or
 * rtg_serve_wait_any returned it) or rtg_serve_stop returned. */
typedef struct rtg_server rtg_server;

typedef struct rtg_serve_config {
    uint64_t hbm_budget_bytes; /* resident graphs + counting plans + launch buffers;
                                  0 = 90% of the free device memory at start            */
    uint32_t max_batch_pairs;  /* pairs per set-intersection launch (default 1 << 19)   */
    uint32_t si_slots;         /* set-intersection launches in flight (default 2; 1..4) */
    uint32_t max_graphs;       /* resident graph slots (default 1024)                   */
    uint32_t flags;            /* RTG_SERVE_*                                           */
    uint32_t inject_fail_launch; /* testing: the n-th set-intersection launch (1-based)
                                    is reported failed on the host, as if its completion
                                    query had returned an error (0 = off)              */
    uint32_t reserved;
} rtg_serve_config;

/* The engine launches nothing until rtg_serve_release (deterministic tests). */
#define RTG_SERVE_START_HELD 0x1u

typedef enum rtg_request_kind { RTG_REQ_TC = 0, RTG_REQ_PAIRS = 1 } rtg_request_kind;

typedef struct rtg_request_info {
    rtg_status status;       /* OK, CANCELLED, DEVICE, TIMEOUT, OOM                      */
    uint32_t kind;           /* rtg_request_kind                                          */
    uint32_t graph;
    uint32_t launches;       /* launches the request took part in                        */
    uint32_t batch_requests; /* most requests that shared one of those launches          */
    uint32_t reserved;
    uint64_t npairs;
    uint64_t triangles;      /* RTG_REQ_TC                                                */
    double latency_ms;       /* submission -> completion                                 */
    double queue_ms;         /* submission -> first launch                               */
} rtg_request_info;

typedef struct rtg_serve_stats {
    uint64_t submitted, completed, failed, cancelled;
    uint64_t tc_launches, tc_coalesced;   /* TC requests served by another's launch      */
    uint64_t si_launches, si_pairs, max_requests_per_launch;
    uint64_t max_inflight_launches;       /* TC + SI launches in flight at one time      */
    uint64_t resident_graphs, resident_bytes, plan_bytes, buffer_bytes, budget_bytes;
    uint64_t plan_evictions, admission_waits;
    uint64_t tc_direct;  /* TC launches without a cached plan (shared run scratch)       */
} rtg_serve_stats;

rtg_status rtg_serve_start(int device, const rtg_serve_config *cfg, rtg_server **out);
/* Cancels queued requests, waits for launches in flight, frees every graph. */
void rtg_serve_stop(rtg_server *s);
/* Text of the server's most recent error; the returned string belongs to the calling
 * thread and stays valid until that thread's next call. */
const char *rtg_serve_last_error(const rtg_server *s);
/* Build a resident graph from host edges (copied). RTG_ERR_OOM when it does not fit the
 * budget, RTG_ERR_BUSY when every graph slot is taken. */
rtg_status rtg_serve_add_graph(rtg_server *s, const uint32_t *src, const uint32_t *dst,
                               uint64_t m, uint32_t *graph_id);
/* With RTG_FMT_RTG_CSR the file must hold the counting form and the symmetric CSR (as
 * written by rtg_serve_save_graph); nothing is rebuilt. */
rtg_status rtg_serve_add_graph_file(rtg_server *s, const char *path, rtg_format fmt,
                                    uint32_t *graph_id);
/* Write a resident graph to a CSR cache file for a later rtg_serve_add_graph_file. */
rtg_status rtg_serve_save_graph(rtg_server *s, uint32_t graph_id, const char *path);
/* New requests on the graph are refused at once; it is freed when its last queued or
 * running request completes. */
rtg_status rtg_serve_remove_graph(rtg_server *s, uint32_t graph_id);
rtg_status rtg_serve_graph_info(rtg_server *s, uint32_t graph_id, rtg_graph_info *info);
rtg_status rtg_serve_submit_tc(rtg_server *s, uint32_t graph_id, uint64_t *request_id);
/* Vertex ids must be below the graph's n_sym (checked here: RTG_ERR_INVALID_ARG). */
rtg_status rtg_serve_submit_pairs(rtg_server *s, uint32_t graph_id, const uint32_t *u,
                                  const uint32_t *v, uint64_t npairs, uint32_t *out_counts,
                                  uint64_t *request_id);
/* wait_ms: 0 polls, < 0 waits without limit. RTG_OK with *info once the request is
 * complete (the id is then forgotten); RTG_ERR_BUSY while it is not; RTG_ERR_INVALID_ARG
 * for an unknown id. */
rtg_status rtg_serve_poll(rtg_server *s, uint64_t request_id, int32_t wait_ms,
                          rtg_request_info *info);
/* The next completed request not yet collected, in completion order. */
rtg_status rtg_serve_wait_any(rtg_server *s, int32_t wait_ms, uint64_t *request_id,
                              rtg_request_info *info);
/* A queued request completes at once as RTG_ERR_CANCELLED; a running one stops taking
 * new launches, its results are discarded, and it completes as RTG_ERR_CANCELLED when
 * its launches in flight finish. */
rtg_status rtg_serve_cancel(rtg_server *s, uint64_t request_id);
rtg_status rtg_serve_release(rtg_server *s);
/* Wait until no request is queued or running (wait_ms as for rtg_serve_poll). */
rtg_status rtg_serve_drain(rtg_server *s, int32_t wait_ms);
rtg_status rtg_serve_stats_get(rtg_server *s, rtg_serve_stats *st);

/* --------------------------------------------------------- dataset files */
/* Reference .s_data/.m_data header (set_intersection/utils/util.cpp:3-23 and
 * data_generator/data.cpp:344-373). */
typedef struct rtg_dataset_info {
    uint32_t num_a;
    uint32_t num_b;
    uint32_t max_element;
    uint32_t intersection;
    uint64_t elems;
} rtg_dataset_info;
/* Two calls: with offsets/elems NULL it fills only `info`; then with arrays of
 * num_a+num_b+1 and info.elems entries. */
rtg_status rtg_dataset_read(const char *path, rtg_dataset_info *info, uint32_t *offsets,
                            uint32_t *elems);
rtg_status rtg_dataset_write(const char *path, const rtg_dataset_info *info,
                             const uint32_t *offsets, const uint32_t *elems);
/* Binary int32 edge list (the reference's .edge files). */
rtg_status rtg_edges_write_bin(const char *path, const uint32_t *src, const uint32_t *dst,
                               uint64_t m);
/* Reads an edge file into host arrays; two calls as for rtg_dataset_read. */
rtg_status rtg_edges_read(const char *path, rtg_format fmt, uint64_t *m, uint32_t *src,
                          uint32_t *dst);

/* ------------------------------------------------------ seeded generators */
/* R-MAT: ef << scale edges, quadrant probabilities (a, b, c, 1-a-b-c). */
rtg_status rtg_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c,
                        uint64_t seed, uint32_t *src, uint32_t *dst);
/* Barabasi-Albert: m*(n-m) + m edges (star seed on m+1 vertices). */
rtg_status rtg_gen_ba(uint32_t n, uint32_t m, uint64_t seed, uint32_t *src, uint32_t *dst,
                      uint64_t *m_out);
/* Holme-Kim power-law cluster graph: m*(n-m) edges, triad closure probability p. */
rtg_status rtg_gen_hk(uint32_t n, uint32_t m, double p, uint64_t seed, uint32_t *src,
                      uint32_t *dst, uint64_t *m_out);
/* Batched-SI pair workload. Phase 1 (elems == NULL): draws the list lengths into
 * len (2*npairs entries) and the total into *total. Phase 2: fills offsets (2*npairs+1),
 * elems (total) and expected[npairs] (the exact |A_i ∩ B_i| by construction). Pair i
 * uses sets 2i and 2i+1. */
rtg_status rtg_gen_si_pairs(uint64_t npairs, double median, double sigma, uint32_t min_len,
                            uint32_t max_len, uint32_t universe_log2, double overlap_max,
                            uint64_t seed, uint32_t *len, uint64_t *total, uint64_t *offsets,
                            uint32_t *elems, uint32_t *expected);

#ifdef __cplusplus
}
#endif
#endif /* RTG_H */
