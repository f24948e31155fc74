// Internal declarations shared by the librtg translation units.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <cstdio>
#include <set>
#include <string>
#include <vector>

#include "host_guard.h"
#include "rtg.h"

namespace rtg {

// Sentinel used for empty hash slots and padding; vertex ids and set elements must be
// smaller (checked on input).
constexpr uint32_t kEmpty = 0xFFFFFFFFu;

// Device status word values written by kernels (never a trap).
constexpr uint32_t kStatusOk = 0;
constexpr uint32_t kStatusTimeout = 1;
constexpr uint32_t kStatusBadInput = 2;
constexpr uint32_t kStatusBadForm = 3;  // a CSR or counting form failed a device-side check

// The checked build (compiled with -DRTG_CHECKED into librtg_checked.so): every CSR and
// counting form is validated on the device before a count reads it, and the hot kernels
// check the indexes they derive from it; a violation writes the status word (the call
// returns RTG_ERR_FORMAT or RTG_ERR_INVALID_ARG) instead of reaching memory it must not.
#ifdef RTG_CHECKED
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif

struct DeviceBuffer {
    void *ptr = nullptr;
    size_t bytes = 0;
};

// One oriented or symmetric CSR resident in HBM.
// Bytes of tail padding after every adjacency array: the bulk-copy stager widens a list's
// byte range to 16-byte boundaries and may read up to 12 bytes past the last element.
constexpr size_t kAdjPadBytes = 64;

struct Csr {
    uint64_t *off = nullptr;  // n+1
    uint32_t *adj = nullptr;  // m (+ kAdjPadBytes)
    uint32_t *src = nullptr;  // m, source vertex of each entry (oriented CSR only)
    uint32_t n = 0;
    uint64_t m = 0;
    uint32_t max_deg = 0;
    uint64_t work_elems = 0;  // sum over entries (u,v) of deg(u)+deg(v)
    bool built = false;
};

// The counting form of an oriented graph: vertices relabelled by rank in (degree, id)
// order and every edge oriented from the lower rank to the higher one, rows ascending.
// For an in-edge u->v at position e of N+(u), only the suffix N+(u)[after v] can meet
// N+(v) (both hold ranks above v), so the in-edge is stored as that element range.
struct CountCsr {
    uint64_t *off = nullptr;     // n+1
    uint32_t *adj = nullptr;     // m (+ kAdjPadBytes), rank ids
    uint64_t *in_off = nullptr;  // n+1, in-edges grouped by head v
    uint2 *in_rng = nullptr;     // m: [x, y) = element range of N+(u) after v, per in-edge
    uint32_t n = 0;
    uint64_t m = 0;
    uint32_t max_deg = 0;
    int64_t core_auto = -1;  // the library's dense-core size for this form (-1: not known)
    // in-edges held: all m (kAllInEdges), or, in a one-shot count's form, only those of the
    // rows below its dense core (the core count never reads the others)
    uint64_t m_in = kAllInEdges;
    bool built = false;
    static constexpr uint64_t kAllInEdges = ~0ull;
    uint64_t inedges() const { return m_in == kAllInEdges ? m : m_in; }
};

struct TcPlan;   // cached per-graph counting plans (tc.cu)

}  // namespace rtg

struct rtg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    rtg_config cfg{};
    uint64_t launches = 0;
    // the batched SI launch (queue-head reset + persistent kernel) as a CUDA graph per kernel
    // form, captured on the first launch; later launches update the kernel node's
    // parameters and replay it
    struct KernelGraph {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        cudaGraphNode_t knode = nullptr;
    } si_graphs[2];
    // test hook (rtg_debug_si_wait_limit): applied to the next batched SI launch, then reset
    uint32_t dbg_wait_polls = 0, dbg_extra_tx = 0;
    int sm_count = 0;
    int smem_optin = 0;
    int cc_major = 0, cc_minor = 0;
    void *flush_buf = nullptr;
    size_t flush_bytes = 0;
    uint32_t *d_status = nullptr;        // device status word (kernels write errors here)
    unsigned long long *d_scalars = nullptr;  // small device scratch for counters (16 words)
    cudaEvent_t ev[8] = {};
    // page-locked staging for device-to-host copies into pageable caller memory (two
    // buffers, allocated on the first such copy) and the events that mark their copies
    void *h_stage = nullptr;
    cudaEvent_t stage_ev[2] = {};
    // grow-only scratch for CUB temp storage and per-call buffers
    rtg::DeviceBuffer scratch[9];
    // grow-only temporaries of the CSR builder (kept between builds: no allocation, and
    // none of the implicit synchronisation of a free, on repeated builds)
    rtg::DeviceBuffer work[12];
    // graphs and set collections created on this context (released by rtg_destroy)
    std::set<rtg_graph *> graphs;
    std::set<rtg_sets *> sets;
};

struct rtg_graph {
    rtg_ctx *ctx = nullptr;
    uint32_t *d_src = nullptr;  // raw edges on the device
    uint32_t *d_dst = nullptr;
    uint64_t m_input = 0;
    bool edges_released = false;
    rtg::Csr ori;               // oriented CSR
    rtg::CountCsr cnt;          // rank-relabelled counting form of ori
    int orient = -1;
    rtg::Csr sym;               // symmetric CSR
    rtg::TcPlan *plan_batched = nullptr;
    rtg::TcPlan *plan_plain = nullptr;
    rtg::TcPlan *plan_bucketed = nullptr;
};

struct rtg_sets {
    rtg_ctx *ctx = nullptr;
    uint64_t *off = nullptr;  // nsets+1
    uint32_t *elems = nullptr;
    uint64_t nsets = 0;
    uint64_t nelems = 0;
    uint32_t max_len = 0;
    bool borrowed = false;    // views a graph CSR (not freed here)
};

namespace rtg {

// Error helpers: record the message on the context and return a status.
rtg_status fail(rtg_ctx *ctx, rtg_status s, const char *fmt, ...);
rtg_status cuda_fail(rtg_ctx *ctx, cudaError_t e, const char *what, const char *file, int line);

#define RTG_CUDA(ctx, call)                                                        \
    do {                                                                           \
        cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess) return ::rtg::cuda_fail((ctx), e_, #call, __FILE__, __LINE__); \
    } while (0)

#define RTG_TRY(expr)                       \
    do {                                    \
        rtg_status s_ = (expr);             \
        if (s_ != RTG_OK) return s_;        \
    } while (0)

rtg_status dev_alloc(rtg_ctx *ctx, void **p, size_t bytes);
void dev_free(void *p);
// Grow-only scratch slot i of the context (contents undefined).
rtg_status scratch(rtg_ctx *ctx, int slot, size_t bytes, void **p);
rtg_status check_status_word(rtg_ctx *ctx);

// CSR cache file (csr_cache.cpp): a new graph of ctx from a file written by rtg_graph_save
rtg_status graph_load_cached(rtg_ctx *ctx, const char *path, rtg_graph **out);

// CSR builder (csr.cu)
rtg_status build_csr(rtg_ctx *ctx, rtg_graph *g, rtg_orient orient);
// counting form (rank relabel + in-edge suffix ranges) of an oriented CSR
rtg_status csr_build_count(rtg_ctx *ctx, const Csr &c, CountCsr &cc);
// the same counting form straight from g's raw edges (degree order, simple graph), without
// building the oriented CSR: what a one-shot batched count needs
// With in_scratch the counting form's arrays live in a context scratch slot (reused by the
// next such build); the caller must detach them (null the pointers) before the graph dies.
// With raw_degree vertices are ranked by their degree in the input list (duplicates and
// self loops counted; on long lists a 1-in-kDegreeSample sample of it), which saves the
// sort that removes duplicates before ranking: a different orientation of the same simple
// graph, so the same triangle total.
// pre (raw_degree only): the largest vertex id, and with deg_valid the (sampled) raw
// degrees of ids 0..maxid already counted into scratch slot kDegreeSlot, as the pass that
// copies pinned host edges in computes them (edge_pull in api.cu).
struct EdgePrePass {
    uint32_t maxid = 0;
    bool deg_valid = false;
};
constexpr int kDegreeSlot = 8;               // scratch slot of the raw-degree counters
constexpr uint64_t kDegreeSampleFrom = 1ull << 22;
constexpr uint32_t kDegreeSample = 8;
rtg_status build_count_direct(rtg_ctx *ctx, rtg_graph *g, bool in_scratch = false,
                              bool raw_degree = false, const EdgePrePass *pre = nullptr);
rtg_status graph_free_csr(Csr &c);
void count_csr_free(CountCsr &cc);

// Device-side validation (check.cu): offsets non-decreasing from 0 to m, ids below n, rows
// strictly ascending (and, for an oriented CSR, above their vertex); for a counting form
// also its in-edge offsets and every suffix range inside one row, above its head. A
// violation returns RTG_ERR_FORMAT. Every read index is a loop counter or a value checked
// against its array's size first, so a forged form is refused without a fault.
rtg_status check_csr(rtg_ctx *ctx, const Csr &c, bool above_vertex);
rtg_status check_count_form(rtg_ctx *ctx, const CountCsr &cc);
// test hook of the checked build: rtg_graph_load(RTG_FMT_RTG_CSR) skips the host-side
// structure checks of a cache file (sizes and checksum are still checked)
extern bool g_skip_file_structure_checks;

// Triangle counting (tc.cu)
rtg_status tc_count(rtg_ctx *ctx, rtg_graph *g, rtg_tc_mode mode, uint64_t *total,
                    rtg_timing *t);
void tc_plan_free(TcPlan *p);
// Serving: enqueue the batched count of g (building its plan on first use) on ctx's
// stream without waiting; the total lands in the pinned host word *h_total when the
// stream reaches it. At most one such count of a graph may be in flight.
rtg_status tc_launch_async(rtg_ctx *ctx, rtg_graph *g, unsigned long long *h_total);
// Device bytes the batched plan of g will hold (upper estimate; also the scratch that
// tc_launch_direct needs).
uint64_t tc_plan_estimate_bytes(const rtg_ctx *ctx, const rtg_graph *g);
// the library's dense-core size of a counting form (its offsets complete on the stream)
// into *out, a device word (tc.cu)
void enqueue_core_auto(cudaStream_t st, const CountCsr &cc, unsigned long long *out);
// the same choice from host offsets (forms read from a cache file) (tc.cu)
uint32_t core_auto_host(const uint64_t *off, uint32_t n, uint64_t m);
// the dense-core size a schedule setting (rtg_config.tc_core_ranks) gives a counting form and
// the first adj index of its core rows, into out[0] and out[1] (tc.cu)
void enqueue_core_choice(cudaStream_t st, const CountCsr &cc, uint32_t setting,
                         unsigned long long *out);
// The same count without a plan: the kernels are launched directly on ctx's stream with
// their buffers carved from the caller's device scratch, which must stay untouched until
// the count has completed.
rtg_status tc_launch_direct(rtg_ctx *ctx, rtg_graph *g, void *scratch, uint64_t scratch_bytes,
                            unsigned long long *h_total);
// Free the batched plan of g (no count of g may be in flight).
void tc_plan_release(rtg_graph *g);

// One set collection resident on the device (a symmetric CSR or an rtg_sets).
struct SetRef {
    const uint64_t *off;
    const uint32_t *elems;
    uint64_t nsets;
};

// Set intersection (si.cu). Sets are any CSR-like (off, elems); pairs may be implicit
// dense A x B (dense_nb > 0: pair k = (a_begin + k / dense_nb, b_begin + k % dense_nb)).
// With gtab set, pair k = (pa[k], pb[k]) of collection gtab[pg[k]] (one launch serving
// pairs of many collections); off/elems/nsets are then unused.
struct PairSpec {
    const uint64_t *off = nullptr;
    const uint32_t *elems = nullptr;
    uint64_t nsets = 0;
    const uint32_t *pa = nullptr;  // device
    const uint32_t *pb = nullptr;  // device
    uint64_t npairs = 0;
    uint32_t dense_nb = 0;
    uint32_t a_begin = 0, b_begin = 0;
    const uint32_t *pg = nullptr;    // device, with gtab
    const SetRef *gtab = nullptr;    // device table of ngraphs collections
    uint32_t ngraphs = 0;
};
rtg_status si_count_device(rtg_ctx *ctx, const PairSpec &ps, uint32_t *d_out, uint32_t family,
                           float *kernel_ms, uint64_t *launches);
rtg_status si_materialize_device(rtg_ctx *ctx, const PairSpec &ps, uint64_t *d_out_off,
                                 uint32_t *d_out_elems, uint64_t capacity, uint64_t *needed,
                                 uint64_t *launches);

double now_ms();

// NVTX range around a library stage: named ranges in Nsight Systems timelines and for
// Nsight Compute's --nvtx filters, next to nothing when no tool is attached (NVTX v3 is
// header-only).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

}  // namespace rtg
