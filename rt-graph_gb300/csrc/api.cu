// librtg C ABI: context, errors, memory, graphs, set collections and the call wrappers
// that time each stage. Kernels live in csr.cu, tc.cu and si.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstring>

#include "internal.h"

namespace rtg {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

rtg_status fail(rtg_ctx *ctx, rtg_status s, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return s;
}

rtg_status cuda_fail(rtg_ctx *ctx, cudaError_t e, const char *what, const char *file, int line) {
    rtg_status s = (e == cudaErrorMemoryAllocation) ? RTG_ERR_OOM : RTG_ERR_DEVICE;
    cudaGetLastError();  // clear a non-sticky error so the context stays usable
    return fail(ctx, s, "CUDA error %d (%s) in %s at %s:%d", (int)e, cudaGetErrorString(e),
                what, file, line);
}

rtg_status dev_alloc(rtg_ctx *ctx, void **p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(ctx, e, "cudaMalloc", __FILE__, __LINE__);
    }
    return RTG_OK;
}

void dev_free(void *p) {
    if (p) cudaFree(p);
}

rtg_status scratch(rtg_ctx *ctx, int slot, size_t bytes, void **p) {
    DeviceBuffer &b = ctx->scratch[slot];
    if (b.bytes < bytes) {
        dev_free(b.ptr);
        b.ptr = nullptr;
        b.bytes = 0;
        size_t want = std::max(bytes, (size_t)4096);
        RTG_TRY(dev_alloc(ctx, &b.ptr, want));
        b.bytes = want;
    }
    *p = b.ptr;
    return RTG_OK;
}

rtg_status check_status_word(rtg_ctx *ctx) {
    uint32_t st = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&st, ctx->d_status, sizeof st, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (st == kStatusOk) return RTG_OK;
    RTG_CUDA(ctx, cudaMemsetAsync(ctx->d_status, 0, sizeof(uint32_t), ctx->stream));
    if (st == kStatusTimeout)
        return fail(ctx, RTG_ERR_TIMEOUT, "a bounded device wait ran out (status word %u)", st);
    if (st == kStatusBadForm)
        return fail(ctx, RTG_ERR_FORMAT, "device-side CSR check failed (status word %u)", st);
    return fail(ctx, RTG_ERR_INVALID_ARG, "device-side input check failed (status word %u)", st);
}

rtg_status graph_free_csr(Csr &c) {
    dev_free(c.off);
    dev_free(c.adj);
    dev_free(c.src);
    c = Csr{};
    return RTG_OK;
}

void count_csr_free(CountCsr &cc) {
    dev_free(cc.off);
    dev_free(cc.adj);
    dev_free(cc.in_off);
    dev_free(cc.in_rng);
    cc = CountCsr{};
}

}  // namespace rtg

using namespace rtg;

extern "C" {

int rtg_abi_version(void) { return RTG_ABI_VERSION; }

const char *rtg_status_str(rtg_status s) {
    switch (s) {
    case RTG_OK: return "ok";
    case RTG_ERR_INVALID_ARG: return "invalid argument";
    case RTG_ERR_OOM: return "out of memory";
    case RTG_ERR_IO: return "i/o error";
    case RTG_ERR_FORMAT: return "malformed input";
    case RTG_ERR_DEVICE: return "device error";
    case RTG_ERR_TIMEOUT: return "device wait timed out";
    case RTG_ERR_CANCELLED: return "cancelled";
    case RTG_ERR_STATE: return "call out of order";
    case RTG_ERR_BUSY: return "busy";
    }
    return "unknown status";
}

const char *rtg_last_error(const rtg_ctx *ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

rtg_status rtg_init(int device, rtg_ctx **out) {
    if (!out) return RTG_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return RTG_ERR_DEVICE;
    }
    if (device < 0 || device >= ndev) return RTG_ERR_INVALID_ARG;
    rtg_ctx *ctx = new rtg_ctx();
    ctx->device = device;
    auto bail = [&](cudaError_t err) {
        cudaGetLastError();
        delete ctx;
        return err == cudaErrorMemoryAllocation ? RTG_ERR_OOM : RTG_ERR_DEVICE;
    };
    if ((e = cudaSetDevice(device)) != cudaSuccess) return bail(e);
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess)
        return bail(e);
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, device)) != cudaSuccess) return bail(e);
    ctx->sm_count = prop.multiProcessorCount;
    ctx->smem_optin = (int)prop.sharedMemPerBlockOptin;
    ctx->cc_major = prop.major;
    ctx->cc_minor = prop.minor;
    if ((e = cudaMalloc((void **)&ctx->d_status, 256)) != cudaSuccess) return bail(e);
    if ((e = cudaMemset(ctx->d_status, 0, 256)) != cudaSuccess) return bail(e);
    if ((e = cudaMalloc((void **)&ctx->d_scalars, 16 * sizeof(unsigned long long))) !=
        cudaSuccess)
        return bail(e);
    for (auto &ev : ctx->ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return bail(e);
    *out = ctx;
    return RTG_OK;
}

void rtg_destroy(rtg_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    // release what the caller did not: graphs and set collections die with their context
    while (!ctx->graphs.empty()) rtg_graph_destroy(*ctx->graphs.begin());
    while (!ctx->sets.empty()) rtg_sets_destroy(*ctx->sets.begin());
    for (auto &b : ctx->scratch) dev_free(b.ptr);
    for (auto &b : ctx->work) dev_free(b.ptr);
    dev_free(ctx->flush_buf);
    for (auto &kg : ctx->si_graphs) {
        if (kg.exec) cudaGraphExecDestroy(kg.exec);
        if (kg.graph) cudaGraphDestroy(kg.graph);
    }
    dev_free(ctx->d_status);
    dev_free(ctx->d_scalars);
    for (auto &ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    for (auto &ev : ctx->stage_ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

rtg_status rtg_set_config(rtg_ctx *ctx, const rtg_config *cfg) {
    if (!ctx || !cfg) return RTG_ERR_INVALID_ARG;
    if (cfg->tc_region_words && (cfg->tc_region_words & (cfg->tc_region_words - 1)))
        return fail(ctx, RTG_ERR_INVALID_ARG, "tc_region_words must be a power of two");
    if (cfg->tc_region_words && (cfg->tc_region_words < 64 || cfg->tc_region_words > 16384))
        return fail(ctx, RTG_ERR_INVALID_ARG, "tc_region_words must be in [64, 16384]");
    if (cfg->tc_block_warps > 32 || cfg->si_block_warps > 32)
        return fail(ctx, RTG_ERR_INVALID_ARG, "at most 32 warps per block");
    if (cfg->si_stage_slots && (cfg->si_stage_slots < 2 || cfg->si_stage_slots > 32))
        return fail(ctx, RTG_ERR_INVALID_ARG, "si_stage_slots must be in [2, 32]");
    if (cfg->si_stage_bytes && (cfg->si_stage_bytes < 512 || cfg->si_stage_bytes % 128 ||
                                cfg->si_stage_bytes > 32768))
        return fail(ctx, RTG_ERR_INVALID_ARG,
                    "si_stage_bytes must be a multiple of 128 in [512, 32768]");
    if (cfg->si_skew_stream > 1)
        return fail(ctx, RTG_ERR_INVALID_ARG, "si_skew_stream must be 0 or 1");
    if (cfg->si_form > 2)
        return fail(ctx, RTG_ERR_INVALID_ARG, "si_form must be 0, 1 or 2");
    if (cfg->tc_core_ranks > RTG_TC_CORE_MAX_RANKS && cfg->tc_core_ranks != RTG_TC_CORE_NONE)
        return fail(ctx, RTG_ERR_INVALID_ARG,
                    "tc_core_ranks must be 0, RTG_TC_CORE_NONE or in [1, 32768]");
    ctx->cfg = *cfg;
    return RTG_OK;
}

rtg_status rtg_get_config(const rtg_ctx *ctx, rtg_config *cfg) {
    if (!ctx || !cfg) return RTG_ERR_INVALID_ARG;
    *cfg = ctx->cfg;
    return RTG_OK;
}

uint64_t rtg_kernel_launches(const rtg_ctx *ctx) { return ctx ? ctx->launches : 0; }

rtg_status rtg_synchronize(rtg_ctx *ctx) {
    if (!ctx) return RTG_ERR_INVALID_ARG;
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RTG_OK;
}

rtg_status rtg_flush_l2(rtg_ctx *ctx) {
    if (!ctx) return RTG_ERR_INVALID_ARG;
    if (!ctx->flush_buf) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device);
        size_t bytes = std::max((size_t)l2 * 2, (size_t)256 << 20);
        RTG_TRY(dev_alloc(ctx, &ctx->flush_buf, bytes));
        ctx->flush_bytes = bytes;
    }
    static int flip = 0;
    flip ^= 1;
    RTG_CUDA(ctx, cudaMemsetAsync(ctx->flush_buf, flip, ctx->flush_bytes, ctx->stream));
    return RTG_OK;
}

rtg_status rtg_device_info(const rtg_ctx *ctx, int *sm_count, int *smem_optin, int *cc_major,
                           int *cc_minor) {
    if (!ctx) return RTG_ERR_INVALID_ARG;
    if (sm_count) *sm_count = ctx->sm_count;
    if (smem_optin) *smem_optin = ctx->smem_optin;
    if (cc_major) *cc_major = ctx->cc_major;
    if (cc_minor) *cc_minor = ctx->cc_minor;
    return RTG_OK;
}

rtg_status rtg_host_alloc(rtg_ctx *ctx, size_t bytes, void **out) {
    if (!ctx || !out) return RTG_ERR_INVALID_ARG;
    RTG_CUDA(ctx, cudaHostAlloc(out, bytes ? bytes : 16, cudaHostAllocDefault));
    return RTG_OK;
}

void rtg_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

/* ------------------------------------------------------------------ graphs */

static rtg_graph *new_graph(rtg_ctx *ctx) {
    rtg_graph *g = new rtg_graph();
    g->ctx = ctx;
    ctx->graphs.insert(g);
    return g;
}

static rtg_status new_graph_device_edges(rtg_ctx *ctx, uint64_t m, rtg_graph **out) {
    rtg_graph *g = new_graph(ctx);
    g->m_input = m;
    rtg_status s = dev_alloc(ctx, (void **)&g->d_src, m * sizeof(uint32_t));
    if (s == RTG_OK) s = dev_alloc(ctx, (void **)&g->d_dst, m * sizeof(uint32_t));
    if (s != RTG_OK) {
        rtg_graph_destroy(g);
        return s;
    }
    *out = g;
    return RTG_OK;
}

rtg_status rtg_graph_from_host_edges(rtg_ctx *ctx, const uint32_t *src, const uint32_t *dst,
                                     uint64_t m, rtg_graph **out) {
    if (!ctx || !out || (m && (!src || !dst))) return RTG_ERR_INVALID_ARG;
    *out = nullptr;
    rtg_graph *g = nullptr;
    RTG_TRY(new_graph_device_edges(ctx, m, &g));
    cudaError_t e = cudaSuccess;
    if (m) {
        e = cudaMemcpyAsync(g->d_src, src, m * 4, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(g->d_dst, dst, m * 4, cudaMemcpyHostToDevice, ctx->stream);
    }
    if (e != cudaSuccess) {
        rtg_graph_destroy(g);
        return cuda_fail(ctx, e, "edge upload", __FILE__, __LINE__);
    }
    *out = g;
    return RTG_OK;
}

rtg_status rtg_graph_from_device_edges(rtg_ctx *ctx, const uint32_t *d_src,
                                       const uint32_t *d_dst, uint64_t m, rtg_graph **out) {
    if (!ctx || !out || (m && (!d_src || !d_dst))) return RTG_ERR_INVALID_ARG;
    *out = nullptr;
    rtg_graph *g = nullptr;
    RTG_TRY(new_graph_device_edges(ctx, m, &g));
    cudaError_t e = cudaSuccess;
    if (m) {
        e = cudaMemcpyAsync(g->d_src, d_src, m * 4, cudaMemcpyDeviceToDevice, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(g->d_dst, d_dst, m * 4, cudaMemcpyDeviceToDevice, ctx->stream);
    }
    if (e != cudaSuccess) {
        rtg_graph_destroy(g);
        return cuda_fail(ctx, e, "edge copy", __FILE__, __LINE__);
    }
    *out = g;
    return RTG_OK;
}

rtg_status rtg_graph_from_host_pairs(rtg_ctx *ctx, const int32_t *pairs, uint64_t m,
                                     rtg_graph **out) {
    if (!ctx || !out || (m && !pairs)) return RTG_ERR_INVALID_ARG;
    std::vector<uint32_t> s(m), d(m);
    for (uint64_t i = 0; i < m; ++i) {
        if (pairs[2 * i] < 0 || pairs[2 * i + 1] < 0)
            return fail(ctx, RTG_ERR_INVALID_ARG, "negative vertex id at edge %llu",
                        (unsigned long long)i);
        s[i] = (uint32_t)pairs[2 * i];
        d[i] = (uint32_t)pairs[2 * i + 1];
    }
    rtg_status st = rtg_graph_from_host_edges(ctx, s.data(), d.data(), m, out);
    if (st == RTG_OK) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);  // host vectors die here
        if (e != cudaSuccess) return cuda_fail(ctx, e, "sync", __FILE__, __LINE__);
    }
    return st;
}

rtg_status rtg_csr_build(rtg_ctx *ctx, rtg_graph *g, rtg_orient orient) {
    NvtxRange nvtx_("rtg_csr_build");
    if (!ctx || !g) return RTG_ERR_INVALID_ARG;
    if (orient != RTG_ORIENT_DEGREE && orient != RTG_ORIENT_DEGREE_RAW_REF &&
        orient != RTG_ORIENT_SYMMETRIC)
        return fail(ctx, RTG_ERR_INVALID_ARG, "unknown orientation %d", (int)orient);
    if (g->edges_released)
        return fail(ctx, RTG_ERR_STATE, "raw edges were released; cannot build a CSR");
    if (orient != RTG_ORIENT_SYMMETRIC) {
        // cached counting plans point into the CSR about to be replaced
        cudaStreamSynchronize(ctx->stream);
        tc_plan_free(g->plan_batched);
        tc_plan_free(g->plan_plain);
        tc_plan_free(g->plan_bucketed);
        g->plan_batched = g->plan_plain = g->plan_bucketed = nullptr;
        count_csr_free(g->cnt);
    }
    RTG_TRY(build_csr(ctx, g, orient));
    if (orient != RTG_ORIENT_SYMMETRIC) RTG_TRY(csr_build_count(ctx, g->ori, g->cnt));
    return RTG_OK;
}

rtg_status rtg_graph_info_get(const rtg_graph *g, rtg_graph_info *info) {
    if (!g || !info) return RTG_ERR_INVALID_ARG;
    memset(info, 0, sizeof *info);
    info->n = g->ori.n;
    info->m_input = g->m_input;
    info->m = g->ori.m;
    info->max_out_degree = g->ori.max_deg;
    info->work_elems = g->ori.work_elems;
    info->orient = g->ori.built ? g->orient : -1;
    info->has_symmetric = g->sym.built ? 1 : 0;
    info->n_sym = g->sym.n;
    info->m_sym = g->sym.m;
    return RTG_OK;
}

rtg_status rtg_csr_view(const rtg_graph *g, int symmetric, const uint64_t **d_offsets,
                        const uint32_t **d_adj, uint32_t *n, uint64_t *m) {
    if (!g) return RTG_ERR_INVALID_ARG;
    const Csr &c = symmetric ? g->sym : g->ori;
    if (!c.built) return RTG_ERR_STATE;
    if (d_offsets) *d_offsets = c.off;
    if (d_adj) *d_adj = c.adj;
    if (n) *n = c.n;
    if (m) *m = c.m;
    return RTG_OK;
}

rtg_status rtg_csr_to_host(rtg_ctx *ctx, const rtg_graph *g, int symmetric, uint64_t *offsets,
                           uint32_t *adj) {
    if (!ctx || !g || !offsets || !adj) return RTG_ERR_INVALID_ARG;
    const Csr &c = symmetric ? g->sym : g->ori;
    if (!c.built) return fail(ctx, RTG_ERR_STATE, "CSR not built");
    RTG_CUDA(ctx, cudaMemcpyAsync(offsets, c.off, (c.n + 1) * sizeof(uint64_t),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    if (c.m)
        RTG_CUDA(ctx, cudaMemcpyAsync(adj, c.adj, c.m * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                      ctx->stream));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return RTG_OK;
}

rtg_status rtg_graph_release_edges(rtg_graph *g) {
    if (!g) return RTG_ERR_INVALID_ARG;
    if (g->ctx) cudaStreamSynchronize(g->ctx->stream);
    dev_free(g->d_src);
    dev_free(g->d_dst);
    g->d_src = g->d_dst = nullptr;
    g->edges_released = true;
    return RTG_OK;
}

uint64_t rtg_graph_device_bytes(const rtg_graph *g) {
    if (!g) return 0;
    uint64_t b = 0;
    if (!g->edges_released) b += g->m_input * 8;
    auto csr_bytes = [](const Csr &c) -> uint64_t {
        if (!c.built) return 0;
        return (uint64_t)(c.n + 1) * 8 + c.m * 4 + (c.src ? c.m * 4 : 0);
    };
    const CountCsr &cc = g->cnt;
    uint64_t cb = cc.built ? (uint64_t)(cc.n + 1) * 16 + cc.m * 12 : 0;
    return b + csr_bytes(g->ori) + csr_bytes(g->sym) + cb;
}

void rtg_graph_destroy(rtg_graph *g) {
    if (!g) return;
    if (g->ctx) {
        cudaStreamSynchronize(g->ctx->stream);
        g->ctx->graphs.erase(g);
    }
    tc_plan_free(g->plan_batched);
    tc_plan_free(g->plan_plain);
    tc_plan_free(g->plan_bucketed);
    dev_free(g->d_src);
    dev_free(g->d_dst);
    graph_free_csr(g->ori);
    graph_free_csr(g->sym);
    count_csr_free(g->cnt);
    delete g;
}

/* --------------------------------------------------------- CSR given by host */

__global__ void k_csr_from_i32(const int32_t *off32, const int32_t *adj32, uint32_t n,
                               uint64_t m, uint64_t *off, uint32_t *adj, uint32_t *src,
                               uint32_t *status) {
    uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = tid; v <= n; v += stride) {
        int32_t o = off32[v];
        off[v] = (uint64_t)(o < 0 ? 0 : o);
        if (o < 0 || (uint64_t)o > m) atomicExch(status, kStatusBadInput);
        if (v < n) {
            int32_t e = off32[v + 1];
            if (e < o) {
                atomicExch(status, kStatusBadInput);
                continue;
            }
            uint64_t hi = (uint64_t)e > m ? m : (uint64_t)e;
            for (uint64_t k = (uint64_t)o; k < hi; ++k) {
                int32_t w = adj32[k];
                if (w < 0 || (uint32_t)w >= n) atomicExch(status, kStatusBadInput);
                if (k > (uint64_t)o && adj32[k - 1] >= w) atomicExch(status, kStatusBadInput);
                adj[k] = (uint32_t)w;
                src[k] = (uint32_t)v;
            }
        }
    }
}

__global__ void k_csr_stats(const uint64_t *off, const uint32_t *adj, const uint32_t *src,
                            uint64_t m, uint32_t n, unsigned long long *work,
                            unsigned int *maxdeg) {
    uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long acc = 0;
    unsigned int md = 0;
    for (uint64_t e = tid; e < m; e += stride) {
        uint32_t u = src[e], v = adj[e];
        acc += (off[u + 1] - off[u]) + (off[v + 1] - off[v]);
    }
    for (uint64_t v = tid; v < n; v += stride) md = max(md, (unsigned int)(off[v + 1] - off[v]));
    for (int o = 16; o; o >>= 1) {
        acc += __shfl_down_sync(0xffffffffu, acc, o);
        md = max(md, __shfl_down_sync(0xffffffffu, md, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (acc) atomicAdd(work, acc);
        atomicMax(maxdeg, md);
    }
}

rtg_status rtg_graph_from_host_csr(rtg_ctx *ctx, const int32_t *offsets, const int32_t *adjs,
                                   int32_t nodes, int64_t edges, rtg_graph **out) {
    if (!ctx || !out || !offsets || nodes < 0 || edges < 0 || (edges && !adjs))
        return RTG_ERR_INVALID_ARG;
    *out = nullptr;
    if (offsets[nodes] != edges || offsets[0] != 0)
        return fail(ctx, RTG_ERR_INVALID_ARG, "offsets[0] must be 0 and offsets[nodes] == edges");
    rtg_graph *g = new_graph(ctx);
    g->m_input = (uint64_t)edges;
    g->edges_released = true;
    Csr &c = g->ori;
    c.n = (uint32_t)nodes;
    c.m = (uint64_t)edges;
    int32_t *d_off32 = nullptr, *d_adj32 = nullptr;
    rtg_status s = RTG_OK;
    auto cleanup = [&](rtg_status st) {
        dev_free(d_off32);
        dev_free(d_adj32);
        if (st != RTG_OK) rtg_graph_destroy(g);
        return st;
    };
    if ((s = dev_alloc(ctx, (void **)&c.off, (c.n + 1) * 8ull)) != RTG_OK) return cleanup(s);
    if ((s = dev_alloc(ctx, (void **)&c.adj, c.m * 4 + kAdjPadBytes)) != RTG_OK) return cleanup(s);
    if ((s = dev_alloc(ctx, (void **)&c.src, c.m * 4)) != RTG_OK) return cleanup(s);
    if ((s = dev_alloc(ctx, (void **)&d_off32, (c.n + 1) * 4ull)) != RTG_OK) return cleanup(s);
    if ((s = dev_alloc(ctx, (void **)&d_adj32, c.m * 4)) != RTG_OK) return cleanup(s);
    cudaError_t e = cudaMemcpyAsync(d_off32, offsets, (c.n + 1) * 4ull, cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e == cudaSuccess && c.m)
        e = cudaMemcpyAsync(d_adj32, adjs, c.m * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "csr upload", __FILE__, __LINE__));
    int grid = std::max(1, std::min(ctx->sm_count * 8, (int)((c.n + 256) / 256)));
    k_csr_from_i32<<<grid, 256, 0, ctx->stream>>>(d_off32, d_adj32, c.n, c.m, c.off, c.adj, c.src,
                                                  ctx->d_status);
    ctx->launches++;
    unsigned long long *d_work = ctx->d_scalars;
    e = cudaMemsetAsync(d_work, 0, 16, ctx->stream);
    if (e == cudaSuccess) {
        int grid2 = std::max(1, std::min(ctx->sm_count * 8, (int)((c.m + c.n + 255) / 256)));
        k_csr_stats<<<grid2, 256, 0, ctx->stream>>>(c.off, c.adj, c.src, c.m, c.n, d_work,
                                                    (unsigned int *)(d_work + 1));
        ctx->launches++;
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "csr checks", __FILE__, __LINE__));
    unsigned long long hw[2] = {0, 0};
    e = cudaMemcpyAsync(hw, d_work, 16, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "csr checks", __FILE__, __LINE__));
    if ((s = check_status_word(ctx)) != RTG_OK) {
        ctx->last_error = "CSR rows must be sorted ascending with ids in [0, nodes)";
        return cleanup(RTG_ERR_INVALID_ARG);
    }
    c.work_elems = hw[0];
    c.max_deg = (uint32_t)hw[1];
    c.built = true;
    if ((s = csr_build_count(ctx, c, g->cnt)) != RTG_OK) return cleanup(s);
    g->orient = RTG_ORIENT_DEGREE_RAW_REF;
    *out = g;
    return cleanup(RTG_OK);
}

/* ----------------------------------------------------- triangle counting */

rtg_status rtg_tc_count(rtg_ctx *ctx, rtg_graph *g, rtg_tc_mode mode, uint64_t *out_total,
                        rtg_timing *timing) {
    NvtxRange nvtx_("rtg_tc_count");
    if (!ctx || !g || !out_total) return RTG_ERR_INVALID_ARG;
    if (mode != RTG_TC_PLAIN && mode != RTG_TC_BATCHED && mode != RTG_TC_BUCKETED)
        return fail(ctx, RTG_ERR_INVALID_ARG, "unknown tc mode %d", (int)mode);
    // PLAIN reads the oriented CSR; the other forms the counting form, which a graph read
    // from a cache file may hold alone
    if (mode == RTG_TC_PLAIN ? !g->ori.built : !(g->ori.built || g->cnt.built))
        return fail(ctx, RTG_ERR_STATE, "oriented CSR not built");
    rtg_timing t{};
    double t0 = now_ms();
    RTG_TRY(tc_count(ctx, g, mode, out_total, &t));
    t.total_ms = now_ms() - t0;
    if (timing) *timing = t;
    return RTG_OK;
}

// Device address of a page-locked host array that the GPU can address directly (pinned
// memory is mapped into the device's address space), or nullptr for pageable memory.
static void *mapped_host(const void *p) {
    cudaPointerAttributes a{};
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // not a CUDA pointer: clear the non-sticky error
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Copies page-locked host edges into device memory, reading them over the host link in
// 16-byte loads, and on the way finds the largest id and counts the raw degrees of the
// sampled edges (edge i when i % stride == 0, the edges k_degree_raw samples) into deg,
// for ids below cap; *d_over becomes 1 when a sampled id is at or above cap. The copy is
// bound by the host link, so the two passes that would otherwise follow it are hidden.
// Quad q holds edges 4q .. 4q+3; stride is 1 or a multiple of 4.
__global__ void k_edge_pull(const uint4 *__restrict__ hs, const uint4 *__restrict__ hd,
                            const uint32_t *__restrict__ hs1, const uint32_t *__restrict__ hd1,
                            uint64_t m, uint4 *ds, uint4 *dd, uint32_t *ds1, uint32_t *dd1,
                            uint32_t *deg, uint32_t cap, uint32_t stride, unsigned *d_max,
                            unsigned *d_over) {
    unsigned mx = 0, over = 0;
    auto count = [&](uint32_t x) {
        if (x < cap) atomicAdd(&deg[x], 1u);
        else over = 1u;
    };
    const uint64_t m4 = m / 4;
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < m4;
         q += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 a = hs[q], b = hd[q];
        ds[q] = a;
        dd[q] = b;
        mx = max(mx, max(max(max(a.x, a.y), max(a.z, a.w)), max(max(b.x, b.y), max(b.z, b.w))));
        if (stride == 1) {
            count(a.x); count(a.y); count(a.z); count(a.w);
            count(b.x); count(b.y); count(b.z); count(b.w);
        } else if ((4 * q) % stride == 0) {
            count(a.x);
            count(b.x);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the last m % 4 edges
        for (uint64_t i = 4 * m4; i < m; ++i) {
            const uint32_t a = hs1[i], b = hd1[i];
            ds1[i] = a;
            dd1[i] = b;
            mx = max(mx, max(a, b));
            if (i % stride == 0) {
                count(a);
                count(b);
            }
        }
    }
    for (int o = 16; o; o >>= 1) {
        mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
        over |= __shfl_down_sync(0xffffffffu, over, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(d_max, mx);
        if (over) atomicOr(d_over, 1u);
    }
}

// The one-shot batched count of edges already in tg.d_src / tg.d_dst (context scratch; the
// host -> device stage was bracketed by ev[6] and now ends): the counting form is built
// straight from them (no oriented CSR) and counted with direct launches (no plan). Fills the
// stage times of t. tg only borrows scratch: nothing in it is freed.
static rtg_status one_shot_count(rtg_ctx *ctx, rtg_graph &tg, const EdgePrePass *pre,
                                 uint64_t h2d_bytes, uint64_t *out_total, rtg_timing &t) {
    rtg_graph *g = &tg;
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
    rtg_status s;
    {
        NvtxRange r("one-shot counting-form build");
        s = build_count_direct(ctx, g, true, true, pre);
    }
    void *scr = nullptr;
    const uint64_t need = s == RTG_OK ? tc_plan_estimate_bytes(ctx, g) : 0;
    if (s == RTG_OK) s = scratch(ctx, 6, need, &scr);
    unsigned long long h = 0;
    if (s == RTG_OK) {
        float h2d = 0;
        cudaEventElapsedTime(&h2d, ctx->ev[6], ctx->ev[7]);
        t.h2d_ms = h2d;
        t.h2d_bytes = h2d_bytes;
        t.algo_bytes = 0;
        cudaError_t e = cudaEventRecord(ctx->ev[0], ctx->stream);
        if (e != cudaSuccess) s = cuda_fail(ctx, e, "event", __FILE__, __LINE__);
    }
    if (s == RTG_OK) {
        NvtxRange r("one-shot batched count");
        s = tc_launch_direct(ctx, g, scr, need, &h);
    }
    if (s == RTG_OK) {
        cudaError_t e = cudaEventRecord(ctx->ev[1], ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) s = cuda_fail(ctx, e, "count", __FILE__, __LINE__);
    }
    if (s == RTG_OK) s = check_status_word(ctx);
    tg.d_src = tg.d_dst = nullptr;
    tg.cnt = CountCsr{};
    if (s != RTG_OK) return s;
    float ms = 0, bms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&bms, ctx->ev[7], ctx->ev[0]);  // device time of the build
    t.count_ms = t.main_kernel_ms = ms;
    t.build_ms = bms;
    *out_total = h;
    return RTG_OK;
}

rtg_status rtg_tc_count_host_edges(rtg_ctx *ctx, const uint32_t *src, const uint32_t *dst,
                                   uint64_t m, rtg_orient orient, rtg_tc_mode mode,
                                   uint64_t *out_total, rtg_timing *timing) {
    NvtxRange nvtx_("rtg_tc_count_host_edges");
    if (!ctx || !out_total || (m && (!src || !dst))) return RTG_ERR_INVALID_ARG;
    if (orient == RTG_ORIENT_SYMMETRIC)
        return fail(ctx, RTG_ERR_INVALID_ARG, "triangle counting needs an oriented CSR");
    rtg_timing t{};
    double t0 = now_ms();
    uint64_t l0 = ctx->launches;
    if (mode == RTG_TC_BATCHED && orient == RTG_ORIENT_DEGREE) {
        // one-shot batched count: the counting form is built straight from the edges (no
        // oriented CSR) and counted with direct launches (no plan); the edges, the counting
        // form and the count's buffers live in grow-only context scratch, so repeated calls
        // allocate and free nothing. The graph object is local and only borrows them.
        rtg_graph tg;
        rtg_graph *g = &tg;
        void *pe = nullptr;
        const uint64_t mpad = (m + 63) & ~63ull;
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
        RTG_TRY(scratch(ctx, 2, mpad * 8 + 256, &pe));
        tg.d_src = static_cast<uint32_t *>(pe);
        tg.d_dst = tg.d_src + mpad;
        tg.m_input = m;
        // page-locked host edges are pulled in by one kernel that also finds the largest
        // id and counts the sampled degrees (into the counters the previous one-shot build
        // sized; when they are too small the build counts again); pageable ones are copied
        EdgePrePass pre;
        bool have_pre = false;
        void *hsrc = m >= (1ull << 20) ? mapped_host(src) : nullptr;
        void *hdst = hsrc ? mapped_host(dst) : nullptr;
        if (hsrc && hdst &&
            ((reinterpret_cast<uintptr_t>(hsrc) | reinterpret_cast<uintptr_t>(hdst)) & 15) == 0) {
            DeviceBuffer &db = ctx->scratch[kDegreeSlot];
            const uint32_t cap = (uint32_t)std::min<uint64_t>(db.bytes / 4, 0xFFFFFFFFull);
            if (cap) RTG_CUDA(ctx, cudaMemsetAsync(db.ptr, 0, cap * 4ull, ctx->stream));
            unsigned *d_w = reinterpret_cast<unsigned *>(ctx->d_scalars);
            RTG_CUDA(ctx, cudaMemsetAsync(d_w, 0, 8, ctx->stream));
            const uint32_t stride = m >= kDegreeSampleFrom ? kDegreeSample : 1u;
            const int grid = (int)std::max<uint64_t>(
                1, std::min<uint64_t>((m / 4 + 255) / 256, (uint64_t)ctx->sm_count * 8));
            k_edge_pull<<<grid, 256, 0, ctx->stream>>>(
                static_cast<const uint4 *>(hsrc), static_cast<const uint4 *>(hdst),
                static_cast<const uint32_t *>(hsrc), static_cast<const uint32_t *>(hdst), m,
                reinterpret_cast<uint4 *>(tg.d_src), reinterpret_cast<uint4 *>(tg.d_dst),
                tg.d_src, tg.d_dst, static_cast<uint32_t *>(db.ptr), cap, stride, d_w, d_w + 1);
            ctx->launches++;
            RTG_CUDA(ctx, cudaGetLastError());
            unsigned hw[2] = {0, 0};
            RTG_CUDA(ctx, cudaMemcpyAsync(hw, d_w, 8, cudaMemcpyDeviceToHost, ctx->stream));
            RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            pre.maxid = hw[0];
            pre.deg_valid = hw[1] == 0 && cap > 0 && (uint64_t)hw[0] < cap;
            have_pre = true;
        } else if (m) {
            RTG_CUDA(ctx, cudaMemcpyAsync(tg.d_src, src, m * 4, cudaMemcpyHostToDevice, ctx->stream));
            RTG_CUDA(ctx, cudaMemcpyAsync(tg.d_dst, dst, m * 4, cudaMemcpyHostToDevice, ctx->stream));
        }
        RTG_TRY(one_shot_count(ctx, tg, have_pre ? &pre : nullptr, m * 8, out_total, t));
        t.d2h_bytes = 8;
        t.kernel_launches = ctx->launches - l0;
        t.total_ms = now_ms() - t0;
        if (timing) *timing = t;
        return RTG_OK;
    }
    rtg_graph *g = nullptr;
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
    RTG_TRY(rtg_graph_from_host_edges(ctx, src, dst, m, &g));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
    rtg_status s = rtg_csr_build(ctx, g, orient);
    if (s == RTG_OK) {
        float h2d = 0;
        cudaEventElapsedTime(&h2d, ctx->ev[6], ctx->ev[7]);
        t.h2d_ms = h2d;
        t.h2d_bytes = m * 8;
        double tb = now_ms();
        t.build_ms = tb - t0 - t.h2d_ms;
        rtg_graph_release_edges(g);
        s = tc_count(ctx, g, mode, out_total, &t);
    }
    rtg_graph_destroy(g);
    if (s != RTG_OK) return s;
    t.d2h_bytes = 8;
    t.kernel_launches = ctx->launches - l0;
    t.total_ms = now_ms() - t0;
    if (timing) *timing = t;
    return RTG_OK;
}

rtg_status rtg_tc_count_host_csr(rtg_ctx *ctx, const int32_t *offsets, const int32_t *adjs,
                                 int32_t nodes, int64_t edges, rtg_tc_mode mode,
                                 uint64_t *out_total, rtg_timing *timing) {
    NvtxRange nvtx_("rtg_tc_count_host_csr");
    if (!ctx || !out_total) return RTG_ERR_INVALID_ARG;
    rtg_timing t{};
    double t0 = now_ms();
    uint64_t l0 = ctx->launches;
    if (mode == RTG_TC_BATCHED) {
        // one-shot: the CSR's edges are counted like a host edge list (the counting form built
        // straight from them, direct launches), after the same validation as a graph handle's
        if (!offsets || nodes < 0 || edges < 0 || (edges && !adjs)) return RTG_ERR_INVALID_ARG;
        if (offsets[nodes] != edges || offsets[0] != 0)
            return fail(ctx, RTG_ERR_INVALID_ARG,
                        "offsets[0] must be 0 and offsets[nodes] == edges");
        const uint64_t n = (uint64_t)nodes, m = (uint64_t)edges;
        const uint64_t mpad = (m + 63) & ~63ull, npad = (n + 1 + 63) & ~63ull;
        rtg_graph tg;
        void *pe = nullptr, *pc = nullptr;
        RTG_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
        RTG_TRY(scratch(ctx, 2, mpad * 8 + 256, &pe));
        tg.d_src = static_cast<uint32_t *>(pe);
        tg.d_dst = tg.d_src + mpad;
        tg.m_input = m;
        // int32 offsets and ids in, u64 offsets as the validation kernel's by-product
        RTG_TRY(scratch(ctx, 1, npad * 16 + mpad * 4 + 256, &pc));
        int32_t *d_off32 = static_cast<int32_t *>(pc), *d_adj32 = d_off32 + npad;
        uint64_t *d_off64 = reinterpret_cast<uint64_t *>(d_adj32 + mpad);
        RTG_CUDA(ctx, cudaMemcpyAsync(d_off32, offsets, (n + 1) * 4, cudaMemcpyHostToDevice,
                                      ctx->stream));
        if (m)
            RTG_CUDA(ctx, cudaMemcpyAsync(d_adj32, adjs, m * 4, cudaMemcpyHostToDevice,
                                          ctx->stream));
        const int grid = std::max(1, std::min(ctx->sm_count * 8, (int)((n + 256) / 256)));
        k_csr_from_i32<<<grid, 256, 0, ctx->stream>>>(d_off32, d_adj32, (uint32_t)n, m, d_off64,
                                                      tg.d_dst, tg.d_src, ctx->d_status);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        if (check_status_word(ctx) != RTG_OK) {  // synchronises
            tg.d_src = tg.d_dst = nullptr;
            return fail(ctx, RTG_ERR_INVALID_ARG,
                        "CSR rows must be sorted ascending with ids in [0, nodes)");
        }
        RTG_TRY(one_shot_count(ctx, tg, nullptr, (n + 1) * 4 + m * 4, out_total, t));
        t.d2h_bytes = 8;
        t.kernel_launches = ctx->launches - l0;
        t.total_ms = now_ms() - t0;
        if (timing) *timing = t;
        return RTG_OK;
    }
    rtg_graph *g = nullptr;
    RTG_TRY(rtg_graph_from_host_csr(ctx, offsets, adjs, nodes, edges, &g));
    t.h2d_ms = now_ms() - t0;
    t.h2d_bytes = (uint64_t)(nodes + 1) * 4 + (uint64_t)edges * 4;
    rtg_status s = tc_count(ctx, g, mode, out_total, &t);
    rtg_graph_destroy(g);
    if (s != RTG_OK) return s;
    t.d2h_bytes = 8;
    t.kernel_launches = ctx->launches - l0;
    t.total_ms = now_ms() - t0;
    if (timing) *timing = t;
    return RTG_OK;
}

/* ------------------------------------------------------ set collections */

__global__ void k_check_sets(const uint64_t *off, const uint32_t *elems, uint64_t nsets,
                             uint64_t nelems, uint32_t *status, unsigned int *maxlen) {
    uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned int ml = 0;
    for (uint64_t s = tid; s < nsets; s += stride) {
        uint64_t b = off[s], e = off[s + 1];
        if (e < b || e > nelems) {
            atomicExch(status, kStatusBadInput);
            continue;
        }
        ml = max(ml, (unsigned int)min(e - b, (uint64_t)0xFFFFFFFFu));
    }
    for (uint64_t i = tid; i < nelems; i += stride) {
        if (elems[i] == kEmpty) atomicExch(status, kStatusBadInput);
    }
    for (int o = 16; o; o >>= 1) ml = max(ml, __shfl_down_sync(0xffffffffu, ml, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxlen, ml);
}

static rtg_status sets_finish(rtg_ctx *ctx, rtg_sets *s) {
    unsigned int *d_ml = (unsigned int *)ctx->d_scalars;
    RTG_CUDA(ctx, cudaMemsetAsync(d_ml, 0, 4, ctx->stream));
    int grid = std::max<int>(1, (int)std::min<uint64_t>(ctx->sm_count * 8ull,
                                                       (s->nelems + s->nsets + 255) / 256));
    k_check_sets<<<grid, 256, 0, ctx->stream>>>(s->off, s->elems, s->nsets, s->nelems,
                                                ctx->d_status, d_ml);
    ctx->launches++;
    RTG_CUDA(ctx, cudaGetLastError());
    unsigned int ml = 0;
    RTG_CUDA(ctx, cudaMemcpyAsync(&ml, d_ml, 4, cudaMemcpyDeviceToHost, ctx->stream));
    RTG_TRY(check_status_word(ctx));
    s->max_len = ml;
    return RTG_OK;
}

rtg_status rtg_sets_from_host(rtg_ctx *ctx, const uint64_t *offsets, uint64_t nsets,
                              const uint32_t *elems, rtg_sets **out) {
    NvtxRange nvtx_("rtg_sets_from_host");
    if (!ctx || !out || !offsets) return RTG_ERR_INVALID_ARG;
    *out = nullptr;
    uint64_t ne = offsets[nsets];
    if (offsets[0] != 0) return fail(ctx, RTG_ERR_INVALID_ARG, "offsets[0] must be 0");
    if (ne && !elems) return RTG_ERR_INVALID_ARG;
    rtg_sets *s = new rtg_sets();
    s->ctx = ctx;
    ctx->sets.insert(s);
    s->nsets = nsets;
    s->nelems = ne;
    rtg_status st = dev_alloc(ctx, (void **)&s->off, (nsets + 1) * 8);
    // tail padding: staged copies widen a list's byte range to 16-byte boundaries
    if (st == RTG_OK) st = dev_alloc(ctx, (void **)&s->elems, ne * 4 + kAdjPadBytes);
    if (st == RTG_OK) {
        cudaError_t pe = cudaMemsetAsync((char *)s->elems + ne * 4, 0, kAdjPadBytes, ctx->stream);
        if (pe != cudaSuccess) st = cuda_fail(ctx, pe, "pad", __FILE__, __LINE__);
    }
    cudaError_t e = cudaSuccess;
    if (st == RTG_OK) {
        e = cudaMemcpyAsync(s->off, offsets, (nsets + 1) * 8, cudaMemcpyHostToDevice, ctx->stream);
        if (e == cudaSuccess && ne)
            e = cudaMemcpyAsync(s->elems, elems, ne * 4, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) st = cuda_fail(ctx, e, "set upload", __FILE__, __LINE__);
    }
    if (st == RTG_OK) st = sets_finish(ctx, s);
    if (st != RTG_OK) {
        rtg_sets_destroy(s);
        return st;
    }
    *out = s;
    return RTG_OK;
}

rtg_status rtg_sets_from_host_u32(rtg_ctx *ctx, const uint32_t *offsets, uint32_t nsets,
                                  const uint32_t *elems, rtg_sets **out) {
    if (!ctx || !out || !offsets) return RTG_ERR_INVALID_ARG;
    std::vector<uint64_t> off64(nsets + 1ull);
    for (uint64_t i = 0; i <= nsets; ++i) off64[i] = offsets[i];
    for (uint64_t i = 0; i < nsets; ++i)
        if (off64[i + 1] < off64[i])
            return fail(ctx, RTG_ERR_INVALID_ARG, "set offsets must be non-decreasing");
    rtg_status st = rtg_sets_from_host(ctx, off64.data(), nsets, elems, out);
    return st;
}

uint64_t rtg_sets_count(const rtg_sets *s) { return s ? s->nsets : 0; }
uint64_t rtg_sets_elems(const rtg_sets *s) { return s ? s->nelems : 0; }

void rtg_sets_destroy(rtg_sets *s) {
    if (!s) return;
    if (s->ctx) {
        cudaStreamSynchronize(s->ctx->stream);
        s->ctx->sets.erase(s);
    }
    if (!s->borrowed) {
        dev_free(s->off);
        dev_free(s->elems);
    }
    delete s;
}

/* ------------------------------------------------------ set intersection */

static rtg_status si_run(rtg_ctx *ctx, PairSpec &ps, const uint32_t *pair_a,
                         const uint32_t *pair_b, uint32_t *out, uint32_t flags, rtg_timing *t) {
    double t0 = now_ms();
    uint64_t l0 = ctx->launches;
    uint32_t family = flags & RTG_SI_FAMILY_MASK;
    if (family > RTG_SI_PLAIN)
        return fail(ctx, RTG_ERR_INVALID_ARG, "unknown SI family %u", family);
    uint64_t np = ps.npairs;
    uint32_t *d_pa = nullptr, *d_pb = nullptr, *d_out = nullptr;
    rtg_timing tm{};
    bool copied_in = false;
    // Pinned host pair ids and counts are read and written by the kernel itself over the
    // host link (no staging copies, no copy time outside the kernel); pageable ones are
    // copied through device scratch.
    void *mapped_a = nullptr, *mapped_b = nullptr, *mapped_out = nullptr;
    if (np && !ps.dense_nb && !(flags & RTG_PAIRS_DEVICE)) {
        mapped_a = mapped_host(pair_a);
        mapped_b = mapped_a ? mapped_host(pair_b) : nullptr;
    }
    if (np && !(flags & RTG_OUT_DEVICE)) mapped_out = mapped_host(out);
    if (!ps.dense_nb) {
        if (flags & RTG_PAIRS_DEVICE) {
            d_pa = const_cast<uint32_t *>(pair_a);
            d_pb = const_cast<uint32_t *>(pair_b);
        } else if (mapped_a && mapped_b) {
            d_pa = static_cast<uint32_t *>(mapped_a);
            d_pb = static_cast<uint32_t *>(mapped_b);
            tm.h2d_bytes = np * 8;
        } else {
            void *p = nullptr;
            RTG_TRY(scratch(ctx, 3, np * 8 + 16, &p));
            d_pa = (uint32_t *)p;
            d_pb = d_pa + np;
            RTG_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
            if (np) {
                RTG_CUDA(ctx, cudaMemcpyAsync(d_pa, pair_a, np * 4, cudaMemcpyHostToDevice,
                                              ctx->stream));
                RTG_CUDA(ctx, cudaMemcpyAsync(d_pb, pair_b, np * 4, cudaMemcpyHostToDevice,
                                              ctx->stream));
            }
            RTG_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
            tm.h2d_bytes = np * 8;
            copied_in = true;
        }
        ps.pa = d_pa;
        ps.pb = d_pb;
    }
    if (flags & RTG_OUT_DEVICE) {
        d_out = out;
    } else if (mapped_out) {
        d_out = static_cast<uint32_t *>(mapped_out);
        tm.d2h_bytes = np * 4;
    } else {
        void *p = nullptr;
        RTG_TRY(scratch(ctx, 4, np * 4 + 16, &p));
        d_out = (uint32_t *)p;
    }
    float kms = 0;
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    RTG_TRY(si_count_device(ctx, ps, d_out, family, &kms, &ctx->launches));
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
    const bool copy_out = !(flags & RTG_OUT_DEVICE) && np && !mapped_out;
    if (copy_out) {
        RTG_CUDA(ctx, cudaMemcpyAsync(out, d_out, np * 4, cudaMemcpyDeviceToHost, ctx->stream));
        tm.d2h_bytes = np * 4;
    }
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
    RTG_CUDA(ctx, cudaEventSynchronize(ctx->ev[2]));
    RTG_TRY(check_status_word(ctx));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    tm.count_ms = ms;
    tm.main_kernel_ms = kms;
    if (copied_in) {
        cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
        tm.h2d_ms = ms;
    }
    if (copy_out) {
        cudaEventElapsedTime(&ms, ctx->ev[1], ctx->ev[2]);
        tm.d2h_ms = ms;
    }
    tm.kernel_launches = ctx->launches - l0;
    tm.total_ms = now_ms() - t0;
    if (t) *t = tm;
    return RTG_OK;
}

rtg_status rtg_debug_si_wait_limit(rtg_ctx *ctx, uint32_t max_polls, uint32_t extra_tx_bytes) {
    if (!ctx || max_polls == 0 || extra_tx_bytes == 0 || (extra_tx_bytes & 15u))
        return RTG_ERR_INVALID_ARG;
    ctx->dbg_wait_polls = max_polls;
    ctx->dbg_extra_tx = extra_tx_bytes;
    return RTG_OK;
}

rtg_status rtg_si_count(rtg_ctx *ctx, const rtg_sets *s, const uint32_t *pair_a,
                        const uint32_t *pair_b, uint64_t npairs, uint32_t *out_counts,
                        uint32_t flags, rtg_timing *timing) {
    NvtxRange nvtx_("rtg_si_count");
    if (!ctx || !s || (npairs && (!pair_a || !pair_b || !out_counts))) return RTG_ERR_INVALID_ARG;
    if (npairs > 0xFFFFFFFFull)
        return fail(ctx, RTG_ERR_INVALID_ARG, "at most 2^32-1 pairs per call");
    PairSpec ps;
    ps.off = s->off;
    ps.elems = s->elems;
    ps.nsets = s->nsets;
    ps.npairs = npairs;
    return si_run(ctx, ps, pair_a, pair_b, out_counts, flags, timing);
}

rtg_status rtg_si_count_dense(rtg_ctx *ctx, const rtg_sets *s, uint32_t a_begin, uint32_t a_end,
                              uint32_t b_begin, uint32_t b_end, uint32_t *out_counts,
                              uint32_t flags, rtg_timing *timing) {
    NvtxRange nvtx_("rtg_si_count_dense");
    if (!ctx || !s || a_end < a_begin || b_end < b_begin || a_end > s->nsets ||
        b_end > s->nsets)
        return RTG_ERR_INVALID_ARG;
    uint64_t np = (uint64_t)(a_end - a_begin) * (b_end - b_begin);
    if (np && !out_counts) return RTG_ERR_INVALID_ARG;
    if (np > 0xFFFFFFFFull)
        return fail(ctx, RTG_ERR_INVALID_ARG, "at most 2^32-1 pairs per call");
    PairSpec ps;
    ps.off = s->off;
    ps.elems = s->elems;
    ps.nsets = s->nsets;
    ps.npairs = np;
    ps.dense_nb = b_end - b_begin;
    ps.a_begin = a_begin;
    ps.b_begin = b_begin;
    if (np == 0) {
        if (timing) *timing = rtg_timing{};
        return RTG_OK;
    }
    return si_run(ctx, ps, nullptr, nullptr, out_counts, flags & ~RTG_PAIRS_DEVICE, timing);
}

// Device-to-host copy of `bytes` into caller memory after the work on the context stream.
// Page-locked destinations and small copies go straight there, only enqueued (the caller
// synchronises the stream). A large pageable destination is filled through two page-locked
// staging buffers, and the call returns once it is filled: each chunk's copy over the host
// link runs while the host threads move the previous chunk into the caller's pages (the
// driver's own pageable path maps and fills those pages on one thread). Without staging
// memory the copy goes straight there too. Chunks are an eighth of the copy, 4 to 32 MB,
// so that a copy of a few tens of MB still overlaps its pieces.
constexpr size_t kStageBytes = size_t(32) << 20;  // each of the two staging buffers
constexpr size_t kStageMin = size_t(16) << 20;    // smaller copies go straight there

static rtg_status d2h_copy(rtg_ctx *ctx, void *dst, const void *src, size_t bytes) {
    if (!bytes) return RTG_OK;
    if (bytes >= kStageMin && !mapped_host(dst) && !ctx->h_stage) {
        void *h = nullptr;
        cudaEvent_t e[2] = {};
        bool ok = cudaHostAlloc(&h, 2 * kStageBytes, cudaHostAllocDefault) == cudaSuccess;
        for (auto &x : e) ok = ok && cudaEventCreateWithFlags(&x, cudaEventDisableTiming) == cudaSuccess;
        if (ok) {
            ctx->h_stage = h;
            ctx->stage_ev[0] = e[0];
            ctx->stage_ev[1] = e[1];
        } else {  // no staging: the copy goes straight to the caller's memory
            cudaGetLastError();
            for (auto &x : e)
                if (x) cudaEventDestroy(x);
            if (h) cudaFreeHost(h);
        }
    }
    if (bytes < kStageMin || !ctx->h_stage || mapped_host(dst)) {
        RTG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        return RTG_OK;
    }
    char *stage = static_cast<char *>(ctx->h_stage);
    const size_t C = std::min(kStageBytes,
                              std::max(size_t(4) << 20, (bytes / 8 + 4095) & ~size_t(4095)));
    const size_t chunks = (bytes + C - 1) / C;
    // chunk i lands in stage half i % 2; that half's previous chunk (i - 2) was moved out in
    // the iteration before
    for (size_t i = 0; i <= chunks; ++i) {
        if (i < chunks) {
            const size_t len = std::min(C, bytes - i * C);
            RTG_CUDA(ctx, cudaMemcpyAsync(stage + (i & 1) * kStageBytes,
                                          static_cast<const char *>(src) + i * C, len,
                                          cudaMemcpyDeviceToHost, ctx->stream));
            RTG_CUDA(ctx, cudaEventRecord(ctx->stage_ev[i & 1], ctx->stream));
        }
        if (i > 0) {
            const size_t j = i - 1, len = std::min(C, bytes - j * C);
            RTG_CUDA(ctx, cudaEventSynchronize(ctx->stage_ev[j & 1]));
            char *to = static_cast<char *>(dst) + j * C;
            const char *from = stage + (j & 1) * kStageBytes;
            constexpr size_t kPiece = size_t(1) << 20;
            const long long pieces = (long long)((len + kPiece - 1) / kPiece);
#pragma omp parallel for schedule(static)
            for (long long q = 0; q < pieces; ++q) {
                const size_t a = (size_t)q * kPiece;
                std::memcpy(to + a, from + a, std::min(kPiece, len - a));
            }
        }
    }
    return RTG_OK;
}

// Count -> scan -> write for the pairs of ps, then the offsets and elements to the host.
static rtg_status materialize_to_host(rtg_ctx *ctx, const PairSpec &ps, uint64_t *out_offsets,
                                      uint32_t *out_elems, uint64_t out_capacity,
                                      rtg_timing *timing, double t0, uint64_t l0) {
    const uint64_t npairs = ps.npairs;
    rtg_timing tm{};
    void *p = nullptr;
    uint64_t *d_off = nullptr;
    RTG_TRY(scratch(ctx, 4, (npairs + 1) * 8, &p));
    d_off = (uint64_t *)p;
    uint32_t *d_elems = nullptr;
    if (out_capacity) {
        RTG_TRY(scratch(ctx, 5, out_capacity * 4, &p));
        d_elems = (uint32_t *)p;
    }
    uint64_t needed = 0;
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    rtg_status st = si_materialize_device(ctx, ps, d_off, d_elems, out_capacity, &needed,
                                          &ctx->launches);
    if (st != RTG_OK && st != RTG_ERR_INVALID_ARG) return st;
    RTG_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
    RTG_TRY(d2h_copy(ctx, out_offsets, d_off, (npairs + 1) * 8));
    if (st == RTG_OK && needed) RTG_TRY(d2h_copy(ctx, out_elems, d_elems, needed * 4));
    RTG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    RTG_TRY(check_status_word(ctx));
    if (st != RTG_OK)
        return fail(ctx, RTG_ERR_INVALID_ARG, "output capacity %llu < %llu elements needed",
                    (unsigned long long)out_capacity, (unsigned long long)needed);
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]);
    tm.count_ms = ms;
    tm.d2h_bytes = (npairs + 1) * 8 + needed * 4;
    tm.kernel_launches = ctx->launches - l0;
    tm.total_ms = now_ms() - t0;
    if (timing) *timing = tm;
    return RTG_OK;
}

rtg_status rtg_si_materialize(rtg_ctx *ctx, const rtg_sets *s, const uint32_t *pair_a,
                              const uint32_t *pair_b, uint64_t npairs, uint64_t *out_offsets,
                              uint32_t *out_elems, uint64_t out_capacity, rtg_timing *timing) {
    NvtxRange nvtx_("rtg_si_materialize");
    if (!ctx || !s || !out_offsets || (npairs && (!pair_a || !pair_b))) return RTG_ERR_INVALID_ARG;
    if (npairs > 0xFFFFFFFFull)
        return fail(ctx, RTG_ERR_INVALID_ARG, "at most 2^32-1 pairs per call");
    double t0 = now_ms();
    uint64_t l0 = ctx->launches;
    void *p = nullptr;
    RTG_TRY(scratch(ctx, 3, npairs * 8 + 16, &p));
    uint32_t *d_pa = (uint32_t *)p, *d_pb = d_pa + npairs;
    if (npairs) {
        RTG_CUDA(ctx, cudaMemcpyAsync(d_pa, pair_a, npairs * 4, cudaMemcpyHostToDevice,
                                      ctx->stream));
        RTG_CUDA(ctx, cudaMemcpyAsync(d_pb, pair_b, npairs * 4, cudaMemcpyHostToDevice,
                                      ctx->stream));
    }
    PairSpec ps;
    ps.off = s->off;
    ps.elems = s->elems;
    ps.nsets = s->nsets;
    ps.npairs = npairs;
    ps.pa = d_pa;
    ps.pb = d_pb;
    return materialize_to_host(ctx, ps, out_offsets, out_elems, out_capacity, timing, t0, l0);
}

__global__ void k_row_ids(const uint64_t *off, uint32_t n, uint32_t *src) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n;
         v += (uint64_t)gridDim.x * blockDim.x)
        for (uint64_t e = off[v]; e < off[v + 1]; ++e) src[e] = (uint32_t)v;
}

rtg_status rtg_tc_list(rtg_ctx *ctx, rtg_graph *g, uint64_t *out_offsets, uint32_t *out_elems,
                       uint64_t out_capacity, rtg_timing *timing) {
    NvtxRange nvtx_("rtg_tc_list");
    if (!ctx || !g || !out_offsets || (out_capacity && !out_elems)) return RTG_ERR_INVALID_ARG;
    const Csr &c = g->ori;
    if (!c.built) return fail(ctx, RTG_ERR_STATE, "oriented CSR not built (rtg_csr_build)");
    if (c.m > 0xFFFFFFFFull)
        return fail(ctx, RTG_ERR_INVALID_ARG, "at most 2^32-1 oriented edges for listing");
    if (kChecked) RTG_TRY(check_csr(ctx, c, false));
    double t0 = now_ms();
    uint64_t l0 = ctx->launches;
    // the pairs are the edges themselves: (row of e, adj[e]) over the CSR's own rows
    const uint32_t *src = c.src;
    if (!src && c.m) {
        void *p = nullptr;
        RTG_TRY(scratch(ctx, 3, c.m * 4, &p));
        uint32_t *d_src = (uint32_t *)p;
        const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((c.n + 255) / 256,
                                                                        ctx->sm_count * 16ull));
        k_row_ids<<<grid, 256, 0, ctx->stream>>>(c.off, c.n, d_src);
        ctx->launches++;
        RTG_CUDA(ctx, cudaGetLastError());
        src = d_src;
    }
    PairSpec ps;
    ps.off = c.off;
    ps.elems = c.adj;
    ps.nsets = c.n;
    ps.npairs = c.m;
    ps.pa = src;
    ps.pb = c.adj;
    return materialize_to_host(ctx, ps, out_offsets, out_elems, out_capacity, timing, t0, l0);
}

rtg_status rtg_graph_pair_count(rtg_ctx *ctx, rtg_graph *g, const uint32_t *u, const uint32_t *v,
                                uint64_t npairs, uint32_t *out, uint32_t flags,
                                rtg_timing *timing) {
    NvtxRange nvtx_("rtg_graph_pair_count");
    if (!ctx || !g || (npairs && (!u || !v || !out))) return RTG_ERR_INVALID_ARG;
    if (!g->sym.built) return fail(ctx, RTG_ERR_STATE, "symmetric CSR not built");
    if (npairs > 0xFFFFFFFFull)
        return fail(ctx, RTG_ERR_INVALID_ARG, "at most 2^32-1 pairs per call");
    if (kChecked) RTG_TRY(check_csr(ctx, g->sym, false));
    PairSpec ps;
    ps.off = g->sym.off;
    ps.elems = g->sym.adj;
    ps.nsets = g->sym.n;
    ps.npairs = npairs;
    return si_run(ctx, ps, u, v, out, flags, timing);
}

}  // extern "C"
