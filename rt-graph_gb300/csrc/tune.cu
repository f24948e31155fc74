// Schedule autotuner for the batched forms.
//
// For a graph (TC) or a pair workload (SI) it times a grid of schedules — items per work
// unit, shared-memory region per warp and warps per block for the triangle count; staging
// slot size, slots per warp, warps per block and the search/merge length ratio for set
// intersection — each after an L2 flush, median of several runs with CUDA events, and keeps
// the fastest whose result is bit-identical to the library default's. The winner is set on
// the context and, with a cache path, stored under a key made of the device (SM count,
// compute capability) and the workload's size class, so later runs on the same kind of
// input skip the search.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "internal.h"

namespace rtg {
namespace {

uint32_t lg(uint64_t x) {
    uint32_t r = 0;
    while ((1ull << (r + 1)) <= x) ++r;
    return r;
}

const uint32_t *cfg_words(const rtg_config &c) { return reinterpret_cast<const uint32_t *>(&c); }
constexpr int kCfgWords = sizeof(rtg_config) / sizeof(uint32_t);

// the device, and the schedule's word count: entries written for another rtg_config layout
// do not match
std::string device_key(const rtg_ctx *ctx) {
    char b[64];
    snprintf(b, sizeof b, "sm%d/cc%d.%d/w%d", ctx->sm_count, ctx->cc_major, ctx->cc_minor,
             kCfgWords);
    return b;
}

bool cache_lookup(const char *path, const std::string &key, rtg_config *cfg, double *ms) {
    if (!path) return false;
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        std::istringstream in(line);
        std::string k;
        if (!(in >> k) || k != key) continue;
        uint32_t w[kCfgWords];
        bool ok = true;
        for (int i = 0; i < kCfgWords && ok; ++i) ok = static_cast<bool>(in >> w[i]);
        double t = 0;
        if (ok && (in >> t)) {
            memcpy(cfg, w, sizeof w);
            *ms = t;
            found = true;  // the last entry for a key wins
        }
    }
    return found;
}

void cache_store(const char *path, const std::string &key, const rtg_config &cfg, double ms) {
    if (!path) return;
    std::vector<std::string> keep;
    {
        std::ifstream f(path);
        std::string line;
        while (std::getline(f, line)) {
            std::istringstream in(line);
            std::string k;
            if ((in >> k) && k != key) keep.push_back(line);
        }
    }
    std::ofstream f(path, std::ios::trunc);
    for (auto &l : keep) f << l << "\n";
    f << key;
    for (int i = 0; i < kCfgWords; ++i) f << " " << cfg_words(cfg)[i];
    f << " " << ms << "\n";
}

double median(std::vector<double> v) {
    std::sort(v.begin(), v.end());
    return v.empty() ? 0 : v[v.size() / 2];
}

constexpr int kReps = 3;

}  // namespace
}  // namespace rtg

using namespace rtg;

extern "C" rtg_status rtg_tune_tc(rtg_ctx *ctx, rtg_graph *g, const char *cache_path,
                                  rtg_tune_result *res) {
    NvtxRange nvtx_("rtg_tune_tc");
    if (!ctx || !g || !res) return RTG_ERR_INVALID_ARG;
    memset(res, 0, sizeof *res);
    if (!g->ori.built || !g->cnt.built) return fail(ctx, RTG_ERR_STATE, "oriented CSR not built");
    char kb[128];
    snprintf(kb, sizeof kb, "tc/%s/n%u/m%u/d%u", device_key(ctx).c_str(), lg(g->cnt.n + 1ull),
             lg(g->cnt.m + 1), lg(g->cnt.max_deg + 1ull));
    const std::string key = kb;
    const rtg_config saved = ctx->cfg;
    rtg_config cached{};
    double cached_ms = 0;
    if (cache_lookup(cache_path, key, &cached, &cached_ms) &&
        rtg_set_config(ctx, &cached) == RTG_OK) {
        res->best = cached;
        res->best_ms = cached_ms;
        res->from_cache = 1;
        return RTG_OK;
    }
    auto run = [&](const rtg_config &c, uint64_t *total, double *ms,
                   uint32_t *core = nullptr) -> rtg_status {
        rtg_status st = rtg_set_config(ctx, &c);
        if (st != RTG_OK) return st;
        rtg_timing t{};
        RTG_TRY(tc_count(ctx, g, RTG_TC_BATCHED, total, &t));  // builds the plan
        if (core) *core = t.core_ranks;
        std::vector<double> v;
        for (int r = 0; r < kReps; ++r) {
            RTG_TRY(rtg_flush_l2(ctx));
            uint64_t x = 0;
            RTG_TRY(tc_count(ctx, g, RTG_TC_BATCHED, &x, &t));
            if (x != *total) return fail(ctx, RTG_ERR_STATE, "count changed between runs");
            v.push_back(t.count_ms);
        }
        *ms = median(v);
        return RTG_OK;
    };
    // the SI fields of the context's schedule are kept as they are
    rtg_config def = saved;
    def.tc_item_edges = def.tc_region_words = def.tc_block_warps = def.tc_blocks_per_sm = 0;
    def.tc_core_ranks = 0;
    uint64_t want = 0;
    double def_ms = 0;
    uint32_t core0 = 0;  // the library's dense-core size on this graph
    rtg_status st = run(def, &want, &def_ms, &core0);
    if (st != RTG_OK) {
        ctx->cfg = saved;
        return st;
    }
    rtg_config best = def;
    double best_ms = def_ms;
    for (uint32_t E : {128u, 256u, 512u, 1024u})
        for (uint32_t R : {512u, 1024u, 2048u})
            for (uint32_t W : {4u, 8u, 16u}) {
                rtg_config c = def;
                c.tc_item_edges = E;
                c.tc_region_words = R;
                c.tc_block_warps = W;
                uint64_t got = 0;
                double ms = 0;
                res->candidates++;
                if ((size_t)W * (R + 1) * 4 + 256 > (size_t)ctx->smem_optin ||
                    run(c, &got, &ms) != RTG_OK || got != want) {
                    res->rejected++;
                    continue;
                }
                if (ms < best_ms) {
                    best_ms = ms;
                    best = c;
                }
            }
    // the dense core on the best schedule: none, half and twice the library's choice (within
    // 1024 .. 32768 ranks), or, where it chose none, 4096 and 16384 ranks; one replaces the
    // library's choice only when it is at least 1 % faster (R-MAT-21: 24576 and 32768 ranks
    // are within 0.5 % of each other, and run-to-run noise would otherwise decide)
    std::vector<uint32_t> cores;
    if (core0) {
        cores.push_back(RTG_TC_CORE_NONE);
        if (core0 / 2 >= 1024) cores.push_back(core0 / 2);
        if (core0 < RTG_TC_CORE_MAX_RANKS)
            cores.push_back(std::min<uint32_t>(2 * core0, RTG_TC_CORE_MAX_RANKS));
    } else {
        for (uint32_t K : {4096u, 16384u})
            if (K <= g->cnt.n) cores.push_back(K);
    }
    const rtg_config sched = best;
    for (uint32_t K : cores) {
        rtg_config c = sched;
        c.tc_core_ranks = K;
        uint64_t got = 0;
        double ms = 0;
        res->candidates++;
        if (run(c, &got, &ms) != RTG_OK || got != want) {
            res->rejected++;
            continue;
        }
        if (ms < 0.99 * best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    ctx->last_error.clear();
    rtg_set_config(ctx, &best);
    res->best = best;
    res->best_ms = best_ms;
    res->default_ms = def_ms;
    cache_store(cache_path, key, best, best_ms);
    return RTG_OK;
}

extern "C" rtg_status rtg_tune_si(rtg_ctx *ctx, const rtg_sets *s, const uint32_t *pair_a,
                                  const uint32_t *pair_b, uint64_t npairs,
                                  const char *cache_path, rtg_tune_result *res) {
    NvtxRange nvtx_("rtg_tune_si");
    if (!ctx || !s || !res || !npairs || !pair_a || !pair_b) return RTG_ERR_INVALID_ARG;
    memset(res, 0, sizeof *res);
    std::vector<uint64_t> off(s->nsets + 1);
    uint64_t elems = 0;
    // the size class of the workload: pairs, mean and largest list of the pairs given
    RTG_CUDA(ctx, cudaMemcpy(off.data(), s->off, off.size() * 8, cudaMemcpyDeviceToHost));
    uint64_t mx = 0;
    for (uint64_t i = 0; i < npairs; ++i) {
        if (pair_a[i] >= s->nsets || pair_b[i] >= s->nsets)
            return fail(ctx, RTG_ERR_INVALID_ARG, "pair %llu names a set out of range",
                        (unsigned long long)i);
        const uint64_t la = off[pair_a[i] + 1] - off[pair_a[i]], lb = off[pair_b[i] + 1] - off[pair_b[i]];
        elems += la + lb;
        mx = std::max(mx, std::max(la, lb));
    }
    char kb[128];
    snprintf(kb, sizeof kb, "si/%s/p%u/l%u/x%u", device_key(ctx).c_str(), lg(npairs),
             lg(elems / (2 * npairs) + 1), lg(mx + 1));
    const std::string key = kb;
    const rtg_config saved = ctx->cfg;
    rtg_config cached{};
    double cached_ms = 0;
    if (cache_lookup(cache_path, key, &cached, &cached_ms) &&
        rtg_set_config(ctx, &cached) == RTG_OK) {
        res->best = cached;
        res->best_ms = cached_ms;
        res->from_cache = 1;
        return RTG_OK;
    }
    uint32_t *d = nullptr;
    RTG_TRY(dev_alloc(ctx, (void **)&d, npairs * 16 + 64));
    uint32_t *dpa = d, *dpb = d + npairs, *dwant = d + 2 * npairs, *dgot = d + 3 * npairs;
    struct Free {
        uint32_t *p;
        ~Free() { dev_free(p); }
    } fr{d};
    RTG_CUDA(ctx, cudaMemcpyAsync(dpa, pair_a, npairs * 4, cudaMemcpyHostToDevice, ctx->stream));
    RTG_CUDA(ctx, cudaMemcpyAsync(dpb, pair_b, npairs * 4, cudaMemcpyHostToDevice, ctx->stream));
    PairSpec ps;
    ps.off = s->off;
    ps.elems = s->elems;
    ps.nsets = s->nsets;
    ps.pa = dpa;
    ps.pb = dpb;
    ps.npairs = npairs;
    std::vector<uint32_t> hw(npairs), hg(npairs);
    auto run = [&](const rtg_config &c, uint32_t *out, double *ms) -> rtg_status {
        RTG_TRY(rtg_set_config(ctx, &c));
        float k = 0;
        RTG_TRY(si_count_device(ctx, ps, out, RTG_SI_AUTO, &k, &ctx->launches));
        std::vector<double> v;
        for (int r = 0; r < kReps; ++r) {
            RTG_TRY(rtg_flush_l2(ctx));
            RTG_TRY(si_count_device(ctx, ps, out, RTG_SI_AUTO, &k, &ctx->launches));
            v.push_back(k);
        }
        RTG_TRY(check_status_word(ctx));
        *ms = median(v);
        return RTG_OK;
    };
    // the TC fields of the context's schedule are kept as they are
    rtg_config def = saved;
    def.si_block_warps = def.si_search_ratio = def.si_stage_slots = def.si_stage_bytes = 0;
    def.si_blocks_per_sm = def.si_skew_stream = def.si_form = 0;
    double def_ms = 0;
    rtg_status st = run(def, dwant, &def_ms);
    if (st != RTG_OK) {
        ctx->cfg = saved;
        return st;
    }
    RTG_CUDA(ctx, cudaMemcpy(hw.data(), dwant, npairs * 4, cudaMemcpyDeviceToHost));
    rtg_config best = def;
    double best_ms = def_ms;
    auto consider = [&](const rtg_config &c, size_t smem) {
        double ms = 0;
        res->candidates++;
        if (smem > (size_t)ctx->smem_optin || run(c, dgot, &ms) != RTG_OK ||
            cudaMemcpy(hg.data(), dgot, npairs * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            hg != hw) {
            res->rejected++;
            return;
        }
        if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    };
    // per-warp rings: slot size x slots per warp x warps per block x search ratio
    for (uint32_t B : {2048u, 4096u, 8192u})
        for (uint32_t S : {2u, 3u, 4u})
            for (uint32_t W : {4u, 8u, 16u})
                for (uint32_t ratio : {4u, 8u, 16u, 32u}) {
                    rtg_config c = def;
                    c.si_form = 1;
                    c.si_stage_bytes = B;
                    c.si_stage_slots = S;
                    c.si_block_warps = W;
                    c.si_search_ratio = ratio;
                    consider(c, (size_t)W * S * (B + 512) + 4096);
                }
    // producer/consumer: slot size x ring slots x merging warps per producer x search ratio
    for (uint32_t B : {6144u, 8192u, 10240u})
        for (uint32_t S : {3u, 4u, 5u, 6u})
            for (uint32_t W : {2u, 3u, 4u})
                for (uint32_t ratio : {8u, 16u}) {
                    rtg_config c = def;
                    c.si_form = 2;
                    c.si_stage_bytes = B;
                    c.si_stage_slots = S;
                    c.si_block_warps = W;
                    c.si_search_ratio = ratio;
                    consider(c, (size_t)S * (B + 512) + 4096);
                }
    {
        // the best schedule with skewed pairs staged and streamed instead of searched
        rtg_config c = best;
        c.si_skew_stream = 1;
        double ms = 0;
        res->candidates++;
        if (run(c, dgot, &ms) != RTG_OK ||
            cudaMemcpy(hg.data(), dgot, npairs * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            hg != hw) {
            res->rejected++;
        } else if (ms < best_ms) {
            best_ms = ms;
            best = c;
        }
    }
    ctx->last_error.clear();
    rtg_set_config(ctx, &best);
    res->best = best;
    res->best_ms = best_ms;
    res->default_ms = def_ms;
    cache_store(cache_path, key, best, best_ms);
    return RTG_OK;
}
