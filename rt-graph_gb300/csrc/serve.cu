// Serving: a request loop over many graphs resident in HBM.
//
// One engine thread owns every launch. It keeps
//   - a build context (graph construction, serialised by build_mu),
//   - kTcRuns TC contexts, each with its own stream, that replay a graph's captured
//     batched-count graph (or launch the count directly into the run's scratch),
//   - si_slots set-intersection contexts, each with its own stream, pinned staging and
//     device buffers for one merged launch.
// Each pass of the engine loop: completes launches whose events have fired (copying
// counts into the callers' buffers), then launches triangle counts for graphs with none in
// flight (admitting their counting plans against the HBM budget, evicting idle plans in
// LRU order) and packs the pair requests waiting at that moment — any graphs, any sizes,
// large requests split across launches — into one persistent k_si_stream launch per free
// slot. Pairs carry their graph's slot in a per-pair table index, so one launch reads the
// symmetric CSRs of many graphs. TC and SI launches run on different streams and overlap
// on the device; the engine never blocks on the device while work is in flight.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace rtg {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

constexpr uint32_t kDefaultBatchPairs = 1u << 19;
constexpr uint32_t kDefaultSlots = 2;
constexpr uint32_t kMaxSlots = 4;
constexpr uint32_t kDefaultMaxGraphs = 1024;
constexpr uint32_t kTcRuns = 8;  // triangle counts in flight at once

struct SGraph {
    rtg_graph *g = nullptr;
    rtg_graph_info info{};
    uint32_t n_sym = 0;
    uint64_t bytes = 0;       // resident CSR bytes
    uint64_t plan_bytes = 0;  // batched counting plan, while it exists
    bool removing = false;
    uint32_t refs = 0;        // queued + running requests
    bool tc_busy = false;
    uint64_t tc_tick = 0;     // last TC launch (LRU order of plans)
};

struct Req {
    uint64_t id = 0;
    uint32_t kind = RTG_REQ_TC, graph = 0;
    const uint32_t *u = nullptr, *v = nullptr;
    uint32_t *out = nullptr;
    uint64_t np = 0;
    uint64_t next = 0;    // pairs handed to launches
    uint64_t landed = 0;  // pairs whose launches completed
    uint64_t tri = 0;
    rtg_status status = RTG_OK;
    bool cancelled = false, launched = false;
    bool closed = false;  // no further pairs are handed out (cancelled or failed)
    uint32_t launches = 0, batch_requests = 0;
    Clock::time_point t_submit, t_launch, t_done;
};

struct Piece {
    Req *r;
    uint64_t begin, count, at;
};

struct SiSlot {
    rtg_ctx *ctx = nullptr;
    uint32_t *d_pairs = nullptr;  // pa | pb | pg, cap entries each
    uint32_t *d_out = nullptr;
    SetRef *d_tab = nullptr;
    uint32_t *h_pairs = nullptr;  // pinned
    uint32_t *h_out = nullptr;    // pinned
    uint32_t *h_status = nullptr; // pinned
    SetRef *h_tab = nullptr;      // pinned
    uint64_t tab_version = ~0ull;
    cudaEvent_t done = nullptr;
    bool busy = false;
    std::vector<Piece> pieces;
    uint64_t launch_no = 0;
};

struct TcRun {
    rtg_ctx *ctx = nullptr;  // own stream: counts of different graphs overlap
    SGraph *sg = nullptr;
    uint32_t slot = 0;
    std::vector<Req *> reqs;
    unsigned long long *h_total = nullptr;  // pinned
    cudaEvent_t done = nullptr;
    bool busy = false;
    void *scratch = nullptr;  // direct counts of graphs without a cached plan
    uint64_t scratch_bytes = 0;
};

}  // namespace
}  // namespace rtg

using namespace rtg;

struct rtg_server {
    int device = 0;
    rtg_serve_config cfg{};
    std::mutex mu;               // requests, graphs, stats
    std::condition_variable cv;  // engine wake-up
    std::condition_variable cv_done;
    std::mutex build_mu;         // the build context and graph destruction
    std::mutex err_mu;
    std::string last_error;
    rtg_ctx *build = nullptr, *tcx = nullptr;
    std::vector<SiSlot> slots;
    std::vector<TcRun> runs;
    std::vector<SGraph> graphs;  // by slot; g == nullptr when free
    SetRef *h_tab = nullptr;     // host copy of the collection table (max_graphs entries)
    uint64_t tab_version = 0;
    std::unordered_map<uint64_t, Req *> active;
    std::deque<Req *> tc_queue, si_queue;
    std::map<uint64_t, rtg_request_info> done;
    std::deque<uint64_t> done_order;
    uint64_t next_id = 1;
    uint64_t tick = 0;
    uint64_t si_launch_count = 0;
    bool held = false, stopping = false;
    std::thread engine;
    rtg_serve_stats st{};
    uint64_t resident = 0, plans = 0, buffers = 0;
};

namespace {

rtg_status srv_fail(rtg_server *s, rtg_status st, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    std::lock_guard<std::mutex> lk(s->err_mu);
    s->last_error = buf;
    return st;
}

uint64_t used_bytes(const rtg_server *s) { return s->resident + s->plans + s->buffers; }

// Record a finished request (caller holds mu).
void finish(rtg_server *s, Req *r) {
    r->t_done = Clock::now();
    rtg_request_info in{};
    in.status = r->cancelled ? RTG_ERR_CANCELLED : r->status;
    in.kind = r->kind;
    in.graph = r->graph;
    in.launches = r->launches;
    in.batch_requests = r->batch_requests;
    in.npairs = r->np;
    in.triangles = r->tri;
    in.latency_ms = ms_between(r->t_submit, r->t_done);
    in.queue_ms = r->launched ? ms_between(r->t_submit, r->t_launch) : in.latency_ms;
    s->done[r->id] = in;
    s->done_order.push_back(r->id);
    s->active.erase(r->id);
    if (in.status == RTG_OK) s->st.completed++;
    else if (in.status == RTG_ERR_CANCELLED) s->st.cancelled++;
    else s->st.failed++;
    SGraph &g = s->graphs[r->graph];
    if (g.refs) g.refs--;
    delete r;
    s->cv_done.notify_all();
}

void mark_launched(Req *r, Clock::time_point now, uint32_t nreq) {
    if (!r->launched) {
        r->launched = true;
        r->t_launch = now;
    }
    r->launches++;
    r->batch_requests = std::max(r->batch_requests, nreq);
}

rtg_status map_status_word(uint32_t w) {
    if (w == kStatusOk) return RTG_OK;
    return w == kStatusTimeout ? RTG_ERR_TIMEOUT : RTG_ERR_INVALID_ARG;
}

// ---------------------------------------------------------------- completions

bool complete_si(rtg_server *s, SiSlot &sl) {
    cudaError_t q = cudaEventQuery(sl.done);
    if (q == cudaErrorNotReady) return false;
    rtg_status st = RTG_OK;
    if (q != cudaSuccess) {
        cudaGetLastError();
        st = srv_fail(s, RTG_ERR_DEVICE, "set-intersection launch failed: %s", cudaGetErrorString(q));
    } else if (s->cfg.inject_fail_launch && sl.launch_no == s->cfg.inject_fail_launch) {
        st = srv_fail(s, RTG_ERR_DEVICE, "set-intersection launch %llu reported failed (injected)",
                      (unsigned long long)sl.launch_no);
    } else if (*sl.h_status != kStatusOk) {
        st = map_status_word(*sl.h_status);
        srv_fail(s, st, "device status word %u after set-intersection launch", *sl.h_status);
    }
    for (const Piece &p : sl.pieces) {
        Req *r = p.r;
        if (st != RTG_OK && !r->closed) {
            // a failed launch ends the request: the rest of it is not handed out
            if (r->status == RTG_OK) r->status = st;
            r->closed = true;
            auto qi = std::find(s->si_queue.begin(), s->si_queue.end(), r);
            if (qi != s->si_queue.end()) s->si_queue.erase(qi);
        }
        if (!r->cancelled && st == RTG_OK)
            memcpy(r->out + p.begin, sl.h_out + p.at, p.count * sizeof(uint32_t));
        r->landed += p.count;
        if (r->landed == (r->closed ? r->next : r->np)) finish(s, r);
    }
    sl.pieces.clear();
    sl.busy = false;
    return true;
}

bool complete_tc(rtg_server *s, TcRun &run) {
    cudaError_t q = cudaEventQuery(run.done);
    if (q == cudaErrorNotReady) return false;
    rtg_status st = RTG_OK;
    if (q != cudaSuccess) {
        cudaGetLastError();
        st = srv_fail(s, RTG_ERR_DEVICE, "triangle-count launch failed: %s", cudaGetErrorString(q));
    }
    for (Req *r : run.reqs) {
        r->status = st;
        r->tri = *run.h_total;
        r->landed = 1;
        finish(s, r);
    }
    run.reqs.clear();
    run.sg->tc_busy = false;
    run.busy = false;
    return true;
}

// ---------------------------------------------------------------- launches

// Free idle counting plans, least recently used first, until `need` more bytes fit.
bool make_room(rtg_server *s, uint64_t need, const SGraph *keep) {
    while (used_bytes(s) + need > s->st.budget_bytes) {
        SGraph *victim = nullptr;
        for (SGraph &g : s->graphs)
            if (g.g && &g != keep && g.plan_bytes && !g.tc_busy &&
                (!victim || g.tc_tick < victim->tc_tick))
                victim = &g;
        if (!victim) return false;
        tc_plan_release(victim->g);
        s->plans -= victim->plan_bytes;
        victim->plan_bytes = 0;
        s->st.plan_evictions++;
    }
    return true;
}

void launch_tc(rtg_server *s) {
    for (auto it = s->tc_queue.begin(); it != s->tc_queue.end();) {
        Req *r = *it;
        SGraph &g = s->graphs[r->graph];
        if (g.tc_busy) {
            ++it;
            continue;
        }
        TcRun *run = nullptr;
        for (TcRun &x : s->runs)
            if (!x.busy) {
                run = &x;
                break;
            }
        if (!run) return;
        // A graph keeps a captured counting plan when the budget has room for one; otherwise
        // it is counted with direct launches in the run's own scratch, grown to the largest
        // graph seen (idle plans are evicted only when that scratch cannot grow otherwise).
        bool use_plan = g.plan_bytes != 0;
        if (!use_plan) {
            const uint64_t need = tc_plan_estimate_bytes(s->tcx, g.g);
            if (used_bytes(s) + need <= s->st.budget_bytes) {
                g.plan_bytes = need;
                s->plans += need;
                use_plan = true;
            } else if (run->scratch_bytes < need) {
                const uint64_t grow = need - run->scratch_bytes;
                if (!make_room(s, grow, &g)) {
                    bool any_running = false;
                    for (TcRun &x : s->runs) any_running |= x.busy;
                    if (!any_running) {  // nothing will free memory: refuse
                        it = s->tc_queue.erase(it);
                        r->status = srv_fail(s, RTG_ERR_OOM,
                                             "count of graph %u needs %llu B beyond the budget",
                                             r->graph, (unsigned long long)grow);
                        finish(s, r);
                        continue;
                    }
                    s->st.admission_waits++;
                    ++it;
                    continue;
                }
                dev_free(run->scratch);  // the run is idle: its last count has completed
                s->buffers -= run->scratch_bytes;
                run->scratch = nullptr;
                run->scratch_bytes = 0;
                if (dev_alloc(run->ctx, &run->scratch, need) != RTG_OK) {
                    it = s->tc_queue.erase(it);
                    r->status = srv_fail(s, RTG_ERR_OOM, "run scratch of %llu B",
                                         (unsigned long long)need);
                    finish(s, r);
                    continue;
                }
                run->scratch_bytes = need;
                s->buffers += need;
            }
        }
        // every waiting TC request of this graph shares this launch
        run->reqs.clear();
        for (auto jt = it; jt != s->tc_queue.end();) {
            if ((*jt)->graph == r->graph) {
                run->reqs.push_back(*jt);
                jt = s->tc_queue.erase(jt);
            } else {
                ++jt;
            }
        }
        it = s->tc_queue.begin();
        const auto now = Clock::now();
        for (Req *q : run->reqs) mark_launched(q, now, (uint32_t)run->reqs.size());
        s->st.tc_coalesced += run->reqs.size() - 1;
        rtg_status st = use_plan ? tc_launch_async(run->ctx, g.g, run->h_total)
                                 : tc_launch_direct(run->ctx, g.g, run->scratch,
                                                    run->scratch_bytes, run->h_total);
        if (!use_plan) s->st.tc_direct++;
        if (st == RTG_OK) {
            cudaError_t e = cudaEventRecord(run->done, run->ctx->stream);
            if (e != cudaSuccess) st = cuda_fail(run->ctx, e, "event", __FILE__, __LINE__);
        }
        if (st != RTG_OK) {
            srv_fail(s, st, "triangle count of graph %u: %s", r->graph, rtg_last_error(run->ctx));
            for (Req *q : run->reqs) {
                q->status = st;
                finish(s, q);
            }
            run->reqs.clear();
            continue;
        }
        s->st.tc_launches++;
        g.tc_busy = true;
        g.tc_tick = ++s->tick;
        run->sg = &g;
        run->busy = true;
    }
}

void launch_si(rtg_server *s) {
    const uint64_t cap = s->cfg.max_batch_pairs;
    for (SiSlot &sl : s->slots) {
        if (sl.busy) continue;
        while (!s->si_queue.empty() && s->si_queue.front()->closed) s->si_queue.pop_front();
        if (s->si_queue.empty()) return;
        // take the waiting pair requests in arrival order, splitting the last one
        sl.pieces.clear();
        uint64_t np = 0;
        for (auto it = s->si_queue.begin(); it != s->si_queue.end() && np < cap;) {
            Req *r = *it;
            if (r->closed) {
                it = s->si_queue.erase(it);
                continue;
            }
            const uint64_t take = std::min(r->np - r->next, cap - np);
            sl.pieces.push_back({r, r->next, take, np});
            r->next += take;
            np += take;
            if (r->next == r->np) it = s->si_queue.erase(it);
            else ++it;
        }
        if (np == 0) return;
        uint32_t *pa = sl.h_pairs, *pb = pa + np, *pg = pb + np;
        for (const Piece &p : sl.pieces) {
            memcpy(pa + p.at, p.r->u + p.begin, p.count * 4);
            memcpy(pb + p.at, p.r->v + p.begin, p.count * 4);
            std::fill(pg + p.at, pg + p.at + p.count, p.r->graph);
        }
        const auto now = Clock::now();
        const uint32_t nreq = (uint32_t)sl.pieces.size();
        for (const Piece &p : sl.pieces) mark_launched(p.r, now, nreq);
        rtg_ctx *c = sl.ctx;
        rtg_status st = RTG_OK;
        auto cu = [&](cudaError_t e, const char *what) {
            if (st == RTG_OK && e != cudaSuccess) st = cuda_fail(c, e, what, __FILE__, __LINE__);
        };
        if (sl.tab_version != s->tab_version) {
            memcpy(sl.h_tab, s->h_tab, sizeof(SetRef) * s->cfg.max_graphs);
            cu(cudaMemcpyAsync(sl.d_tab, sl.h_tab, sizeof(SetRef) * s->cfg.max_graphs,
                               cudaMemcpyHostToDevice, c->stream), "table copy");
            sl.tab_version = s->tab_version;
        }
        cu(cudaMemcpyAsync(sl.d_pairs, sl.h_pairs, np * 12, cudaMemcpyHostToDevice, c->stream),
           "pair copy");
        if (st == RTG_OK) {
            PairSpec ps;
            ps.pa = sl.d_pairs;
            ps.pb = sl.d_pairs + np;
            ps.pg = sl.d_pairs + 2 * np;
            ps.gtab = sl.d_tab;
            ps.ngraphs = s->cfg.max_graphs;
            ps.npairs = np;
            st = si_count_device(c, ps, sl.d_out, RTG_SI_AUTO, nullptr, &c->launches);
        }
        cu(cudaMemcpyAsync(sl.h_out, sl.d_out, np * 4, cudaMemcpyDeviceToHost, c->stream), "count copy");
        cu(cudaMemcpyAsync(sl.h_status, c->d_status, 4, cudaMemcpyDeviceToHost, c->stream), "status copy");
        cu(cudaMemsetAsync(c->d_status, 0, 4, c->stream), "status reset");
        cu(cudaEventRecord(sl.done, c->stream), "event");
        sl.launch_no = ++s->si_launch_count;
        if (st != RTG_OK) {
            srv_fail(s, st, "set-intersection launch: %s", rtg_last_error(c));
            for (const Piece &p : sl.pieces) {
                Req *r = p.r;
                if (r->status == RTG_OK) r->status = st;
                r->closed = true;
                auto qi = std::find(s->si_queue.begin(), s->si_queue.end(), r);
                if (qi != s->si_queue.end()) s->si_queue.erase(qi);
                r->landed += p.count;
                if (r->landed == r->next) finish(s, r);
            }
            sl.pieces.clear();
            continue;
        }
        s->st.si_launches++;
        s->st.si_pairs += np;
        s->st.max_requests_per_launch = std::max<uint64_t>(s->st.max_requests_per_launch, nreq);
        sl.busy = true;
    }
}

void engine_loop(rtg_server *s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        for (SiSlot &sl : s->slots)
            if (sl.busy) complete_si(s, sl);
        for (TcRun &run : s->runs)
            if (run.busy) complete_tc(s, run);
        // graphs marked for removal with no request left
        std::vector<rtg_graph *> dead;
        for (uint32_t i = 0; i < s->graphs.size(); ++i) {
            SGraph &g = s->graphs[i];
            if (g.g && g.removing && g.refs == 0 && !g.tc_busy) {
                dead.push_back(g.g);
                s->resident -= g.bytes;
                s->plans -= g.plan_bytes;
                g = SGraph{};
                s->h_tab[i] = SetRef{nullptr, nullptr, 0};
                s->tab_version++;
                s->st.resident_graphs--;
            }
        }
        if (!dead.empty()) {
            lk.unlock();
            {
                std::lock_guard<std::mutex> bl(s->build_mu);
                for (rtg_graph *g : dead) rtg_graph_destroy(g);
            }
            lk.lock();
        }
        if (!s->held) {
            launch_tc(s);
            launch_si(s);
        }
        uint32_t inflight = 0;
        for (SiSlot &sl : s->slots) inflight += sl.busy;
        for (TcRun &run : s->runs) inflight += run.busy;
        s->st.max_inflight_launches = std::max<uint64_t>(s->st.max_inflight_launches, inflight);
        if (s->stopping && inflight == 0) break;
        if (inflight) {
            lk.unlock();
            std::this_thread::yield();
            lk.lock();
        } else {
            s->cv.wait_for(lk, std::chrono::milliseconds(2));
        }
    }
}

rtg_status get_graph(rtg_server *s, uint32_t id, SGraph **out) {
    if (id >= s->graphs.size() || !s->graphs[id].g || s->graphs[id].removing)
        return srv_fail(s, RTG_ERR_INVALID_ARG, "unknown graph %u", id);
    *out = &s->graphs[id];
    return RTG_OK;
}

rtg_status add_built_graph(rtg_server *s, rtg_graph *g, uint32_t *graph_id) {
    // the oriented CSR is not needed once its counting form exists
    uint64_t bytes = 0;
    {
        std::lock_guard<std::mutex> bl(s->build_mu);
        cudaStreamSynchronize(s->build->stream);
        graph_free_csr(g->ori);
        g->ori.built = false;
        const CountCsr &cc = g->cnt;
        bytes = (uint64_t)(g->sym.n + 1) * 8 + g->sym.m * 4 + kAdjPadBytes +
                (uint64_t)(cc.n + 1) * 16 + cc.m * 12 + kAdjPadBytes;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    rtg_status st = RTG_OK;
    if (s->stopping) st = srv_fail(s, RTG_ERR_STATE, "server is stopping");
    else if (used_bytes(s) + bytes > s->st.budget_bytes && !make_room(s, bytes, nullptr))
        st = srv_fail(s, RTG_ERR_OOM, "graph needs %llu B; %llu of %llu B in use",
                      (unsigned long long)bytes, (unsigned long long)used_bytes(s),
                      (unsigned long long)s->st.budget_bytes);
    uint32_t slot = 0;
    if (st == RTG_OK) {
        while (slot < s->graphs.size() && s->graphs[slot].g) ++slot;
        if (slot == s->graphs.size()) st = srv_fail(s, RTG_ERR_BUSY, "every graph slot is taken");
    }
    if (st != RTG_OK) {
        std::lock_guard<std::mutex> bl(s->build_mu);
        rtg_graph_destroy(g);
        return st;
    }
    SGraph &sg = s->graphs[slot];
    sg = SGraph{};
    sg.g = g;
    sg.bytes = bytes;
    sg.n_sym = g->sym.n;
    sg.info.n = g->cnt.n;
    sg.info.m_input = g->m_input;
    sg.info.m = g->cnt.m;
    sg.info.max_out_degree = g->cnt.max_deg;
    sg.info.orient = RTG_ORIENT_DEGREE;
    sg.info.has_symmetric = 1;
    sg.info.n_sym = g->sym.n;
    sg.info.m_sym = g->sym.m;
    s->h_tab[slot] = SetRef{g->sym.off, g->sym.adj, g->sym.n};
    s->tab_version++;
    s->resident += bytes;
    s->st.resident_graphs++;
    *graph_id = slot;
    return RTG_OK;
}

rtg_status build_graph(rtg_server *s, rtg_graph *g) {
    rtg_status st = rtg_csr_build(s->build, g, RTG_ORIENT_DEGREE);
    if (st == RTG_OK) st = rtg_csr_build(s->build, g, RTG_ORIENT_SYMMETRIC);
    if (st == RTG_OK) st = rtg_graph_release_edges(g);
    if (st != RTG_OK) {
        srv_fail(s, st, "graph build: %s", rtg_last_error(s->build));
        rtg_graph_destroy(g);
    }
    return st;
}

rtg_status wait_for(rtg_server *s, std::unique_lock<std::mutex> &lk, int32_t wait_ms,
                    const std::function<bool()> &ready) {
    if (ready()) return RTG_OK;
    if (wait_ms == 0) return RTG_ERR_BUSY;
    if (wait_ms < 0) {
        s->cv_done.wait(lk, ready);
        return RTG_OK;
    }
    return s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), ready) ? RTG_OK
                                                                              : RTG_ERR_BUSY;
}

}  // namespace

extern "C" {

rtg_status rtg_serve_start(int device, const rtg_serve_config *cfg, rtg_server **out) {
    if (!out) return RTG_ERR_INVALID_ARG;
    *out = nullptr;
    rtg_serve_config c = cfg ? *cfg : rtg_serve_config{};
    if (!c.max_batch_pairs) c.max_batch_pairs = kDefaultBatchPairs;
    if (!c.si_slots) c.si_slots = kDefaultSlots;
    if (!c.max_graphs) c.max_graphs = kDefaultMaxGraphs;
    if (c.si_slots > kMaxSlots || c.max_batch_pairs > (1u << 26) || c.max_graphs > (1u << 16))
        return RTG_ERR_INVALID_ARG;
    rtg_server *s = new rtg_server();
    s->device = device;
    s->cfg = c;
    s->held = (c.flags & RTG_SERVE_START_HELD) != 0;
    auto bail = [&](rtg_status st) {
        rtg_serve_stop(s);
        return st;
    };
    rtg_status st;
    if ((st = rtg_init(device, &s->build)) != RTG_OK) return bail(st);
    if ((st = rtg_init(device, &s->tcx)) != RTG_OK) return bail(st);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return bail(RTG_ERR_DEVICE);
    s->st.budget_bytes = c.hbm_budget_bytes ? c.hbm_budget_bytes : (uint64_t)(free_b * 0.9);
    if (cudaMallocHost((void **)&s->h_tab, sizeof(SetRef) * c.max_graphs) != cudaSuccess)
        return bail(RTG_ERR_OOM);
    memset(s->h_tab, 0, sizeof(SetRef) * c.max_graphs);
    s->graphs.resize(c.max_graphs);
    s->slots.resize(c.si_slots);
    const uint64_t cap = c.max_batch_pairs;
    for (SiSlot &sl : s->slots) {
        if ((st = rtg_init(device, &sl.ctx)) != RTG_OK) return bail(st);
        if ((st = dev_alloc(sl.ctx, (void **)&sl.d_pairs, cap * 12 + 16)) != RTG_OK) return bail(st);
        if ((st = dev_alloc(sl.ctx, (void **)&sl.d_out, cap * 4 + 16)) != RTG_OK) return bail(st);
        if ((st = dev_alloc(sl.ctx, (void **)&sl.d_tab, sizeof(SetRef) * c.max_graphs)) != RTG_OK)
            return bail(st);
        if (cudaMallocHost((void **)&sl.h_pairs, cap * 12 + 16) != cudaSuccess ||
            cudaMallocHost((void **)&sl.h_out, cap * 4 + 16) != cudaSuccess ||
            cudaMallocHost((void **)&sl.h_status, 64) != cudaSuccess ||
            cudaMallocHost((void **)&sl.h_tab, sizeof(SetRef) * c.max_graphs) != cudaSuccess)
            return bail(RTG_ERR_OOM);
        if (cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess)
            return bail(RTG_ERR_DEVICE);
        s->buffers += cap * 16 + 32 + sizeof(SetRef) * c.max_graphs;
    }
    s->runs.resize(kTcRuns);
    for (uint32_t i = 0; i < kTcRuns; ++i) {
        TcRun &r = s->runs[i];
        r.slot = i;
        if ((st = rtg_init(device, &r.ctx)) != RTG_OK) return bail(st);
        if (cudaMallocHost((void **)&r.h_total, 64) != cudaSuccess) return bail(RTG_ERR_OOM);
        if (cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming) != cudaSuccess)
            return bail(RTG_ERR_DEVICE);
    }
    if (used_bytes(s) > s->st.budget_bytes) return bail(RTG_ERR_OOM);
    s->engine = std::thread(engine_loop, s);
    *out = s;
    return RTG_OK;
}

void rtg_serve_stop(rtg_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->held = false;
        // queued work is cancelled; launches in flight finish
        for (Req *r : s->tc_queue) {
            r->cancelled = true;
            finish(s, r);
        }
        s->tc_queue.clear();
        for (Req *r : s->si_queue) {
            r->cancelled = true;
            r->closed = true;  // nothing more is handed out
            if (r->landed == r->next) finish(s, r);
        }
        s->si_queue.clear();
    }
    s->cv.notify_all();
    if (s->engine.joinable()) s->engine.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &kv : s->active) delete kv.second;
        s->active.clear();
    }
    for (SGraph &g : s->graphs)
        if (g.g) rtg_graph_destroy(g.g);
    for (SiSlot &sl : s->slots) {
        if (sl.ctx) cudaStreamSynchronize(sl.ctx->stream);
        dev_free(sl.d_pairs);
        dev_free(sl.d_out);
        dev_free(sl.d_tab);
        if (sl.h_pairs) cudaFreeHost(sl.h_pairs);
        if (sl.h_out) cudaFreeHost(sl.h_out);
        if (sl.h_status) cudaFreeHost(sl.h_status);
        if (sl.h_tab) cudaFreeHost(sl.h_tab);
        if (sl.done) cudaEventDestroy(sl.done);
        rtg_destroy(sl.ctx);
    }
    for (TcRun &r : s->runs) {
        if (r.ctx) cudaStreamSynchronize(r.ctx->stream);
        dev_free(r.scratch);
        if (r.h_total) cudaFreeHost(r.h_total);
        if (r.done) cudaEventDestroy(r.done);
        rtg_destroy(r.ctx);
    }
    if (s->h_tab) cudaFreeHost(s->h_tab);
    rtg_destroy(s->tcx);
    rtg_destroy(s->build);
    delete s;
}

const char *rtg_serve_last_error(const rtg_server *s) {
    if (!s) return "null server";
    // the engine thread may record a new error at any time: hand out a copy owned by the
    // calling thread (valid until its next call)
    thread_local std::string copy;
    rtg_server *m = const_cast<rtg_server *>(s);
    std::lock_guard<std::mutex> lk(m->err_mu);
    copy = m->last_error;
    return copy.c_str();
}

rtg_status rtg_serve_add_graph(rtg_server *s, const uint32_t *src, const uint32_t *dst,
                               uint64_t m, uint32_t *graph_id) {
    if (!s || !graph_id || (m && (!src || !dst))) return RTG_ERR_INVALID_ARG;
    rtg_graph *g = nullptr;
    {
        std::lock_guard<std::mutex> bl(s->build_mu);
        rtg_status st = rtg_graph_from_host_edges(s->build, src, dst, m, &g);
        if (st != RTG_OK) return srv_fail(s, st, "graph upload: %s", rtg_last_error(s->build));
        if ((st = build_graph(s, g)) != RTG_OK) return st;
    }
    return add_built_graph(s, g, graph_id);
}

rtg_status rtg_serve_add_graph_file(rtg_server *s, const char *path, rtg_format fmt,
                                    uint32_t *graph_id) {
    if (!s || !path || !graph_id) return RTG_ERR_INVALID_ARG;
    rtg_graph *g = nullptr;
    {
        std::lock_guard<std::mutex> bl(s->build_mu);
        rtg_status st = rtg_graph_load(s->build, path, fmt, &g);
        if (st != RTG_OK) return srv_fail(s, st, "graph load: %s", rtg_last_error(s->build));
        if (fmt == RTG_FMT_RTG_CSR) {  // a cached graph is used as it is
            if (!g->cnt.built || !g->sym.built) {
                rtg_graph_destroy(g);
                return srv_fail(s, RTG_ERR_FORMAT,
                                "%s lacks the counting form or the symmetric CSR", path);
            }
        } else if ((st = build_graph(s, g)) != RTG_OK) {
            return st;
        }
    }
    return add_built_graph(s, g, graph_id);
}

rtg_status rtg_serve_save_graph(rtg_server *s, uint32_t graph_id, const char *path) {
    if (!s || !path) return RTG_ERR_INVALID_ARG;
    rtg_graph *g = nullptr;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        SGraph *sg = nullptr;
        RTG_TRY(get_graph(s, graph_id, &sg));
        g = sg->g;
        sg->refs++;  // keeps the graph resident while it is written
    }
    rtg_status st;
    {
        std::lock_guard<std::mutex> bl(s->build_mu);
        st = rtg_graph_save(s->build, g, path);
        if (st != RTG_OK) srv_fail(s, st, "graph save: %s", rtg_last_error(s->build));
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->graphs[graph_id].refs--;
    s->cv.notify_all();
    return st;
}

rtg_status rtg_serve_remove_graph(rtg_server *s, uint32_t graph_id) {
    if (!s) return RTG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    SGraph *g = nullptr;
    RTG_TRY(get_graph(s, graph_id, &g));
    g->removing = true;
    s->cv.notify_all();
    return RTG_OK;
}

rtg_status rtg_serve_graph_info(rtg_server *s, uint32_t graph_id, rtg_graph_info *info) {
    if (!s || !info) return RTG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    SGraph *g = nullptr;
    RTG_TRY(get_graph(s, graph_id, &g));
    *info = g->info;
    return RTG_OK;
}

rtg_status rtg_serve_submit_tc(rtg_server *s, uint32_t graph_id, uint64_t *request_id) {
    if (!s || !request_id) return RTG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return srv_fail(s, RTG_ERR_STATE, "server is stopping");
    SGraph *g = nullptr;
    RTG_TRY(get_graph(s, graph_id, &g));
    Req *r = new Req();
    r->id = s->next_id++;
    r->kind = RTG_REQ_TC;
    r->graph = graph_id;
    r->t_submit = Clock::now();
    g->refs++;
    s->active[r->id] = r;
    s->tc_queue.push_back(r);
    s->st.submitted++;
    *request_id = r->id;
    s->cv.notify_all();
    return RTG_OK;
}

rtg_status rtg_serve_submit_pairs(rtg_server *s, uint32_t graph_id, const uint32_t *u,
                                  const uint32_t *v, uint64_t npairs, uint32_t *out_counts,
                                  uint64_t *request_id) {
    if (!s || !request_id || (npairs && (!u || !v || !out_counts))) return RTG_ERR_INVALID_ARG;
    uint32_t n = 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        SGraph *g = nullptr;
        RTG_TRY(get_graph(s, graph_id, &g));
        n = g->n_sym;
    }
    // ids are checked here, on the caller's thread, so a bad request fails alone
    uint32_t bad = 0;
    for (uint64_t i = 0; i < npairs; ++i) bad |= (u[i] >= n) | (v[i] >= n);
    if (bad) return srv_fail(s, RTG_ERR_INVALID_ARG, "pair vertex id out of range (n = %u)", n);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stopping) return srv_fail(s, RTG_ERR_STATE, "server is stopping");
    SGraph *g = nullptr;
    RTG_TRY(get_graph(s, graph_id, &g));
    Req *r = new Req();
    r->id = s->next_id++;
    r->kind = RTG_REQ_PAIRS;
    r->graph = graph_id;
    r->u = u;
    r->v = v;
    r->out = out_counts;
    r->np = npairs;
    r->t_submit = Clock::now();
    g->refs++;
    s->active[r->id] = r;
    s->st.submitted++;
    *request_id = r->id;
    if (npairs == 0) {
        finish(s, r);
        return RTG_OK;
    }
    s->si_queue.push_back(r);
    s->cv.notify_all();
    return RTG_OK;
}

rtg_status rtg_serve_poll(rtg_server *s, uint64_t request_id, int32_t wait_ms,
                          rtg_request_info *info) {
    if (!s || !info) return RTG_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (!s->done.count(request_id) && !s->active.count(request_id))
        return srv_fail(s, RTG_ERR_INVALID_ARG, "unknown request %llu",
                        (unsigned long long)request_id);
    RTG_TRY(wait_for(s, lk, wait_ms, [&] { return s->done.count(request_id) != 0; }));
    *info = s->done[request_id];
    s->done.erase(request_id);
    return RTG_OK;
}

rtg_status rtg_serve_wait_any(rtg_server *s, int32_t wait_ms, uint64_t *request_id,
                              rtg_request_info *info) {
    if (!s || !request_id || !info) return RTG_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto ready = [&] {
        while (!s->done_order.empty() && !s->done.count(s->done_order.front()))
            s->done_order.pop_front();  // already collected by rtg_serve_poll
        return !s->done_order.empty();
    };
    RTG_TRY(wait_for(s, lk, wait_ms, ready));
    const uint64_t id = s->done_order.front();
    s->done_order.pop_front();
    *request_id = id;
    *info = s->done[id];
    s->done.erase(id);
    return RTG_OK;
}

rtg_status rtg_serve_cancel(rtg_server *s, uint64_t request_id) {
    if (!s) return RTG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->active.find(request_id);
    if (it == s->active.end()) {
        if (s->done.count(request_id)) return RTG_OK;  // already complete
        return srv_fail(s, RTG_ERR_INVALID_ARG, "unknown request %llu",
                        (unsigned long long)request_id);
    }
    Req *r = it->second;
    r->cancelled = true;
    if (r->kind == RTG_REQ_TC) {
        auto qi = std::find(s->tc_queue.begin(), s->tc_queue.end(), r);
        if (qi != s->tc_queue.end()) {  // not launched yet
            s->tc_queue.erase(qi);
            finish(s, r);
        }
        return RTG_OK;  // a running count completes (cancelled) with its launch
    }
    r->closed = true;
    auto qi = std::find(s->si_queue.begin(), s->si_queue.end(), r);
    if (qi != s->si_queue.end()) s->si_queue.erase(qi);
    if (r->landed == r->next) finish(s, r);  // no launch of it in flight
    return RTG_OK;
}

rtg_status rtg_serve_release(rtg_server *s) {
    if (!s) return RTG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->held = false;
    s->cv.notify_all();
    return RTG_OK;
}

rtg_status rtg_serve_drain(rtg_server *s, int32_t wait_ms) {
    if (!s) return RTG_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    return wait_for(s, lk, wait_ms, [&] { return s->active.empty(); });
}

rtg_status rtg_serve_stats_get(rtg_server *s, rtg_serve_stats *st) {
    if (!s || !st) return RTG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *st = s->st;
    st->resident_bytes = s->resident;
    st->plan_bytes = s->plans;
    st->buffer_bytes = s->buffers;
    return RTG_OK;
}

}  // extern "C"
