"""Serving: the request loop over resident graphs (rtg_serve_*).

Every result is an exact integer, so "the same alone and in the mix" means bit-identical:
triangle totals and per-pair |N(u) ∩ N(v)| counts are compared with the oracle and with
the same requests served one at a time. Failure paths are driven from the host (a
cancelled request, an out-of-range id, an over-budget graph, a malformed file, a launch
reported failed by the injection hook); none of them faults the GPU.
"""
from __future__ import annotations

import threading

import numpy as np
import pytest

import oracle
import rtg

pytestmark = pytest.mark.gpu

SCALES = [8, 9, 10, 11, 12, 13]


@pytest.fixture(scope="module")
def graphs():
    out = []
    for i, sc in enumerate(SCALES):
        s, d = rtg.gen_rmat(sc, 16, seed=100 + i)
        off, adj = oracle.degree_csr(s, d)
        soff, sadj = oracle.symmetric_csr(s, d)
        out.append(dict(s=s, d=d, tri=oracle.tc_merge(off, adj), soff=soff, sadj=sadj,
                        n=len(soff) - 1))
    return out


def make_requests(graphs, count, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(count):
        g = int(rng.integers(len(graphs)))
        if rng.random() < 0.25:
            reqs.append(("tc", g, None, None))
        else:
            k = int(rng.integers(1, 20000))
            n = graphs[g]["n"]
            reqs.append(("pairs", g, rng.integers(0, n, k, dtype=np.uint32),
                         rng.integers(0, n, k, dtype=np.uint32)))
    return reqs


def expected(graphs, req):
    kind, g, u, v = req
    if kind == "tc":
        return graphs[g]["tri"]
    return oracle.si_pairs(graphs[g]["soff"], graphs[g]["sadj"], u, v)


def serve_one_by_one(srv, gids, reqs):
    res = []
    for kind, g, u, v in reqs:
        if kind == "tc":
            info = srv.poll(srv.submit_tc(gids[g]))
            assert info["status"] == rtg.OK
            res.append(info["triangles"])
        else:
            rid, out = srv.submit_pairs(gids[g], u, v)
            info = srv.poll(rid)
            assert info["status"] == rtg.OK
            res.append(out.copy())
    return res


def add_all(srv, graphs):
    return [srv.add_graph(g["s"], g["d"]) for g in graphs]


def test_results_same_alone_and_in_the_mix(graphs):
    reqs = make_requests(graphs, 60, seed=7)
    want = [expected(graphs, r) for r in reqs]
    with rtg.Server(0) as srv:
        gids = add_all(srv, graphs)
        alone = serve_one_by_one(srv, gids, reqs)
    for a, w in zip(alone, want):
        assert np.array_equal(np.asarray(a), np.asarray(w))
    # the mix: everything queued while the engine is held, then released at once, so
    # pair requests of different graphs and sizes share launches and TC counts overlap them
    with rtg.Server(0, held=True, max_batch_pairs=1 << 16) as srv:
        gids = add_all(srv, graphs)
        ids, outs = [], []
        for kind, g, u, v in reqs:
            if kind == "tc":
                ids.append(srv.submit_tc(gids[g]))
                outs.append(None)
            else:
                rid, out = srv.submit_pairs(gids[g], u, v)
                ids.append(rid)
                outs.append(out)
        srv.release()
        infos = [srv.poll(i) for i in ids]
        st = srv.stats()
    for info, out, a, (kind, *_r) in zip(infos, outs, alone, reqs):
        assert info["status"] == rtg.OK
        got = info["triangles"] if kind == "tc" else out
        assert np.array_equal(np.asarray(got), np.asarray(a))
    assert st["max_requests_per_launch"] > 1
    assert st["max_inflight_launches"] >= 2
    assert st["tc_coalesced"] > 0  # several waiting TC requests of one graph, one launch
    assert st["completed"] == len(reqs)


def test_concurrent_submitters(graphs):
    reqs = make_requests(graphs, 80, seed=11)
    want = [expected(graphs, r) for r in reqs]
    with rtg.Server(0, max_batch_pairs=1 << 15) as srv:
        gids = add_all(srv, graphs)
        got = [None] * len(reqs)
        errors = []

        def worker(idx):
            try:
                for i in idx:
                    kind, g, u, v = reqs[i]
                    if kind == "tc":
                        got[i] = srv.poll(srv.submit_tc(gids[g]))["triangles"]
                    else:
                        rid, out = srv.submit_pairs(gids[g], u, v)
                        assert srv.poll(rid)["status"] == rtg.OK
                        got[i] = out
            except Exception as e:  # surfaced below
                errors.append(e)

        ts = [threading.Thread(target=worker, args=(range(k, len(reqs), 4),)) for k in range(4)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        assert not errors, errors
    for a, w in zip(got, want):
        assert np.array_equal(np.asarray(a), np.asarray(w))


def test_large_request_split_across_launches(graphs):
    g = graphs[-1]
    rng = np.random.default_rng(3)
    u = rng.integers(0, g["n"], 50_000, dtype=np.uint32)
    v = rng.integers(0, g["n"], 50_000, dtype=np.uint32)
    with rtg.Server(0, max_batch_pairs=4096, si_slots=3) as srv:
        gid = srv.add_graph(g["s"], g["d"])
        rid, out = srv.submit_pairs(gid, u, v)
        info = srv.poll(rid)
    assert info["status"] == rtg.OK and info["launches"] >= 13
    assert np.array_equal(out, oracle.si_pairs(g["soff"], g["sadj"], u, v))


def test_budget_admission_and_plan_eviction(graphs):
    # the counting plans as the library sizes them: one count of each graph without a budget
    with rtg.Server(0) as srv:
        gids = add_all(srv, graphs[:3])
        st = srv.stats()
        sizes, before = [], st["plan_bytes"]
        for gid in gids:
            assert srv.poll(srv.submit_tc(gid))["status"] == rtg.OK
            after = srv.stats()["plan_bytes"]
            sizes.append(after - before)
            before = after
    base = st["resident_bytes"] + st["buffer_bytes"]
    plan = max(sizes)
    assert min(sizes) > 0
    # room for the three graphs and one counting plan, not two
    with rtg.Server(0, budget_bytes=base + plan + plan // 2) as srv:
        gids = add_all(srv, graphs[:3])
        with pytest.raises(rtg.RtgError) as e:
            srv.add_graph(graphs[3]["s"], graphs[3]["d"])
        assert e.value.status == rtg.ERR_OOM
        for rep in range(3):
            for k, gid in enumerate(gids):
                info = srv.poll(srv.submit_tc(gid))
                assert info["status"] == rtg.OK
                assert info["triangles"] == graphs[k]["tri"]
        st = srv.stats()
    assert st["plan_evictions"] > 0
    assert st["tc_direct"] > 0  # counted in run scratch when no plan fit
    assert st["resident_graphs"] == 3


def test_cancel_remove_and_invalid_requests(graphs, tmp_path):
    g = graphs[2]
    rng = np.random.default_rng(5)
    u = rng.integers(0, g["n"], 3000, dtype=np.uint32)
    v = rng.integers(0, g["n"], 3000, dtype=np.uint32)
    with rtg.Server(0, held=True) as srv:
        gid = srv.add_graph(g["s"], g["d"])
        other = srv.add_graph(graphs[0]["s"], graphs[0]["d"])
        a, out_a = srv.submit_pairs(gid, u, v)
        b, out_b = srv.submit_pairs(gid, v, u)
        c = srv.submit_tc(gid)
        t = srv.submit_tc(other)
        srv.cancel(b)
        srv.cancel(t)
        assert srv.poll(b, 0)["status"] == rtg.ERR_CANCELLED
        assert srv.poll(t, 0)["status"] == rtg.ERR_CANCELLED
        # out-of-range ids and unknown graphs fail at submission, alone
        bad = u.copy()
        bad[17] = g["n"]
        with pytest.raises(rtg.RtgError) as e:
            srv.submit_pairs(gid, bad, v)
        assert e.value.status == rtg.ERR_INVALID_ARG
        with pytest.raises(rtg.RtgError) as e:
            srv.submit_tc(999)
        assert e.value.status == rtg.ERR_INVALID_ARG
        # removal waits for the graph's queued requests; new ones are refused at once
        srv.remove_graph(gid)
        with pytest.raises(rtg.RtgError):
            srv.submit_tc(gid)
        assert srv.poll(a, 0) is None  # still held
        srv.release()
        ia, ic = srv.poll(a), srv.poll(c)
        assert ia["status"] == rtg.OK and ic["status"] == rtg.OK
        assert np.array_equal(out_a, oracle.si_pairs(g["soff"], g["sadj"], u, v))
        assert ic["triangles"] == g["tri"]
        srv.drain()
        for _ in range(200):
            if srv.stats()["resident_graphs"] == 1:
                break
            threading.Event().wait(0.01)
        assert srv.stats()["resident_graphs"] == 1
        # malformed graph file
        p = tmp_path / "bad.edge"
        p.write_bytes(b"\x01\x02\x03")
        with pytest.raises(rtg.RtgError):
            srv.add_graph_file(str(p))
        # the server still serves
        info = srv.poll(srv.submit_tc(other))
        assert info["status"] == rtg.OK and info["triangles"] == graphs[0]["tri"]


def test_injected_launch_failure_is_contained(graphs):
    g = graphs[1]
    rng = np.random.default_rng(9)
    u = rng.integers(0, g["n"], 2000, dtype=np.uint32)
    v = rng.integers(0, g["n"], 2000, dtype=np.uint32)
    with rtg.Server(0, inject_fail_launch=1) as srv:
        gid = srv.add_graph(g["s"], g["d"])
        r1, _ = srv.submit_pairs(gid, u, v)
        assert srv.poll(r1)["status"] == rtg.ERR_DEVICE
        r2, out2 = srv.submit_pairs(gid, u, v)
        assert srv.poll(r2)["status"] == rtg.OK
        assert np.array_equal(out2, oracle.si_pairs(g["soff"], g["sadj"], u, v))
        st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 1


def test_stop_with_work_queued(graphs):
    g = graphs[0]
    u = np.arange(100, dtype=np.uint32) % g["n"]
    srv = rtg.Server(0, held=True)
    gid = srv.add_graph(g["s"], g["d"])
    srv.submit_pairs(gid, u, u)
    srv.submit_tc(gid)
    srv.close()  # queued requests are cancelled, nothing is left running
