"""Triangle-counting parity on the GPU, through the C ABI.

Bit-exact against the reference-produced golden vectors (CSR and count) and against the
oracle; at full configuration sizes through the oracle merge counter and structural
properties of the GPU-built CSR.
"""
from __future__ import annotations

from math import comb

import numpy as np
import pytest

import oracle
import rtg
from conftest import golden_edges, sha_i32, tc_golden

pytestmark = pytest.mark.gpu
TC = tc_golden()
MODES = (rtg.TC_PLAIN, rtg.TC_BATCHED, rtg.TC_BUCKETED)


@pytest.mark.parametrize("name", sorted(TC))
def test_reference_mode_csr_and_count_bit_exact(ctx, name):
    rec = TC[name]
    s, d = golden_edges(rec)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE_RAW_REF)
    info = g.info()
    assert (info.n, info.m) == (rec["nodes"], rec["edges"])
    off, adj = g.csr()
    assert sha_i32(off) == rec["offsets_sha256"]
    assert sha_i32(adj) == rec["adjs_sha256"]
    for mode in MODES:
        assert g.tc(mode)[0] == rec["triangles"]


@pytest.mark.parametrize("name", sorted(TC))
def test_degree_mode_csr_matches_oracle(ctx, name):
    rec = TC[name]
    s, d = golden_edges(rec)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj = g.csr()
    ooff, oadj = oracle.degree_csr(s, d)
    assert np.array_equal(off, ooff)
    assert np.array_equal(adj, oadj)
    for mode in MODES:
        assert g.tc(mode)[0] == rec["triangles"]


@pytest.mark.parametrize("name", sorted(TC))
def test_host_pairs_entry_matches_golden(ctx, name):
    """rtg_graph_from_host_pairs: the reference's edge_t layout (int32 {src, dst} pairs,
    tc/utils/model.h:16-29) in, the reference's CSR and count out."""
    rec = TC[name]
    s, d = golden_edges(rec)
    pairs = np.stack([s.astype(np.int32), d.astype(np.int32)], axis=1)
    g = ctx.graph_from_pairs(pairs).build(rtg.ORIENT_DEGREE_RAW_REF)
    assert g.info().m_input == len(s)
    off, adj = g.csr()
    assert sha_i32(off) == rec["offsets_sha256"]
    assert sha_i32(adj) == rec["adjs_sha256"]
    assert g.tc(rtg.TC_BATCHED)[0] == rec["triangles"]


@pytest.mark.parametrize("name", sorted(TC))
def test_symmetric_csr_matches_oracle(ctx, name):
    s, d = golden_edges(TC[name])
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_SYMMETRIC)
    off, adj = g.csr(symmetric=True)
    ooff, oadj = oracle.symmetric_csr(s, d)
    assert np.array_equal(off, ooff)
    assert np.array_equal(adj, oadj)


def test_empty_and_tiny(ctx):
    for s, d in [([], []), ([0], [1]), ([3], [3]), ([0, 1], [1, 0])]:
        s = np.array(s, np.uint32)
        d = np.array(d, np.uint32)
        for orient in (rtg.ORIENT_DEGREE, rtg.ORIENT_DEGREE_RAW_REF):
            g = ctx.graph_from_edges(s, d).build(orient)
            for mode in MODES:
                assert g.tc(mode)[0] == 0


@pytest.mark.parametrize("n", [3, 4, 33, 65, 200])
def test_cliques_closed_form(ctx, n):
    s, d = zip(*[(i, j) for i in range(n) for j in range(i + 1, n)])
    g = ctx.graph_from_edges(np.array(s), np.array(d)).build(rtg.ORIENT_DEGREE)
    for mode in MODES:
        assert g.tc(mode)[0] == comb(n, 3)


@pytest.mark.parametrize("cfg", [
    dict(tc_item_edges=1), dict(tc_item_edges=7), dict(tc_item_edges=1024),
    dict(tc_region_words=64), dict(tc_region_words=256),
    dict(tc_region_words=8192, tc_block_warps=4), dict(tc_region_words=16384, tc_block_warps=2),
    dict(tc_block_warps=1), dict(tc_block_warps=16, tc_region_words=1024),
    dict(tc_blocks_per_sm=1), dict(tc_item_edges=3, tc_region_words=128),
])
def test_batched_schedules_agree(ctx, cfg):
    old = ctx.config()
    try:
        ctx.set_config(**cfg)
        for name in ("rmat_s14_ef16_s42", "hk_n20000_m6_p0.9_s3", "rmat_s10_ef8_s5_skewed"):
            rec = TC[name]
            s, d = golden_edges(rec)
            g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
            assert g.tc(rtg.TC_BATCHED)[0] == rec["triangles"], (name, cfg)
    finally:
        ctx.set_config(**old.as_dict())


def test_hub_heavy_graph_uses_merge_fallback(ctx):
    # a dense core makes out-degrees exceed the per-warp hash capacity
    rng = np.random.default_rng(3)
    n = 3000
    s, d = np.triu_indices(n, 1)
    keep = rng.random(len(s)) < 0.5
    s, d = s[keep].astype(np.uint32), d[keep].astype(np.uint32)
    off, adj = oracle.degree_csr(s, d)
    want = oracle.tc_merge(off, adj)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    assert g.info().max_out_degree > 1024
    for mode in MODES:
        assert g.tc(mode)[0] == want


def test_repeatable(ctx):
    s, d = golden_edges(TC["rmat_s14_ef16_s42"])
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    got = {g.tc(rtg.TC_BATCHED)[0] for _ in range(10)} | {g.tc(rtg.TC_PLAIN)[0] for _ in range(3)}
    assert got == {TC["rmat_s14_ef16_s42"]["triangles"]}


def test_drop_in_host_csr_and_host_edges(ctx):
    for name in ("k4_noise", "ba_n4096_m4_s7", "rmat_s12_ef16_s1"):
        rec = TC[name]
        s, d = golden_edges(rec)
        pairs = np.stack([s.astype(np.int32), d.astype(np.int32)], axis=1)
        _, _, off, adj = oracle.reference_csr(pairs)
        for mode in MODES:
            got, t = ctx.tc_count_host_csr(off, adj, mode)
            assert got == rec["triangles"]
            got, t = ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE_RAW_REF, mode)
            assert got == rec["triangles"]
            assert t.h2d_bytes == 8 * len(s) and t.kernel_launches > 0


@pytest.mark.parametrize("name", sorted(TC))
def test_host_csr_batched_all_golden(ctx, name):
    """rtg_tc_count_host_csr (the reference's CountOnGPU entry) in the batched form counts
    the CSR's edges like a one-shot edge list; the golden count on every golden graph."""
    rec = TC[name]
    s, d = golden_edges(rec)
    pairs = np.stack([s.astype(np.int32), d.astype(np.int32)], axis=1)
    _, _, off, adj = oracle.reference_csr(pairs)
    got, t = ctx.tc_count_host_csr(off, adj, rtg.TC_BATCHED)
    assert got == rec["triangles"]
    assert t.h2d_bytes == 4 * (len(off) + len(adj))


def test_host_csr_batched_refuses_bad_csrs(ctx):
    off = np.array([0, 2, 3, 3], np.int32)
    for adj in (np.array([2, 1, 2], np.int32),      # row 0 not ascending
                np.array([1, 3, 2], np.int32),      # id past the vertices
                np.array([1, -1, 2], np.int32)):    # negative id
        with pytest.raises(rtg.RtgError) as e:
            ctx.tc_count_host_csr(off, adj, rtg.TC_BATCHED)
        assert e.value.status == rtg.ERR_INVALID_ARG
    with pytest.raises(rtg.RtgError) as e:           # offsets not ending at the edges
        ctx.tc_count_host_csr(np.array([0, 2, 3, 4], np.int32), np.array([1, 2, 2], np.int32),
                              rtg.TC_BATCHED)
    assert e.value.status == rtg.ERR_INVALID_ARG
    # the context still counts afterwards
    got, _ = ctx.tc_count_host_csr(off, np.array([1, 2, 2], np.int32), rtg.TC_BATCHED)
    assert got == 1


@pytest.mark.parametrize("name", sorted(TC))
def test_one_shot_host_edges_all_golden(ctx, name):
    """rtg_tc_count_host_edges with the degree orientation: the batched form builds the
    counting form straight from the edges; both forms give the reference's count."""
    rec = TC[name]
    s, d = golden_edges(rec)
    for mode in MODES:
        got, t = ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE, mode)
        assert got == rec["triangles"], (name, mode)


@pytest.mark.parametrize("name", ["k4_noise", "ba_n4096_m4_s7", "rmat_s12_ef16_s1",
                                  "rmat_s14_ef16_s42"])
def test_triangle_lists_match_oracle(ctx, name):
    """rtg_tc_list: per-edge lists N+(u) ∩ N+(v) over the oriented CSR, bit-exact against the
    oracle's per-pair merge; the lists hold exactly the reference's triangle count, and
    every listed (u, v, w) is a triangle of the simple undirected graph."""
    rec = TC[name]
    s, d = golden_edges(rec)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj = g.csr()
    n = len(off) - 1
    src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(off.astype(np.int64)))
    loff, w, t = g.tc_list()
    assert int(loff[-1]) == rec["triangles"] and len(w) == rec["triangles"]
    ooff, ow = oracle.si_materialize(off, adj, src, adj)
    assert np.array_equal(loff, ooff)
    assert np.array_equal(w, ow)
    e = np.repeat(np.arange(len(adj)), np.diff(loff.astype(np.int64)))
    u, v, x = src[e].astype(np.int64), adj[e].astype(np.int64), w.astype(np.int64)
    a, b = np.minimum(s, d).astype(np.int64), np.maximum(s, d).astype(np.int64)
    keys = np.unique(a[a != b] * (1 << 32) + b[a != b])

    def has(p, q):
        k = np.minimum(p, q) * (1 << 32) + np.maximum(p, q)
        return np.isin(k, keys)

    assert has(u, v).all() and has(u, x).all() and has(v, x).all()
    assert len(np.unique((np.sort(np.stack([u, v, x]), axis=0) * [[1 << 42], [1 << 21], [1]]).sum(0))) == len(w)


@pytest.mark.parametrize("scale", [16, 18])
def test_triangle_lists_large_staged(ctx, scale):
    """Lists large enough that their copy to pageable host memory goes through the
    page-locked staging buffers (R-MAT 16: 60 MB in chunks of an eighth; R-MAT 18: 316 MB in
    32 MB chunks, the last one partial): bit-exact against the oracle's per-pair merge."""
    s, d = rtg.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed=5)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj = g.csr()
    n = len(off) - 1
    src = np.repeat(np.arange(n, dtype=np.uint32), np.diff(off.astype(np.int64)))
    loff, w, t = g.tc_list()
    assert len(w) * 4 >= 16 << 20
    ooff, ow = oracle.si_materialize(off, adj, src, adj)
    assert np.array_equal(loff, ooff)
    assert np.array_equal(w, ow)
    assert int(loff[-1]) == g.tc(rtg.TC_BATCHED)[0]


def test_triangle_lists_capacity_and_state(ctx):
    rec = TC["rmat_s12_ef16_s1"]
    s, d = golden_edges(rec)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    m = g.info().m
    off = np.empty(m + 1, np.uint64)
    w = np.empty(8, np.uint32)
    st = rtg.lib.rtg_tc_list(ctx.h, g.h, rtg._ptr(off), rtg._ptr(w), 8, None)
    assert st == rtg.ERR_INVALID_ARG and int(off[-1]) == rec["triangles"]
    loff, lw, _ = g.tc_list(capacity=rec["triangles"])
    assert int(loff[-1]) == rec["triangles"]
    raw = ctx.graph_from_edges(s, d)  # no CSR built yet
    assert rtg.lib.rtg_tc_list(ctx.h, raw.h, rtg._ptr(off), None, 0, None) == rtg.ERR_STATE


def test_one_shot_pinned_edges_pulled(ctx):
    """Page-locked host edges: one kernel pulls them over the host link and counts the
    ranking degrees on the way (exact below 2^22 edges, sampled above). First call (no
    degree counters yet), repeat (counters reused), a larger graph after a smaller one
    (counters too small: counted again), and an edge count that is not a multiple of 4."""
    for scale, trim in ((17, 0), (20, 0), (18, 3), (20, 1)):
        s, d = rtg.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed=3)
        if trim:
            s, d = s[:-trim], d[:-trim]
        want = oracle.tc_merge(*oracle.degree_csr(s, d))
        hs = ctx.host_array(len(s), np.uint32)
        hd = ctx.host_array(len(d), np.uint32)
        hs[:] = s
        hd[:] = d
        for _ in range(2):
            got, t = ctx.tc_count_host_edges(hs, hd, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)
            assert got == want, (scale, trim)
            assert t.h2d_bytes == 8 * len(s)


def test_one_shot_degenerate_edge_lists(ctx):
    """rtg_tc_count_host_edges on lists whose rows come out empty or tiny: no edges, only
    self loops (their pairs are the only ones left after the copies go), only copies of one
    edge, and small cliques buried in copies, reversed copies and self loops."""
    tri = [(0, 1), (1, 2), (2, 0)]
    k4 = [(i, j) for i in range(4) for j in range(i + 1, 4)]
    cases = [
        ([], 0), ([(5, 5)], 0), ([(1, 1), (2, 2), (3, 3)], 0), ([(0, 1)] * 10, 0),
        (tri * 3 + [(b, a) for a, b in tri] + [(0, 0), (2, 2)], 1),
        (k4 * 2 + [(7, 7)] + [(b, a) for a, b in k4], 4),
        ([(9, 3), (3, 9), (9, 3)] + [(3 + i, 3 + j) for i, j in k4], 4),
    ]
    for edges, want in cases:
        s = np.array([a for a, _ in edges], np.uint32)
        d = np.array([b for _, b in edges], np.uint32)
        for mode in MODES:
            got, _ = ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE, mode)
            assert got == want, (edges, mode)


@pytest.mark.parametrize("row", [32, 33, 2048, 2049, 5000])
def test_one_shot_long_raw_rows(ctx, row):
    """One-shot build on raw rows (edge copies included) of 32, 33, 2048, 2049 and 5000
    entries, around the warp, block and sort-pass sizes: vertex 0 gets exactly `row` raw
    entries (repeated edges to 60 hubs of a clique whose leaves give them higher degrees);
    a second vertex adds 700 copies of edges to 20 of the hubs. Pageable and page-locked
    edges; counts agree with the oracle on the deduplicated graph."""
    rng = np.random.default_rng(row)
    hubs = np.arange(1, 61, dtype=np.uint32)
    iu, ju = np.triu_indices(len(hubs), 1)
    s = [hubs[iu], np.zeros(row, np.uint32), np.full(700, 100, np.uint32)]
    d = [hubs[ju], rng.choice(hubs, row).astype(np.uint32),
         rng.choice(hubs[:20], 700).astype(np.uint32)]
    leaves = np.arange(1000, 1000 + len(hubs) * (row + 5), dtype=np.uint32)
    s.append(np.repeat(hubs, row + 5))
    d.append(leaves)
    s, d = np.concatenate(s), np.concatenate(d)
    perm = rng.permutation(len(s))
    s, d = s[perm], d[perm]
    flip = rng.random(len(s)) < 0.5
    s, d = np.where(flip, d, s).astype(np.uint32), np.where(flip, s, d).astype(np.uint32)
    off, adj = oracle.degree_csr(s, d)
    want = oracle.tc_merge(off, adj)
    hs = ctx.host_array(len(s), np.uint32)
    hd = ctx.host_array(len(d), np.uint32)
    hs[:] = s
    hd[:] = d
    for src, dst in ((s, d), (hs, hd)):
        got, _ = ctx.tc_count_host_edges(src, dst, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)
        assert got == want, row


def test_file_formats(ctx, tmp_path):
    rec = TC["wheel"]
    s, d = golden_edges(rec)
    rtg.edges_write_bin(str(tmp_path / "g.edge"), s, d)
    (tmp_path / "g.txt").write_text("# comment\n" + "".join(f"{a} {b}\n" for a, b in zip(s, d)))
    lines = ["%%MatrixMarket matrix coordinate pattern symmetric", "% c",
             f"{int(max(s.max(), d.max())) + 1} {int(max(s.max(), d.max())) + 1} {len(s)}"]
    lines += [f"{a + 1} {b + 1}" for a, b in zip(s, d)]
    (tmp_path / "g.mtx").write_text("\n".join(lines) + "\n")
    for path, fmt in (("g.edge", rtg.FMT_EDGE_BIN), ("g.txt", rtg.FMT_EDGE_TXT),
                      ("g.mtx", rtg.FMT_MTX)):
        g = ctx.graph_load(str(tmp_path / path), fmt).build(rtg.ORIENT_DEGREE)
        assert g.tc()[0] == rec["triangles"]


def test_errors_are_status_codes(ctx):
    with pytest.raises(rtg.RtgError) as e:
        ctx.graph_from_edges(np.array([0xFFFFFFFF], np.uint32),
                             np.array([1], np.uint32)).build(rtg.ORIENT_DEGREE)
    assert e.value.status == rtg.ERR_INVALID_ARG
    g = ctx.graph_from_edges(np.array([0, 1], np.uint32), np.array([1, 2], np.uint32))
    with pytest.raises(rtg.RtgError) as e:
        g.tc()
    assert e.value.status == rtg.ERR_STATE
    with pytest.raises(rtg.RtgError) as e:   # unsorted row
        ctx.graph_from_csr(np.array([0, 2, 2, 2], np.int32), np.array([2, 1], np.int32))
    assert e.value.status == rtg.ERR_INVALID_ARG
    # one-shot count: ids of 2^31 - 1 and above are refused before anything is sized by them
    for big in (0x7FFFFFFF, 0x80000000, 0xFFFFFFFE, 0xFFFFFFFF):
        with pytest.raises(rtg.RtgError) as e:
            ctx.tc_count_host_edges(np.array([0, 1], np.uint32), np.array([1, big], np.uint32),
                                    rtg.ORIENT_DEGREE, rtg.TC_BATCHED)
        assert e.value.status == rtg.ERR_INVALID_ARG
    # the context is still usable after errors
    assert ctx.graph_from_edges(np.array([0, 1, 2], np.uint32),
                                np.array([1, 2, 0], np.uint32)).build().tc()[0] == 1
    s, d = np.array([0, 1, 2], np.uint32), np.array([1, 2, 0], np.uint32)
    assert ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)[0] == 1


def test_config2_holme_kim_full_size(ctx):
    """Holme-Kim n=2^20, m=16, p=0.3 (~16.7M edges): GPU vs oracle merge counter."""
    s, d = rtg.gen_hk(1 << 20, 16, 0.3, seed=1)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj = g.csr()
    want = oracle.tc_merge(off, adj)
    assert g.tc(rtg.TC_PLAIN)[0] == want
    assert g.tc(rtg.TC_BATCHED)[0] == want
    # the reference-mode CSR gives the same total
    g2 = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE_RAW_REF)
    assert g2.tc(rtg.TC_BATCHED)[0] == want


def _check_oriented_csr(off, adj):
    deg_out = np.diff(off.astype(np.int64))
    n = len(off) - 1
    src = np.repeat(np.arange(n, dtype=np.int64), deg_out)
    # rows strictly ascending
    same = src[1:] == src[:-1]
    assert (adj[1:][same] > adj[:-1][same]).all()
    # no self loops; total degree order respected (an acyclic orientation)
    assert (src != adj).all()
    deg = np.bincount(src, minlength=n) + np.bincount(adj, minlength=n)
    a = deg[src] * (n + 1) + src
    b = deg[adj] * (n + 1) + adj
    assert (a < b).all()


def test_config4_rmat21_full_size(ctx):
    """R-MAT scale 21, ef 16: PLAIN == BATCHED == oracle merge count; CSR checked; the
    batched and one-shot counts also without a dense core and with cores of 4096 and 32768
    top ranks (the library picks 24576 here)."""
    s, d = rtg.gen_rmat(21, 16, 0.57, 0.19, 0.19, seed=42)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj = g.csr()
    _check_oriented_csr(off, adj)
    want = oracle.tc_merge(off, adj)
    got, t = g.tc(rtg.TC_BATCHED)
    assert (got, t.core_ranks) == (want, 24576)
    assert g.tc(rtg.TC_PLAIN)[0] == want
    saved = ctx.config().as_dict()
    try:
        for K in (rtg.TC_CORE_NONE, 4096, 32768):
            ctx.set_config(**dict(saved, tc_core_ranks=K))
            got, t = g.tc(rtg.TC_BATCHED)
            assert (got, t.core_ranks) == (want, 0 if K == rtg.TC_CORE_NONE else K)
            assert ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)[0] == want
    finally:
        ctx.set_config(**saved)
