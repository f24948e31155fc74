"""The dense-core stage of the batched triangle count, through the C ABI.

The top K ranks of the counting form are counted as word ANDs of their adjacency bit
matrix and the remaining in-edges are streamed; the sum must equal the golden count for
every core size, from a single rank to the whole graph, in the BATCHED (plan + CUDA graph),
BUCKETED and one-shot (caller scratch) paths. The library's own choice (the largest
candidate core of at least 2.5 % edge density) is checked on graphs far from that bar:
R-MAT scale 20 (top 16384 ranks 3.6 % dense, top 24576 2.1 %) and Holme-Kim 2^20 (no
core above 1.5 %).
"""
from __future__ import annotations

from math import comb

import numpy as np
import pytest

import oracle
import rtg
from conftest import golden_edges, tc_golden

pytestmark = pytest.mark.gpu
TC = tc_golden()
GRAPHS = ("rmat_s14_ef16_s42", "hk_n20000_m6_p0.9_s3", "rmat_s10_ef8_s5_skewed")
SIZES = (1, 2, 31, 32, 33, 100, 1000, 4096, 8192, 32768, rtg.TC_CORE_NONE)


class core_config:
    def __init__(self, ctx, **cfg):
        self.ctx, self.cfg = ctx, cfg

    def __enter__(self):
        self.saved = self.ctx.config().as_dict()
        self.ctx.set_config(**dict(self.saved, **self.cfg))

    def __exit__(self, *a):
        self.ctx.set_config(**self.saved)


@pytest.mark.parametrize("K", SIZES)
def test_forced_core_sizes_agree(ctx, K):
    for name in GRAPHS:
        rec = TC[name]
        s, d = golden_edges(rec)
        g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
        n = g.info().n
        want_k = 0 if K == rtg.TC_CORE_NONE else min(K, n)
        with core_config(ctx, tc_core_ranks=K):
            for mode in (rtg.TC_BATCHED, rtg.TC_BUCKETED):
                got, t = g.tc(mode)
                assert got == rec["triangles"], (name, K, mode)
                assert t.core_ranks == want_k, (name, K, mode)
                assert (t.core_ms > 0) == (want_k > 0)
            got, _ = ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)
            assert got == rec["triangles"], (name, K, "one-shot")
            off, adj = g.csr()
            got, _ = ctx.tc_count_host_csr(off.astype(np.int32), adj.astype(np.int32),
                                           rtg.TC_BATCHED)
            assert got == rec["triangles"], (name, K, "host CSR")
        g.close()


@pytest.mark.parametrize("n,K", [(3, 3), (33, 1), (33, 33), (65, 17), (200, 200), (200, 64)])
def test_cliques_with_core(ctx, n, K):
    s, d = zip(*[(i, j) for i in range(n) for j in range(i + 1, n)])
    g = ctx.graph_from_edges(np.array(s), np.array(d)).build(rtg.ORIENT_DEGREE)
    with core_config(ctx, tc_core_ranks=K):
        for mode in (rtg.TC_BATCHED, rtg.TC_BUCKETED):
            got, t = g.tc(mode)
            assert got == comb(n, 3)
            assert t.core_ranks == min(K, n)
    g.close()


def test_dense_random_graph_whole_core(ctx):
    """Out-degrees above the per-warp hash capacity, counted entirely as bit rows."""
    rng = np.random.default_rng(3)
    n = 3000
    s, d = np.triu_indices(n, 1)
    keep = rng.random(len(s)) < 0.5
    s, d = s[keep].astype(np.uint32), d[keep].astype(np.uint32)
    off, adj = oracle.degree_csr(s, d)
    want = oracle.tc_merge(off, adj)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    for K in (n, 1024, 0):
        with core_config(ctx, tc_core_ranks=K):
            for mode in (rtg.TC_BATCHED, rtg.TC_BUCKETED):
                got, t = g.tc(mode)
                assert got == want, (K, mode)
                if K:
                    assert t.core_ranks == K
    g.close()


def test_library_choice(ctx):
    s, d = rtg.gen_rmat(20, 16, 0.57, 0.19, 0.19, seed=42)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj = g.csr()
    want = oracle.tc_merge(off, adj)
    with core_config(ctx, tc_core_ranks=0):
        got, t = g.tc(rtg.TC_BATCHED)
        assert (got, t.core_ranks) == (want, 16384)
        got, t = g.tc(rtg.TC_BUCKETED)
        assert (got, t.core_ranks) == (want, 16384)
        got, _ = ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)
        assert got == want
    with core_config(ctx, tc_core_ranks=rtg.TC_CORE_NONE):
        got, t = g.tc(rtg.TC_BATCHED)
        assert (got, t.core_ranks, t.core_ms) == (want, 0, 0.0)
    g.close()
    s, d = rtg.gen_hk(1 << 20, 8, 0.5, seed=1)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    with core_config(ctx, tc_core_ranks=0):
        got, t = g.tc(rtg.TC_BATCHED)
        assert t.core_ranks == 0
        assert got == g.tc(rtg.TC_PLAIN)[0]
    g.close()


def test_core_config_validation(ctx):
    for bad in (32769, 1 << 20, 0xFFFFFFFE):
        with pytest.raises(rtg.RtgError) as e:
            ctx.set_config(**dict(ctx.config().as_dict(), tc_core_ranks=bad))
        assert e.value.status == rtg.ERR_INVALID_ARG
    for good in (0, 1, 32768, rtg.TC_CORE_NONE):
        saved = ctx.config().as_dict()
        ctx.set_config(**dict(saved, tc_core_ranks=good))
        ctx.set_config(**saved)


def test_plan_follows_core_setting(ctx):
    """A plan is rebuilt when the core setting changes, and replays its own choice."""
    rec = TC["rmat_s14_ef16_s42"]
    s, d = golden_edges(rec)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    seen = []
    for K in (512, rtg.TC_CORE_NONE, 2048, 512):
        with core_config(ctx, tc_core_ranks=K):
            for _ in range(3):
                got, t = g.tc(rtg.TC_BATCHED)
                assert got == rec["triangles"]
                seen.append(t.core_ranks)
    assert seen == [512] * 3 + [0] * 3 + [2048] * 3 + [512] * 3
    g.close()


def test_loaded_graph_keeps_the_core(ctx, tmp_path):
    """A graph read back from its cache file picks the same core (from the file's offsets)
    and counts the same, resident and with a forced core."""
    s, d = rtg.gen_rmat(16, 16, 0.57, 0.19, 0.19, seed=8)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    want, t = g.tc(rtg.TC_BATCHED)
    assert t.core_ranks > 0
    path = tmp_path / "g.rtgcsr"
    g.save(str(path))
    h = ctx.graph_load(str(path), rtg.FMT_RTG_CSR)
    got, t2 = h.tc(rtg.TC_BATCHED)
    assert (got, t2.core_ranks) == (want, t.core_ranks)
    with core_config(ctx, tc_core_ranks=3000):
        assert h.tc(rtg.TC_BATCHED)[0] == want
        assert h.tc(rtg.TC_BUCKETED)[0] == want
    h.close()
    g.close()
