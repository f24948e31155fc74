"""Autotuner: every schedule it keeps gives the default schedule's exact result, the winner
is set on the context, and a cached winner is applied without a search."""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import rtg

pytestmark = pytest.mark.gpu


def test_tune_tc_keeps_exact_count_and_caches(tmp_path):
    cache = str(tmp_path / "tune.txt")
    s, d = rtg.gen_rmat(14, 16, seed=3)
    off, adj = oracle.degree_csr(s, d)
    want = oracle.tc_merge(off, adj)
    with rtg.Context(0) as ctx:
        g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
        r = g.tune(cache)
        # 36 schedules, then up to 3 dense-core sizes on the best of them
        assert not r["from_cache"] and 37 <= r["candidates"] <= 39
        assert r["rejected"] < r["candidates"]
        assert r["best_ms"] <= r["default_ms"]
        assert ctx.config().as_dict()["tc_item_edges"] == r["best"]["tc_item_edges"]
        assert g.tc(rtg.TC_BATCHED)[0] == want
        r2 = g.tune(cache)
        assert r2["from_cache"] and r2["best"] == r["best"]
        assert g.tc(rtg.TC_BATCHED)[0] == want


def test_tune_si_keeps_exact_counts_and_caches(tmp_path):
    cache = str(tmp_path / "tune.txt")
    off, el, pa, pb, exp = rtg.gen_si_pairs(20_000, seed=4)
    with rtg.Context(0) as ctx:
        sets = ctx.sets(off, el)
        r = sets.tune(pa, pb, cache)
        # 108 per-warp ring schedules, 72 producer/consumer ones, then the best one with
        # skewed pairs staged and streamed
        assert not r["from_cache"] and r["candidates"] == 181
        assert r["best_ms"] <= r["default_ms"]
        got, _ = sets.count(pa, pb, rtg.SI_AUTO)
        assert np.array_equal(got, exp)
        r2 = sets.tune(pa, pb, cache)
        assert r2["from_cache"] and r2["best"] == r["best"]
        got, _ = sets.count(pa, pb, rtg.SI_AUTO)
        assert np.array_equal(got, exp)
