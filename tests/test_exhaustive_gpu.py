"""Exhaustive tiny cases against closed-form answers, through the C ABI.

Triangle counting: every labelled graph on 6 vertices (2^15 edge subsets of K6), placed
side by side as one disjoint union (graph i on vertices 6i .. 6i+5), counted in every form
and both orientations; its per-edge triangle lists (which keep vertex ids under the degree
orientation) give each small graph's own count back, which must equal the number of
vertex triples whose three edges are all present.

Set intersection: every pair of subsets of {0, ..., 7} (256 x 256 pairs) in the dense
row-major order; |A ∩ B| is the popcount of the AND of the two subsets' bit masks. Every
kernel form and family, and the batched forms with small staging slots.
"""
from __future__ import annotations

import itertools

import numpy as np
import pytest

import rtg

pytestmark = pytest.mark.gpu

K6 = list(itertools.combinations(range(6), 2))          # the 15 edges of K6
TRIPLES = list(itertools.combinations(range(6), 3))     # the 20 vertex triples


def _all_six_vertex_graphs():
    masks = np.arange(1 << len(K6), dtype=np.int64)
    present = ((masks[:, None] >> np.arange(len(K6))) & 1).astype(bool)  # [graph, edge]
    eidx = {e: i for i, e in enumerate(K6)}
    tri = np.zeros(len(masks), np.int64)
    for a, b, c in TRIPLES:
        tri += present[:, eidx[(a, b)]] & present[:, eidx[(a, c)]] & present[:, eidx[(b, c)]]
    g, e = np.nonzero(present)
    ends = np.array(K6, np.int64)[e]
    s = (6 * g + ends[:, 0]).astype(np.uint32)
    d = (6 * g + ends[:, 1]).astype(np.uint32)
    return s, d, tri


@pytest.fixture(scope="module")
def six():
    return _all_six_vertex_graphs()


@pytest.mark.parametrize("orient", [rtg.ORIENT_DEGREE, rtg.ORIENT_DEGREE_RAW_REF])
@pytest.mark.parametrize("core", [0, 7, 32768, rtg.TC_CORE_NONE])
def test_every_six_vertex_graph_total(ctx, six, orient, core):
    """core: the dense-core size of the batched forms (a core of 7 or 32768 top ranks cuts
    through small graphs, so their triangles are split between the core count and the
    streamed in-edges)."""
    s, d, tri = six
    g = ctx.graph_from_edges(s, d).build(orient)
    saved = ctx.config().as_dict()
    try:
        ctx.set_config(**dict(saved, tc_core_ranks=core))
        for mode in (rtg.TC_PLAIN, rtg.TC_BATCHED, rtg.TC_BUCKETED):
            got, _ = g.tc(mode)
            assert got == int(tri.sum()), mode
        got, _ = ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)
        assert got == int(tri.sum())
        off, adj = g.csr()  # the host-CSR entry, batched: the CSR's edges as a one-shot list
        got, _ = ctx.tc_count_host_csr(off.astype(np.int32), adj.astype(np.int32),
                                       rtg.TC_BATCHED)
        assert got == int(tri.sum())
    finally:
        ctx.set_config(**saved)
    g.close()


def test_every_six_vertex_graph_on_its_own(ctx, six):
    """Per graph: the triangle lists of the union's edges, summed over each small graph's
    edges (vertex ids are kept under the degree orientation, so edge (u, v) belongs to
    graph u // 6)."""
    s, d, tri = six
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj = g.csr()
    loff, w, _ = g.tc_list()
    src = np.repeat(np.arange(len(off) - 1), np.diff(off.astype(np.int64)))
    per_edge = np.diff(loff.astype(np.int64))
    per_graph = np.bincount(src // 6, weights=per_edge, minlength=len(tri)).astype(np.int64)
    assert np.array_equal(per_graph, tri)
    # every listed third vertex lies in the same small graph as its edge
    third_graph = w.astype(np.int64) // 6
    assert np.array_equal(third_graph, np.repeat(src // 6, per_edge))
    g.close()


@pytest.fixture(scope="module")
def subsets():
    lists = [np.array([x for x in range(8) if (m >> x) & 1], np.uint32) for m in range(256)]
    off = np.zeros(257, np.uint64)
    off[1:] = np.cumsum([len(x) for x in lists])
    el = np.concatenate(lists).astype(np.uint32)
    m = np.arange(256)
    want = np.array([bin(x).count("1") for x in range(256)], np.uint32)[m[:, None] & m[None, :]]
    return off, el, want.ravel()


@pytest.mark.parametrize("family", [rtg.SI_AUTO, rtg.SI_MERGE, rtg.SI_SEARCH, rtg.SI_BITMAP,
                                    rtg.SI_PLAIN])
def test_every_pair_of_subsets_of_eight(ctx, subsets, family):
    off, el, want = subsets
    got, _ = ctx.sets(off, el).count_dense(0, 256, 0, 256, family)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("cfg", [dict(si_form=1), dict(si_form=2),
                                 dict(si_form=1, si_stage_bytes=512, si_stage_slots=2),
                                 dict(si_form=2, si_stage_bytes=512, si_stage_slots=2,
                                      si_block_warps=8),
                                 dict(si_form=2, si_search_ratio=1)])
def test_every_pair_of_subsets_batched_schedules(ctx, subsets, cfg):
    off, el, want = subsets
    saved = ctx.config().as_dict()
    try:
        ctx.set_config(**dict(saved, **cfg))
        got, _ = ctx.sets(off, el).count_dense(0, 256, 0, 256, rtg.SI_AUTO)
    finally:
        ctx.set_config(**saved)
    assert np.array_equal(got, want)
