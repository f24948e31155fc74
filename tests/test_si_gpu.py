"""Set-intersection parity on the GPU, through the C ABI.

Known answers from the reference's own generator files, per-pair parity with the oracle on
seeded workloads, every kernel family, edge cases, and the full batched configuration
(10^6 pairs) against the generator's exact per-pair overlap.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
import rtg
from conftest import GOLDEN, si_golden, tc_golden, golden_edges

pytestmark = pytest.mark.gpu
SI = si_golden()
FAMILIES = (rtg.SI_AUTO, rtg.SI_MERGE, rtg.SI_SEARCH, rtg.SI_BITMAP, rtg.SI_PLAIN)


@pytest.mark.parametrize("family", FAMILIES)
@pytest.mark.parametrize("name", sorted(SI))
def test_reference_dataset_files(ctx, name, family):
    info, off, el = rtg.dataset_read(str(GOLDEN / "si" / f"{name}.s_data"))
    sets = ctx.sets(off, el)
    na, nb = info.num_a, info.num_b
    got, t = sets.count_dense(0, na, na, na + nb, family)
    assert got.shape == (na * nb,)
    assert (got == info.intersection).all()


def _random_sets(rng, nsets, max_len, universe):
    lens = rng.integers(0, max_len + 1, nsets)
    lens[rng.random(nsets) < 0.05] = 0
    off = np.zeros(nsets + 1, np.uint64)
    off[1:] = np.cumsum(lens)
    el = np.empty(int(off[-1]), np.uint32)
    for i, L in enumerate(lens):
        el[off[i]:off[i + 1]] = np.sort(rng.choice(universe, size=L, replace=False))
    return off, el


@pytest.mark.parametrize("family", FAMILIES)
def test_random_pairs_match_oracle(ctx, family):
    rng = np.random.default_rng(11)
    off, el = _random_sets(rng, 400, 300, 2000)
    sets = ctx.sets(off, el)
    pa = rng.integers(0, 400, 20000).astype(np.uint32)
    pb = rng.integers(0, 400, 20000).astype(np.uint32)
    got, _ = sets.count(pa, pb, family)
    assert np.array_equal(got, oracle.si_pairs(off, el, pa, pb))


@pytest.mark.parametrize("family", FAMILIES)
def test_edge_cases(ctx, family):
    big = np.arange(0, 2 * 65536, 2, dtype=np.uint32)          # 65,536 elements
    lists = [
        np.array([], np.uint32), np.array([0], np.uint32), np.array([0xFFFFFFFE], np.uint32),
        big, big + 1, big[:1], big[-1:], big[::1000], np.arange(31, dtype=np.uint32),
        np.arange(33, dtype=np.uint32), np.arange(64, dtype=np.uint32) * 3,
        np.array([1, 0xFFFFFFFE], np.uint32),
    ]
    off = np.zeros(len(lists) + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in lists])
    el = np.concatenate(lists).astype(np.uint32)
    sets = ctx.sets(off, el)
    k = len(lists)
    pa, pb = np.meshgrid(np.arange(k, dtype=np.uint32), np.arange(k, dtype=np.uint32))
    pa, pb = pa.ravel(), pb.ravel()
    got, _ = sets.count(pa, pb, family)
    assert np.array_equal(got, oracle.si_pairs(off, el, pa, pb))
    dense, _ = sets.count_dense(0, k, 0, k, family)
    assert np.array_equal(dense, oracle.si_dense(off, el, 0, k, 0, k))


def test_bad_inputs_rejected(ctx):
    off = np.array([0, 2, 3], np.uint64)
    with pytest.raises(rtg.RtgError) as e:
        ctx.sets(off, np.array([1, 0xFFFFFFFF, 3], np.uint32))
    assert e.value.status == rtg.ERR_INVALID_ARG
    sets = ctx.sets(off, np.array([1, 2, 3], np.uint32))
    with pytest.raises(rtg.RtgError) as e:
        sets.count(np.array([0, 5], np.uint32), np.array([1, 1], np.uint32))
    assert e.value.status == rtg.ERR_INVALID_ARG
    got, _ = sets.count(np.array([0], np.uint32), np.array([1], np.uint32))
    assert got.tolist() == [0]


@pytest.mark.parametrize("family", FAMILIES)
def test_generated_workload_known_answers(ctx, family):
    off, el, pa, pb, exp = rtg.gen_si_pairs(20000, seed=5)
    sets = ctx.sets(off, el)
    got, _ = sets.count(pa, pb, family)
    assert np.array_equal(got, exp)
    assert np.array_equal(got, oracle.si_pairs(off, el, pa, pb))


@pytest.mark.parametrize("cfg", [
    dict(si_stage_bytes=512), dict(si_stage_bytes=512, si_stage_slots=2, si_block_warps=1),
    dict(si_stage_bytes=1024, si_stage_slots=16, si_block_warps=2),
    dict(si_stage_bytes=32768, si_stage_slots=2, si_block_warps=1), dict(si_blocks_per_sm=1),
    # search ratio 1: nearly every pair searched (in the slot or in global memory);
    # 1000: nearly every pair merged or chunked
    dict(si_search_ratio=1), dict(si_search_ratio=1000),
    dict(si_search_ratio=2, si_stage_bytes=1024, si_stage_slots=3),
    # skewed pairs staged and streamed (short list in the slot, long list in 16-byte loads)
    dict(si_skew_stream=1), dict(si_skew_stream=1, si_search_ratio=2),
    dict(si_skew_stream=1, si_stage_bytes=1024, si_stage_slots=3),
    # the per-warp ring form named explicitly, then the producer/consumer form: its default,
    # tiny slots (many chunk jobs whose counts meet in the block's accumulators), fewer ring
    # slots than merging warps, long rings, one block per SM, every pair searched or merged,
    # skewed pairs streamed
    dict(si_form=1), dict(si_form=2), dict(si_form=2, si_stage_bytes=512),
    dict(si_form=2, si_stage_bytes=512, si_stage_slots=2, si_block_warps=1),
    dict(si_form=2, si_stage_slots=2, si_block_warps=8),
    dict(si_form=2, si_stage_bytes=1024, si_stage_slots=32, si_block_warps=2),
    dict(si_form=2, si_blocks_per_sm=1), dict(si_form=2, si_search_ratio=1),
    dict(si_form=2, si_search_ratio=1000), dict(si_form=2, si_skew_stream=1),
    dict(si_form=2, si_skew_stream=1, si_stage_bytes=1024, si_stage_slots=3),
])
def test_batched_schedules_agree(ctx, cfg):
    """Small staging slots cut most pairs into many chunk pairs; results must not change."""
    old = ctx.config()
    try:
        ctx.set_config(**cfg)
        off, el, pa, pb, exp = rtg.gen_si_pairs(20000, seed=9)
        got, _ = ctx.sets(off, el).count(pa, pb, rtg.SI_AUTO)
        assert np.array_equal(got, exp)
        big = np.arange(0, 2 * 65536, 2, dtype=np.uint32)
        lists = [big, big[::3], big[5:9000], np.array([big[-1]], np.uint32), big + 1]
        o2 = np.zeros(len(lists) + 1, np.uint64)
        o2[1:] = np.cumsum([len(x) for x in lists])
        e2 = np.concatenate(lists).astype(np.uint32)
        k = len(lists)
        dense, _ = ctx.sets(o2, e2).count_dense(0, k, 0, k, rtg.SI_AUTO)
        assert np.array_equal(dense, oracle.si_dense(o2, e2, 0, k, 0, k))
    finally:
        ctx.set_config(**old.as_dict())


@pytest.mark.parametrize("form,slot_bytes", [(1, 0), (2, 4096), (2, 0)])
def test_slot_and_ratio_boundaries(ctx, form, slot_bytes):
    """4 KB staging slots (the per-warp form's default; 1024 words for both widened lists
    and their sentinels; search ratio 8) in both kernel forms, and the producer/consumer
    form's own default: pairs whose words land just under, on and just over one slot, for
    every 16-byte alignment of either list's start, and pairs on either side of |B| = 8 |A|
    both inside one slot and beyond it. Counts agree with the oracle."""
    rng = np.random.default_rng(17)
    lists = []
    for pad in range(4):  # a list of `pad` elements shifts the next list's alignment
        if pad:
            lists.append(np.sort(rng.choice(1 << 20, pad, replace=False)).astype(np.uint32))
        for n in (500, 503, 504, 505, 506, 507, 508, 509, 510, 511, 512, 513, 1016, 1017):
            lists.append(np.sort(rng.choice(1 << 12, n, replace=False)).astype(np.uint32))
    for a in (40, 200):  # ratio 8 in a slot (40 x 320 / 321), beyond a slot (200 x 1600 / 1601)
        base = np.sort(rng.choice(1 << 16, 8 * a + 1, replace=False)).astype(np.uint32)
        lists += [base[::8][:a].copy(), base[: 8 * a].copy(), base.copy()]
    off = np.zeros(len(lists) + 1, np.uint64)
    off[1:] = np.cumsum([len(x) for x in lists])
    el = np.concatenate(lists).astype(np.uint32)
    k = len(lists)
    pa, pb = np.meshgrid(np.arange(k, dtype=np.uint32), np.arange(k, dtype=np.uint32))
    pa, pb = pa.ravel(), pb.ravel()
    saved = ctx.config().as_dict()
    try:
        ctx.set_config(**dict(saved, si_form=form, si_stage_bytes=slot_bytes))
        got, _ = ctx.sets(off, el).count(pa, pb, rtg.SI_AUTO)
    finally:
        ctx.set_config(**saved)
    assert np.array_equal(got, oracle.si_pairs(off, el, pa, pb))


def test_config3_full_size_known_answers(ctx):
    """10^6 lognormal pairs (median 64, sigma 1.5, lengths in [1, 65536], universe 2^26)."""
    off, el, pa, pb, exp = rtg.gen_si_pairs(1_000_000, seed=1)
    sets = ctx.sets(off, el)
    got, t = sets.count(pa, pb)
    assert np.array_equal(got, exp)
    sample = np.arange(0, 1_000_000, 97)
    assert np.array_equal(got[sample], oracle.si_pairs(off, el, pa[sample], pb[sample]))
    assert t.kernel_launches >= 1


@pytest.mark.parametrize("family", [rtg.SI_AUTO, rtg.SI_PLAIN])
def test_pinned_host_buffers_zero_copy(ctx, family):
    """Page-locked host pair ids and counts: the kernel reads and writes them over the
    host link (no staging copies); counts identical to the pageable path and the oracle."""
    rng = np.random.default_rng(11)
    off, el = _random_sets(rng, 300, 400, 5000)
    sets = ctx.sets(off, el)
    n = 20000
    pa = rng.integers(0, 300, n).astype(np.uint32)
    pb = rng.integers(0, 300, n).astype(np.uint32)
    want = oracle.si_pairs(off, el, pa, pb)
    hpa, hpb, hout = (ctx.host_array(n, np.uint32) for _ in range(3))
    hpa[:] = pa
    hpb[:] = pb
    hout[:] = 0xFFFFFFFF
    _, t = sets.count(hpa, hpb, family, out=hout)
    assert np.array_equal(hout, want)
    assert t.h2d_bytes == 8 * n and t.d2h_bytes == 4 * n and t.h2d_ms == 0 and t.d2h_ms == 0
    got, t2 = sets.count(pa, pb, family)  # pageable: staged copies
    assert np.array_equal(got, want) and t2.h2d_bytes == 8 * n


def test_materialize_matches_oracle(ctx):
    rng = np.random.default_rng(2)
    off, el = _random_sets(rng, 200, 500, 3000)
    sets = ctx.sets(off, el)
    pa = rng.integers(0, 200, 5000).astype(np.uint32)
    pb = rng.integers(0, 200, 5000).astype(np.uint32)
    goff, gel, _ = sets.materialize(pa, pb)
    ooff, oel = oracle.si_materialize(off, el, pa, pb)
    assert np.array_equal(goff, ooff)
    assert np.array_equal(gel, oel)


def test_materialize_skewed_pairs_match_oracle(ctx):
    """Lengths lognormal with sigma 2 (many pairs more than 16x apart, in both orders: the
    write pass searches the short list in the long one) and balanced ones, against the
    oracle's intersections, both pair orders."""
    off, el, pa, pb, exp = rtg.gen_si_pairs(20_000, median=64.0, sigma=2.0, min_len=1,
                                            max_len=65536, universe_log2=26, overlap_max=0.5,
                                            seed=11)
    lens = np.diff(off.astype(np.int64))
    ratio = np.maximum(lens[pa], lens[pb]) / np.maximum(np.minimum(lens[pa], lens[pb]), 1)
    assert (ratio > 16).mean() > 0.1
    sets = ctx.sets(off, el)
    for a, b in ((pa, pb), (pb, pa)):
        goff, gel, _ = sets.materialize(a, b)
        ooff, oel = oracle.si_materialize(off, el, a, b)
        assert np.array_equal(goff, ooff)
        assert np.array_equal(gel, oel)
    assert np.array_equal(np.diff(goff.astype(np.int64)), exp.astype(np.int64))


def test_vertex_pair_queries_on_graph(ctx):
    tc = tc_golden()
    s, d = golden_edges(tc["rmat_s12_ef16_s1"])
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_SYMMETRIC)
    off, adj = g.csr(symmetric=True)
    rng = np.random.default_rng(4)
    n = len(off) - 1
    u = rng.integers(0, n, 30000).astype(np.uint32)
    v = rng.integers(0, n, 30000).astype(np.uint32)
    got, _ = g.pair_count(u, v)
    assert np.array_equal(got, oracle.si_pairs(off, adj, u, v))


@pytest.mark.parametrize("form", [1, 2])
def test_bounded_wait_runs_out_cleanly(ctx, form):
    """A staging-slot wait that cannot complete (the test hook makes one slot expect 16
    bytes more than its copies bring; every copy still lands, nothing stays in flight)
    gives up after a short bound: the call returns RTG_ERR_TIMEOUT, nothing faults or
    hangs, and the next call on the same context is exact."""
    off, el, pa, pb, exp = rtg.gen_si_pairs(20_000, seed=9)
    sets = ctx.sets(off, el)
    out = np.empty(len(pa), np.uint32)
    saved = ctx.config().as_dict()
    try:
        ctx.set_config(**dict(saved, si_form=form))
        assert rtg.lib.rtg_debug_si_wait_limit(ctx.h, 256, 15) == rtg.ERR_INVALID_ARG
        assert rtg.lib.rtg_debug_si_wait_limit(ctx.h, 256, 16) == rtg.OK
        st = rtg.lib.rtg_si_count(ctx.h, sets.h, rtg._ptr(pa), rtg._ptr(pb), len(pa),
                                  rtg._ptr(out), rtg.SI_AUTO, None)
        assert st == rtg.ERR_TIMEOUT
        assert b"bounded device wait" in rtg.lib.rtg_last_error(ctx.h)
        for _ in range(2):  # the hook applied to one launch only; the context stays usable
            got, _ = sets.count(pa, pb, rtg.SI_AUTO)
            assert np.array_equal(got, exp)
    finally:
        ctx.set_config(**saved)
    sets.close()


def test_skewed_pairs_streamed_match_oracle(ctx):
    """Skewed pairs longer than a staging slot, every alignment of the long list and short
    lists from 1 to 128 elements: the staged-and-streamed form (si_skew_stream) against the
    oracle, and against the searched form."""
    rng = np.random.default_rng(21)
    lens = []
    for a in (1, 2, 3, 5, 17, 31, 32, 33, 64, 100, 127, 128):
        for b in (1100, 1101, 1102, 1103, 2000, 4097):
            lens += [a, b]
    off = np.zeros(len(lens) + 1, np.uint64)
    off[1:] = np.cumsum(lens)
    el = np.empty(int(off[-1]), np.uint32)
    for i in range(0, len(lens), 2):
        a, b = lens[i], lens[i + 1]
        B = np.sort(rng.choice(1 << 24, size=b, replace=False)).astype(np.uint32)
        k = int(rng.integers(0, a + 1))
        A = np.concatenate([rng.choice(B, size=k, replace=False),
                            rng.choice(np.setdiff1d(np.arange(1 << 24, (1 << 24) + 4 * a), B),
                                       size=a - k, replace=False)])
        el[off[i]:off[i + 1]] = np.sort(A)
        el[off[i + 1]:off[i + 2]] = B
    pa = np.arange(0, len(lens), 2, dtype=np.uint32)
    pb = pa + 1
    sets = ctx.sets(off, el)
    want = oracle.si_pairs(off, el, pa, pb)
    saved = ctx.config().as_dict()
    try:
        for form in (1, 2):
            for stream in (0, 1):
                ctx.set_config(**dict(saved, si_skew_stream=stream, si_form=form))
                got, _ = sets.count(pa, pb, rtg.SI_AUTO)
                assert np.array_equal(got, want), (form, stream)
                got, _ = sets.count(pb, pa, rtg.SI_AUTO)
                assert np.array_equal(got, want), (form, stream)
    finally:
        ctx.set_config(**saved)
    sets.close()


@pytest.mark.parametrize("cfg", [dict(), dict(si_form=2, si_stage_bytes=512, si_stage_slots=3),
                                 dict(si_form=1, si_stage_bytes=1024)])
def test_batched_counts_repeat_exactly(ctx, cfg):
    """The batched forms hand out jobs dynamically (queue, tickets) and add chunk counts with
    atomics, so which warp does what changes from run to run; the counts must not: ten runs
    of the same pairs, every one equal to the generator's known answers."""
    off, el, pa, pb, exp = rtg.gen_si_pairs(20_000, seed=13)
    sets = ctx.sets(off, el)
    saved = ctx.config().as_dict()
    try:
        ctx.set_config(**dict(saved, **cfg))
        for _ in range(10):
            got, _ = sets.count(pa, pb, rtg.SI_AUTO)
            assert np.array_equal(got, exp)
    finally:
        ctx.set_config(**saved)
    sets.close()
