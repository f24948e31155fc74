"""The CPU oracle against golden vectors produced by the reference's own code.

tests/golden/tc_golden.json holds the CSR and triangle count that the reference's
tc/graph/graph.cpp preprocessing and tc/bs_tc/bs_tc.cu two-hop counting produced for each
input; tests/golden/si/*.s_data are files written by the reference's SI data generator
whose every A x B pair intersects in exactly `intersection` elements.
"""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, edges_sha, golden_edges, sha_i32, si_golden, tc_golden

TC = tc_golden()
SI = si_golden()


@pytest.mark.parametrize("name", sorted(n for n in TC if "edges_sha256" in TC[n]))
def test_generator_inputs_unchanged(name):
    """Records made from librtg's seeded generators: the generator still gives the same
    edge list (inline records carry their edges)."""
    rec = TC[name]
    s, d = golden_edges(rec)
    assert len(s) == rec["m_input"]
    assert edges_sha(s, d) == rec["edges_sha256"]


@pytest.mark.parametrize("name", sorted(TC))
def test_reference_csr_matches_golden(name):
    rec = TC[name]
    s, d = golden_edges(rec)
    pairs = np.stack([s.astype(np.int32), d.astype(np.int32)], axis=1)
    n, e, off, adj = oracle.reference_csr(pairs)
    assert (n, e) == (rec["nodes"], rec["edges"])
    if "offsets" in rec:
        assert off.tolist() == rec["offsets"]
        assert adj.tolist() == rec["adjs"]
    assert sha_i32(off) == rec["offsets_sha256"]
    assert sha_i32(adj) == rec["adjs_sha256"]


@pytest.mark.parametrize("name", sorted(TC))
def test_reference_counts_match_golden(name):
    rec = TC[name]
    s, d = golden_edges(rec)
    pairs = np.stack([s.astype(np.int32), d.astype(np.int32)], axis=1)
    _, _, off, adj = oracle.reference_csr(pairs)
    assert oracle.tc_bsearch_i32(off, adj) == rec["triangles"]
    assert oracle.tc_hashmap_i32(off, adj) == rec["triangles"]
    assert oracle.tc_merge(off.astype(np.uint64), adj.astype(np.uint32)) == rec["triangles"]


@pytest.mark.parametrize("name", sorted(TC))
def test_degree_orientation_total_matches_golden(name):
    """Post-dedup orientation gives a different DAG but the same total."""
    rec = TC[name]
    s, d = golden_edges(rec)
    off, adj = oracle.degree_csr(s, d)
    assert oracle.tc_merge(off, adj) == rec["triangles"]
    # every row sorted, oriented edges unique and the simple edge count preserved
    sym_off, sym_adj = oracle.symmetric_csr(s, d)
    assert len(adj) * 2 == len(sym_adj)


@pytest.mark.parametrize("name", sorted(SI))
def test_si_reference_files_known_answer(name):
    import rtg
    rec = SI[name]
    path = GOLDEN / "si" / f"{name}.s_data"
    assert hashlib.sha256(path.read_bytes()).hexdigest() == rec["sha256"]
    info, off, el = rtg.dataset_read(str(path))
    assert (info.num_a, info.num_b, info.intersection) == (rec["num_a"], rec["num_b"],
                                                           rec["intersection"])
    off64 = off.astype(np.uint64)
    na, nb = info.num_a, info.num_b
    dense = oracle.si_dense(off64, el, 0, na, na, na + nb)
    assert dense.shape == (na * nb,)
    assert (dense == info.intersection).all()
    for a in range(min(na, 3)):
        for b in range(na, na + nb):
            A = el[off[a]:off[a + 1]]
            B = el[off[b]:off[b + 1]]
            assert oracle.si_bsearch(A, B) == info.intersection
            assert oracle.si_bsearch(B, A) == info.intersection
            assert oracle.si_merge(A, B) == info.intersection


def test_si_oracle_edge_cases():
    e = np.array([], np.uint32)
    one = np.array([7], np.uint32)
    assert oracle.si_merge(e, e) == 0
    assert oracle.si_merge(one, e) == 0
    assert oracle.si_merge(one, one) == 1
    big = np.arange(0, 65536 * 2, 2, dtype=np.uint32)
    odd = big + 1
    assert oracle.si_merge(big, big) == 65536
    assert oracle.si_merge(big, odd) == 0
    assert oracle.si_bsearch(one, big[:10]) == 0
    assert oracle.si_bsearch(np.array([8], np.uint32), big) == 1


def test_tc_oracle_closed_forms():
    from math import comb
    for n in (3, 4, 7, 12):
        s, d = zip(*[(i, j) for i in range(n) for j in range(i + 1, n)])
        off, adj = oracle.degree_csr(np.array(s), np.array(d))
        assert oracle.tc_merge(off, adj) == comb(n, 3)
    # a tree has none
    s = np.arange(1, 100, dtype=np.uint32)
    d = (s - 1) // 2
    off, adj = oracle.degree_csr(s, d.astype(np.uint32))
    assert oracle.tc_merge(off, adj) == 0


@pytest.mark.parametrize("scale,seed", [(8, 1), (12, 42), (14, 7)])
def test_oracle_rmat_generator_matches_library(scale, seed):
    """The reference arm of the benchmark makes its R-MAT input with the oracle's
    generator: it must give the library generator's edge list, bit for bit."""
    import rtg
    s0, d0 = rtg.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed=seed)
    s1, d1 = oracle.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed=seed)
    assert np.array_equal(s0, s1) and np.array_equal(d0, d1)


def test_oracle_si_generator_matches_library():
    import rtg
    a = rtg.gen_si_pairs(3000, seed=11)
    b = oracle.gen_si_pairs(3000, seed=11)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    off, el, pa, pb, exp = b
    assert np.array_equal(oracle.si_pairs(off, el, pa, pb), exp)
