"""CPU oracle — TEST INFRASTRUCTURE ONLY.

ctypes binding of oracle/rtg_oracle.c, a plain-C restatement of RT-Graph's reference
algorithms for triangle counting and set intersection (each C function cites the reference
file:line it follows). Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
use it, and only as the checker or the timed CPU baseline; librtg never calls it.

Parity is pinned against golden vectors produced by the reference's own code
(tests/golden/, made by tests/golden/make_golden.py with oracle/build_ref.sh).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"


def _load():
    src = HERE / "rtg_oracle.c"
    stale = (not LIB_PATH.exists() or
             max(src.stat().st_mtime, (HERE / "rtg_oracle.h").stat().st_mtime)
             > LIB_PATH.stat().st_mtime)
    if stale:
        import subprocess
        LIB_PATH.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp", "-std=c11",
                        str(HERE / "rtg_oracle.c"), "-o", str(LIB_PATH), "-lm"], check=True)
    lib = C.CDLL(str(LIB_PATH))
    P = C.c_void_p
    sig = {
        "orc_compact_ids": (C.c_int64, [P, C.c_int64]),
        "orc_tc_preprocess_ref": (C.c_int, [P, C.c_int64, C.c_int32, P, P, P, P]),
        "orc_csr_degree": (C.c_int, [P, P, C.c_uint64, C.c_uint32, P, P, P]),
        "orc_csr_symmetric": (C.c_int, [P, P, C.c_uint64, C.c_uint32, P, P, P]),
        "orc_tc_bsearch_i32": (C.c_uint64, [P, P, C.c_int32, C.c_int]),
        "orc_tc_hashmap_i32": (C.c_uint64, [P, P, C.c_int32, C.c_int]),
        "orc_tc_bsearch_rows": (C.c_uint64, [P, P, P, C.c_int64, C.c_int]),
        "orc_tc_merge": (C.c_uint64, [P, P, C.c_uint32, C.c_int]),
        "orc_si_merge": (C.c_uint32, [P, C.c_uint32, P, C.c_uint32]),
        "orc_si_bsearch": (C.c_uint32, [P, C.c_uint32, P, C.c_uint32]),
        "orc_si_pairs": (None, [P, P, P, P, C.c_uint64, P, C.c_int]),
        "orc_si_dense": (None, [P, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, P, C.c_int]),
        "orc_si_materialize": (C.c_uint64, [P, P, P, P, C.c_uint64, P, P, C.c_uint64]),
        "orc_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                   C.c_uint64, P, P, C.c_int]),
        "orc_gen_si_lengths": (C.c_int, [C.c_uint64, C.c_double, C.c_double, C.c_uint32,
                                         C.c_uint32, C.c_uint64, P, P, C.c_int]),
        "orc_gen_si_lists": (C.c_int, [C.c_uint64, C.c_uint32, C.c_double, C.c_uint64, P, P, P,
                                       P, C.c_int]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype = r
        f.argtypes = a
    return lib


lib = _load()


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def reference_csr(pairs: np.ndarray):
    """Graph::ReadBinaryEdges compaction + TCPreprocessing + ConvertToCSR on int32 pairs.
    Returns (nodes, edges, offsets int32[nodes+1], adjs int32[edges])."""
    p = np.array(pairs, dtype=np.int32).reshape(-1, 2).copy()
    m = len(p)
    nodes = lib.orc_compact_ids(_p(p), m)
    off = np.zeros(max(nodes, 0) + 1, np.int32)
    adj = np.zeros(max(m, 1), np.int32)
    on, oe = C.c_int32(0), C.c_int64(0)
    rc = lib.orc_tc_preprocess_ref(_p(p), m, int(nodes), _p(off), _p(adj), C.byref(on), C.byref(oe))
    assert rc == 0
    return on.value, oe.value, off[: on.value + 1].copy(), adj[: oe.value].copy()


def degree_csr(s: np.ndarray, d: np.ndarray, n: int | None = None):
    s = np.ascontiguousarray(s, np.uint32)
    d = np.ascontiguousarray(d, np.uint32)
    if n is None:
        n = int(max(s.max(initial=0), d.max(initial=0))) + 1 if len(s) else 0
    off = np.zeros(n + 1, np.uint64)
    adj = np.zeros(max(len(s), 1), np.uint32)
    mo = C.c_uint64(0)
    assert lib.orc_csr_degree(_p(s), _p(d), len(s), n, _p(off), _p(adj), C.byref(mo)) == 0
    return off, adj[: mo.value].copy()


def symmetric_csr(s: np.ndarray, d: np.ndarray, n: int | None = None):
    s = np.ascontiguousarray(s, np.uint32)
    d = np.ascontiguousarray(d, np.uint32)
    if n is None:
        n = int(max(s.max(initial=0), d.max(initial=0))) + 1 if len(s) else 0
    off = np.zeros(n + 1, np.uint64)
    adj = np.zeros(max(2 * len(s), 1), np.uint32)
    mo = C.c_uint64(0)
    assert lib.orc_csr_symmetric(_p(s), _p(d), len(s), n, _p(off), _p(adj), C.byref(mo)) == 0
    return off, adj[: mo.value].copy()


def tc_merge(off: np.ndarray, adj: np.ndarray, threads: int = 0) -> int:
    off = np.ascontiguousarray(off, np.uint64)
    adj = np.ascontiguousarray(adj, np.uint32)
    return lib.orc_tc_merge(_p(off), _p(adj), len(off) - 1, threads)


def tc_bsearch_i32(off: np.ndarray, adj: np.ndarray, threads: int = 0) -> int:
    off = np.ascontiguousarray(off, np.int32)
    adj = np.ascontiguousarray(adj, np.int32)
    return lib.orc_tc_bsearch_i32(_p(off), _p(adj), len(off) - 1, threads)


def tc_bsearch_rows(off: np.ndarray, adj: np.ndarray, rows: np.ndarray, threads: int = 0) -> int:
    off = np.ascontiguousarray(off, np.int32)
    adj = np.ascontiguousarray(adj, np.int32)
    rows = np.ascontiguousarray(rows, np.int32)
    return lib.orc_tc_bsearch_rows(_p(off), _p(adj), _p(rows), len(rows), threads)


def tc_hashmap_i32(off: np.ndarray, adj: np.ndarray, threads: int = 0) -> int:
    off = np.ascontiguousarray(off, np.int32)
    adj = np.ascontiguousarray(adj, np.int32)
    return lib.orc_tc_hashmap_i32(_p(off), _p(adj), len(off) - 1, threads)


def si_pairs(off, elems, pa, pb, threads: int = 0) -> np.ndarray:
    off = np.ascontiguousarray(off, np.uint64)
    elems = np.ascontiguousarray(elems, np.uint32)
    pa = np.ascontiguousarray(pa, np.uint32)
    pb = np.ascontiguousarray(pb, np.uint32)
    out = np.zeros(max(len(pa), 1), np.uint32)
    lib.orc_si_pairs(_p(off), _p(elems), _p(pa), _p(pb), len(pa), _p(out), threads)
    return out[: len(pa)]


def si_dense(off, elems, a0, a1, b0, b1, threads: int = 0) -> np.ndarray:
    off = np.ascontiguousarray(off, np.uint64)
    elems = np.ascontiguousarray(elems, np.uint32)
    out = np.zeros(max((a1 - a0) * (b1 - b0), 1), np.uint32)
    lib.orc_si_dense(_p(off), _p(elems), a0, a1, b0, b1, _p(out), threads)
    return out[: (a1 - a0) * (b1 - b0)]


def si_merge(a: np.ndarray, b: np.ndarray) -> int:
    a = np.ascontiguousarray(a, np.uint32)
    b = np.ascontiguousarray(b, np.uint32)
    return lib.orc_si_merge(_p(a), len(a), _p(b), len(b))


def si_bsearch(a: np.ndarray, b: np.ndarray) -> int:
    a = np.ascontiguousarray(a, np.uint32)
    b = np.ascontiguousarray(b, np.uint32)
    return lib.orc_si_bsearch(_p(a), len(a), _p(b), len(b))


def si_materialize(off, elems, pa, pb):
    off = np.ascontiguousarray(off, np.uint64)
    elems = np.ascontiguousarray(elems, np.uint32)
    pa = np.ascontiguousarray(pa, np.uint32)
    pb = np.ascontiguousarray(pb, np.uint32)
    oo = np.zeros(len(pa) + 1, np.uint64)
    need = lib.orc_si_materialize(_p(off), _p(elems), _p(pa), _p(pb), len(pa), _p(oo), None, 0)
    el = np.zeros(max(need, 1), np.uint32)
    lib.orc_si_materialize(_p(off), _p(elems), _p(pa), _p(pb), len(pa), _p(oo), _p(el), need)
    return oo, el[:need]


def gen_rmat(scale: int, edge_factor: int = 16, a=0.57, b=0.19, c=0.19, seed: int = 1,
             threads: int = 0):
    """Seeded R-MAT edge list (the same stream as the library's generator)."""
    m = edge_factor << scale
    s = np.empty(m, np.uint32)
    d = np.empty(m, np.uint32)
    if lib.orc_gen_rmat(scale, edge_factor, a, b, c, seed, _p(s), _p(d), threads) != 0:
        raise ValueError("bad R-MAT parameters")
    return s, d


def gen_si_pairs(npairs: int, median=64.0, sigma=1.5, min_len=1, max_len=65536,
                 universe_log2=26, overlap_max=0.5, seed: int = 1, threads: int = 0):
    """Seeded batched-SI workload (the same streams as the library's generator): set
    offsets, elements, pair ids (2i, 2i + 1) and the known overlap of every pair."""
    if 2 * max_len > (1 << universe_log2):
        raise ValueError("max_len too large for the universe")
    lens = np.empty(2 * npairs, np.uint32)
    tot = C.c_uint64(0)
    if lib.orc_gen_si_lengths(npairs, median, sigma, min_len, max_len, seed, _p(lens),
                              C.byref(tot), threads) != 0:
        raise ValueError("bad SI parameters")
    off = np.empty(2 * npairs + 1, np.uint64)
    el = np.empty(tot.value, np.uint32)
    exp = np.empty(npairs, np.uint32)
    if lib.orc_gen_si_lists(npairs, universe_log2, overlap_max, seed, _p(lens), _p(off), _p(el),
                            _p(exp), threads) != 0:
        raise MemoryError("SI generator")
    pa = np.arange(0, 2 * npairs, 2, dtype=np.uint32)
    return off, el, pa, pa + 1, exp
