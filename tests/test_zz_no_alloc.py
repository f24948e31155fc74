"""The allocation-free triangle count (rtg_tc_count_device_csr_noalloc), through the C ABI.

That entry point serves callers that cannot let the library allocate device memory (an
application pool or framework allocator owns the heap, or an allocation's implicit
synchronisation is not allowed on their path); its scratch is a fixed device array inside
the library. Here its result is compared with the regular entry point's on device CSRs
that librtg already holds, twice in a row, since every call reuses the same array. Exact
integer counts, so the tolerance is zero.
"""
from __future__ import annotations

import ctypes as C

import pytest

import rtg
from conftest import golden_edges, tc_golden

pytestmark = pytest.mark.gpu


def _device_csr(g: rtg.Graph):
    off = C.c_void_p()
    adj = C.c_void_p()
    n = C.c_uint32()
    m = C.c_uint64()
    st = rtg.lib.rtg_csr_view(g.h, 0, C.byref(off), C.byref(adj), C.byref(n), C.byref(m))
    assert st == rtg.OK
    return off, adj, n.value, m.value


def _noalloc_count(off, adj, n, m) -> int:
    out = C.c_uint64(123)
    st = rtg.lib.rtg_tc_count_device_csr_noalloc(off, adj, n, m, C.byref(out), None)
    assert st == rtg.OK, rtg.lib.rtg_status_str(st)
    return out.value


@pytest.mark.parametrize("name", ["rmat_s14_ef16_s42", "ba_n32768_m8_s1", "hk_n8192_m16_p0.3_s1"])
def test_noalloc_matches_regular_entry_point_twice(ctx, name):
    s, d = golden_edges(tc_golden()[name])
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj, n, m = _device_csr(g)
    assert m <= (1 << 19)
    want, _ = g.tc(rtg.TC_BATCHED)
    first = _noalloc_count(off, adj, n, m)
    second = _noalloc_count(off, adj, n, m)
    assert first == want
    assert second == want
    assert want == tc_golden()[name]["triangles"]


def test_noalloc_alternating_graphs_reuse_the_array(ctx):
    graphs = []
    for name in ("wheel", "rmat_s12_ef16_s1"):
        s, d = golden_edges(tc_golden()[name])
        g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE_RAW_REF)
        graphs.append((g, tc_golden()[name]["triangles"]))
    for _ in range(2):
        for g, want in graphs:
            assert _noalloc_count(*_device_csr(g)) == want
            assert g.tc(rtg.TC_PLAIN)[0] == want


def test_noalloc_rejects_graphs_beyond_its_limit(ctx):
    """Real device arrays with an edge count one past the limit: refused before any GPU
    work; the same arrays with their true sizes then count correctly."""
    rec = tc_golden()["rmat_s12_ef16_s1"]
    s, d = golden_edges(rec)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj, n, m = _device_csr(g)
    out = C.c_uint64(7)
    st = rtg.lib.rtg_tc_count_device_csr_noalloc(off, adj, n, (1 << 19) + 1, C.byref(out), None)
    assert st == rtg.ERR_INVALID_ARG
    assert _noalloc_count(off, adj, n, m) == rec["triangles"]
    st = rtg.lib.rtg_tc_count_device_csr_noalloc(None, None, 0, 0, C.byref(out), None)
    assert st == rtg.OK and out.value == 0


def test_noalloc_rejects_sizes_that_do_not_describe_the_csr(ctx):
    """The device-side check of the offsets and ids: an edge count below the CSR's (the
    offsets end past m) and a vertex count at or below the largest stored id are refused with
    RTG_ERR_INVALID_ARG (every read stays inside the real arrays, which are larger); the
    shared scratch array then still gives the right count."""
    rec = tc_golden()["rmat_s12_ef16_s1"]
    s, d = golden_edges(rec)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    off, adj, n, m = _device_csr(g)
    top = int(g.csr()[1].max())  # the largest id stored: a vertex count of `top` excludes it
    out = C.c_uint64(7)
    for bad_n, bad_m in ((n, m - 1), (top, m), (top, m - 1)):
        st = rtg.lib.rtg_tc_count_device_csr_noalloc(off, adj, bad_n, bad_m, C.byref(out), None)
        assert st == rtg.ERR_INVALID_ARG, (bad_n, bad_m)
    for _ in range(2):
        assert _noalloc_count(off, adj, n, m) == rec["triangles"]
