"""On-disk CSR cache: a saved graph reads back bit-identical without the build, and a
damaged or forged file is refused with RTG_ERR_FORMAT before any kernel sees it."""
from __future__ import annotations

import struct

import numpy as np
import pytest

import oracle
import rtg
from cache_forms import payload_sum

pytestmark = pytest.mark.gpu


def built_graph(ctx, scale=10, seed=5):
    s, d = rtg.gen_rmat(scale, 16, seed=seed)
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE).build(rtg.ORIENT_SYMMETRIC)
    return s, d, g


def test_save_load_roundtrip(ctx, tmp_path):
    s, d, g = built_graph(ctx)
    path = tmp_path / "g.rtgcsr"
    g.save(str(path))
    h = ctx.graph_load(str(path), rtg.FMT_RTG_CSR)
    for sym in (False, True):
        o1, a1 = g.csr(symmetric=sym)
        o2, a2 = h.csr(symmetric=sym)
        assert np.array_equal(o1, o2) and np.array_equal(a1, a2)
    want = g.tc(rtg.TC_BATCHED)[0]
    assert h.tc(rtg.TC_BATCHED)[0] == want and h.tc(rtg.TC_PLAIN)[0] == want
    off, adj = oracle.degree_csr(s, d)
    assert want == oracle.tc_merge(off, adj)
    rng = np.random.default_rng(1)
    n = h.info().n_sym
    u = rng.integers(0, n, 5000, dtype=np.uint32)
    v = rng.integers(0, n, 5000, dtype=np.uint32)
    assert np.array_equal(h.pair_count(u, v)[0], g.pair_count(u, v)[0])
    i1, i2 = g.info(), h.info()
    assert (i1.n, i1.m, i1.m_input, i1.n_sym, i1.m_sym) == (i2.n, i2.m, i2.m_input, i2.n_sym, i2.m_sym)
    h.close()
    g.close()


def test_damaged_files_are_refused(ctx, tmp_path):
    _, _, g = built_graph(ctx, scale=8)
    path = tmp_path / "g.rtgcsr"
    g.save(str(path))
    raw = bytearray(path.read_bytes())
    cases = {
        "flipped": raw[:len(raw) // 2] + bytes([raw[len(raw) // 2] ^ 1]) + raw[len(raw) // 2 + 1:],
        "truncated": raw[:-100],
        "magic": b"XXXXXXXX" + raw[8:],
        "trailing": raw + b"\0" * 8,
    }
    for name, data in cases.items():
        p = tmp_path / f"{name}.rtgcsr"
        p.write_bytes(bytes(data))
        with pytest.raises(rtg.RtgError) as e:
            ctx.graph_load(str(p), rtg.FMT_RTG_CSR)
        assert e.value.status == rtg.ERR_FORMAT, name
    with pytest.raises(rtg.RtgError) as e:
        ctx.graph_load(str(tmp_path / "missing.rtgcsr"), rtg.FMT_RTG_CSR)
    assert e.value.status == rtg.ERR_IO
    g.close()


def test_forged_structure_with_valid_checksum_is_refused(ctx, tmp_path):
    """A counting-form row holding a rank below its vertex would index the kernel's
    bitmap out of range; the loader's structural check refuses it even though the
    checksum is right."""
    _, _, g = built_graph(ctx, scale=8)
    path = tmp_path / "g.rtgcsr"
    g.save(str(path))
    raw = bytearray(path.read_bytes())
    # walk the header to the counting form's adjacency
    pos = 8
    version, parts, m_input, orient, _ = struct.unpack_from("<IIQiI", raw, pos)
    pos += 24
    assert parts & 1 and parts & 2
    n, _, m, _, has_src, _ = struct.unpack_from("<IIQQII", raw, pos)
    pos += 32 + (n + 1) * 8 + m * 4 + (m * 4 if has_src else 0)
    cn, _, cm = struct.unpack_from("<IIQ", raw, pos)
    pos += 16
    off = np.frombuffer(bytes(raw[pos:pos + (cn + 1) * 8]), dtype="<u8")
    pos += (cn + 1) * 8
    v = int(np.argmax(np.diff(off) > 0))  # first vertex with an out-neighbour
    struct.pack_into("<I", raw, pos + int(off[v]) * 4, 0 if v > 0 else v)  # rank <= v
    raw[-8:] = struct.pack("<Q", payload_sum(bytes(raw[8:-8])))
    forged = tmp_path / "forged.rtgcsr"
    forged.write_bytes(bytes(raw))
    with pytest.raises(rtg.RtgError) as e:
        ctx.graph_load(str(forged), rtg.FMT_RTG_CSR)
    assert e.value.status == rtg.ERR_FORMAT
    g.close()


def test_serving_loads_saved_graphs(tmp_path):
    s, d = rtg.gen_rmat(11, 16, seed=9)
    soff, sadj = oracle.symmetric_csr(s, d)
    off, adj = oracle.degree_csr(s, d)
    tri = oracle.tc_merge(off, adj)
    u = np.arange(3000, dtype=np.uint32) % (len(soff) - 1)
    w = (u * 13 + 5) % (len(soff) - 1)
    path = tmp_path / "served.rtgcsr"
    with rtg.Server(0) as srv:
        gid = srv.add_graph(s, d)
        srv.save_graph(gid, str(path))
    with rtg.Server(0) as srv:
        gid = srv.add_graph_file(str(path), rtg.FMT_RTG_CSR)
        assert srv.poll(srv.submit_tc(gid))["triangles"] == tri
        rid, out = srv.submit_pairs(gid, u, w)
        assert srv.poll(rid)["status"] == rtg.OK
        assert np.array_equal(out, oracle.si_pairs(soff, sadj, u, w))
