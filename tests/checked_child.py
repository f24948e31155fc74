"""Child process of tests/test_checked_gpu.py: runs against the library named by RTG_LIB
(the checked build) and exits non-zero on any mismatch.

  parity  – triangle counts of golden graphs in every form (the batched forms also with a
            forced dense core), batched set intersections in
            both kernel forms and one serving round (a count and a pair batch), against the
            golden counts and the oracle
  forged  – counting forms forged to break one invariant each, loaded past the host-side
            file check (the checked build's test hook), are refused by the device-side
            check with RTG_ERR_FORMAT, and the context keeps counting correctly
"""
from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "rt-graph_gb300"))
sys.path.insert(0, str(REPO))
sys.path.insert(0, str(REPO / "tests"))

import oracle  # noqa: E402
import rtg  # noqa: E402
from cache_forms import cache_file, counting_form, forgeries  # noqa: E402
from conftest import golden_edges, tc_golden  # noqa: E402


def parity() -> None:
    gold = tc_golden()
    with rtg.Context(0) as ctx:
        for name in ("k8_1based", "rmat_s12_ef16_s1", "ba_n32768_m8_s1", "hk_n8192_m16_p0.3_s1"):
            rec = gold[name]
            s, d = golden_edges(rec)
            g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE_RAW_REF)
            for mode in (rtg.TC_PLAIN, rtg.TC_BATCHED, rtg.TC_BUCKETED):
                got, _ = g.tc(mode)
                assert got == rec["triangles"], (name, mode, got)
            saved = ctx.config().as_dict()
            for K in (100, 32768):  # dense-core stage, checked kernels
                ctx.set_config(**dict(saved, tc_core_ranks=K))
                for mode in (rtg.TC_BATCHED, rtg.TC_BUCKETED):
                    got, t = g.tc(mode)
                    assert got == rec["triangles"] and t.core_ranks, (name, K, mode, got)
            ctx.set_config(**saved)
            g.close()
        s, d = rtg.gen_rmat(14, 16, seed=2)
        off, adj = oracle.degree_csr(s, d)
        want = oracle.tc_merge(off, adj)
        got, _ = ctx.tc_count_host_edges(s, d, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)
        assert got == want
        # the host-CSR entry's one-shot form (in-edges below the core only), checked
        got, _ = ctx.tc_count_host_csr(off.astype(np.int32), adj.astype(np.int32),
                                       rtg.TC_BATCHED)
        assert got == want
        off, el, pa, pb, exp = rtg.gen_si_pairs(20_000, seed=9)
        sets = ctx.sets(off, el)
        saved = ctx.config().as_dict()
        for form in (1, 2):
            ctx.set_config(**dict(saved, si_form=form))
            got, _ = sets.count(pa, pb, rtg.SI_AUTO)
            assert np.array_equal(got, exp), form
        ctx.set_config(**saved)
        sets.close()
    # the serving engine (its own contexts and launches) through the checked library
    s, d = rtg.gen_rmat(11, 16, seed=7)
    want = oracle.tc_merge(*oracle.degree_csr(s, d))
    soff, sadj = oracle.symmetric_csr(s, d)
    u = np.arange(0, 4000, dtype=np.uint32) % (len(soff) - 1)
    v = (u * 7 + 3) % (len(soff) - 1)
    with rtg.Server(0, held=True) as srv:
        gid = srv.add_graph(s, d)
        rt = srv.submit_tc(gid)
        rp, out = srv.submit_pairs(gid, u, v)
        srv.release()
        assert srv.poll(rt)["triangles"] == want
        assert srv.poll(rp)["status"] == rtg.OK
        assert np.array_equal(out, oracle.si_pairs(soff, sadj, u, v))


def forged() -> None:
    s, d = rtg.gen_rmat(9, 8, seed=4)
    form = counting_form(s, d)
    want = oracle.tc_merge(*oracle.degree_csr(s, d))
    assert rtg.lib.rtg_debug_skip_file_checks(1) == rtg.OK
    try:
        with rtg.Context(0) as ctx, tempfile.TemporaryDirectory() as tmp:
            path = Path(tmp) / "g.rtgcsr"
            path.write_bytes(cache_file(*form))
            g = ctx.graph_load(str(path), rtg.FMT_RTG_CSR)
            assert g.tc(rtg.TC_BATCHED)[0] == want
            g.close()
            cases = forgeries(form)
            assert len(cases) >= 8
            for name, f in cases.items():
                path.write_bytes(cache_file(*f))
                g = ctx.graph_load(str(path), rtg.FMT_RTG_CSR)  # host structure checks skipped
                for mode in (rtg.TC_BATCHED, rtg.TC_BUCKETED):
                    t = rtg.Timing()
                    out = rtg.C.c_uint64(0)
                    st = rtg.lib.rtg_tc_count(ctx.h, g.h, mode, rtg.C.byref(out), rtg.C.byref(t))
                    assert st == rtg.ERR_FORMAT, (name, mode, st)
                    assert b"device-side CSR check" in rtg.lib.rtg_last_error(ctx.h), name
                g.close()
                # the context still counts a valid form
                path.write_bytes(cache_file(*form))
                g = ctx.graph_load(str(path), rtg.FMT_RTG_CSR)
                assert g.tc(rtg.TC_BUCKETED)[0] == want, name
                g.close()
    finally:
        rtg.lib.rtg_debug_skip_file_checks(0)


if __name__ == "__main__":
    assert rtg.lib.rtg_checked_build() == 1, "not the checked build"
    {"parity": parity, "forged": forged}[sys.argv[1]]()
    print("ok", sys.argv[1], flush=True)
