"""Host logic of bench.py that needs no GPU: the clock sampler around the timed region.

A fake `nvidia-smi` on PATH prints the sampler's CSV fields every 20 ms after a 0.1 s
start-up delay, the way the real one does."""
from __future__ import annotations

import importlib.util
import os
import stat
import time
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", REPO / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _fake_smi(tmp_path: Path, line: str) -> None:
    exe = tmp_path / "nvidia-smi"
    exe.write_text("#!/bin/sh\nsleep 0.1\nwhile true; do echo '%s'; sleep 0.02; done\n" % line)
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)


@pytest.fixture
def bench(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", f"{tmp_path}{os.pathsep}{os.environ['PATH']}")
    return _bench()


def test_samples_come_from_the_timed_region(bench, tmp_path):
    _fake_smi(tmp_path, "0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active")
    t0 = time.monotonic()
    with bench.ClockSampler(0) as clk:
        entered = time.monotonic()
        time.sleep(0.2)
    s = clk.summary()
    assert entered - t0 >= 0.09          # waited for the first line before the region
    assert clk.first >= 1 and s["samples"] >= 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["reasons"] == []


def test_throttle_reasons_reported(bench, tmp_path):
    _fake_smi(tmp_path, "0, 1800, 2070, 1390.0, 0x4, Not Active, Not Active, Not Active, Active")
    with bench.ClockSampler(0) as clk:
        time.sleep(0.1)
    s = clk.summary()
    assert s["reasons"] == ["sw_power_cap"] and s["sm_mhz"] == 1800.0


def test_no_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))  # nothing to run
    bench = _bench()
    with bench.ClockSampler(0) as clk:
        pass
    assert clk.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def _brute_split(off, adj, K):
    """The batched count's work split restated element by element on a small graph: rank
    vertices by (degree, id), take each out-list in rank order, stream the suffix after v of
    every in-edge u->v from a source below the core (heads with out-edges only), and sweep,
    for every core edge but the last of its row, the 16-byte groups of N+(v)'s rank span up
    to u's last group."""
    import numpy as np
    n = len(off) - 1
    rows = [list(adj[off[u]:off[u + 1]]) for u in range(n)]
    deg = [len(rows[u]) for u in range(n)]
    for u in range(n):
        for v in rows[u]:
            deg[v] += 1
    order = sorted(range(n), key=lambda x: (deg[x], x))
    rank = {x: r for r, x in enumerate(order)}
    c0 = n - K
    rrows = [sorted(rank[w] for w in rows[u]) for u in range(n)]
    byrank = [None] * n
    for u in range(n):
        byrank[rank[u]] = rrows[u]
    elems = inedges = 0
    sdeg = [0] * n
    for ru in range(c0):
        r = byrank[ru]
        for i, rv in enumerate(r):
            if byrank[rv]:
                elems += len(r) - i - 1
                inedges += 1
                sdeg[rv] += 1
    mark = sum(len(byrank[rv]) for rv in range(n) if sdeg[rv] and byrank[rv])
    groups = 0
    for ru in range(c0, n):
        r = byrank[ru]
        for rv in r[:-1]:
            if not byrank[rv]:
                continue
            g0 = ((byrank[rv][0] - c0) >> 5) >> 2
            g1 = min(((byrank[rv][-1] - c0) >> 5) >> 2, ((r[-1] - c0) >> 5) >> 2)
            groups += max(0, g1 - g0 + 1)
    core_edges = sum(len(byrank[ru]) for ru in range(c0, n))
    return elems, inedges, mark, groups, core_edges


@pytest.mark.parametrize("K", [0, 1, 40, 200, 1000])
def test_tc_split_matches_element_count(K):
    """bench.tc_split (the roofline's algorithmic bytes of the streaming kernel and the core
    stage's swept groups) against the element-by-element restatement."""
    import numpy as np
    import oracle
    bench = _bench()
    s, d = oracle.gen_rmat(10, 8, 0.57, 0.19, 0.19, seed=3)
    off, adj = oracle.degree_csr(s, d)
    K = min(K, len(off) - 1)
    got = bench.tc_split(off, adj, K)
    elems, inedges, mark, groups, core_edges = _brute_split(off, adj, K)
    assert got["stream_elems"] == elems
    assert got["stream_inedges"] == inedges
    assert got["mark_elems"] == mark
    assert got["core_groups"] == groups
    assert got["core_edges"] == core_edges
    n = len(off) - 1
    assert got["stream_bytes"] == 4 * elems + 8 * inedges + 4 * mark + 16 * n
