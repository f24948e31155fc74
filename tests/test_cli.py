"""The drop-in command-line tools: same arguments and result lines as the reference's.

CPU: the dataset generator reproduces the reference generator's files byte for byte, and
the text-to-binary convertor matches librtg's writer. GPU: bs_tc / rt_tc on golden graphs
report the reference's counts (and rt_tc its post-preprocessing sizes); every SI tool
accepts the reference's own dataset files.
"""
from __future__ import annotations

import re
import subprocess

import numpy as np
import pytest

import rtg
from conftest import GOLDEN, REPO, golden_edges, si_golden, tc_golden

BIN = REPO / "rt-graph_gb300" / "bin"


def run(tool: str, *args, timeout=300) -> str:
    r = subprocess.run([str(BIN / tool), *map(str, args)], capture_output=True, text=True,
                       timeout=timeout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("name", [n for n, r in si_golden().items() if r["mode"] == "si_single"])
def test_s_generator_reproduces_reference_files(tmp_path, name):
    rec = si_golden()[name]
    length, skew, sel, density, num_a = rec["args"]
    out = run("s_generator", "-l", length, "-r", skew, "-s", sel, "-d", density, "-a", num_a,
              "-f", str(tmp_path) + "/")
    path = re.search(r"written to path: (\S+)", out).group(1)
    assert open(path, "rb").read() == (GOLDEN / "si" / f"{name}.s_data").read_bytes()


@pytest.mark.parametrize("name", [n for n, r in si_golden().items() if r["mode"] == "si_multi"])
def test_m_generator_reproduces_reference_files(tmp_path, name):
    """Uniform, normal and exponential multi-set files, byte for byte as the reference's
    generator wrote them (its fixed 1000 A sets replaced by the recorded count)."""
    rec = si_golden()[name]
    length, skew, sel, dist, lam, num_a, num_b = rec["args"]
    out = run("m_generator", "-l", length, "-r", skew, "-s", sel, "-d", dist, "-b", lam,
              "-a", num_a, "-n", num_b, "-f", str(tmp_path) + "/")
    path = re.search(r"written to path: (\S+)", out).group(1)
    assert path.endswith({"0": "_uni.m_data", "1": "_nor.m_data"}.get(dist, "_exp.m_data"))
    assert open(path, "rb").read() == (GOLDEN / "si" / f"{name}.s_data").read_bytes()


def test_convertor_matches_binary_writer(tmp_path):
    s, d = golden_edges(tc_golden()["wheel"])
    (tmp_path / "g.txt").write_text("".join(f"{a} {b}\n" for a, b in zip(s, d)))
    run("convertor", tmp_path / "g.txt", tmp_path / "g.bin")
    rtg.edges_write_bin(str(tmp_path / "w.bin"), s, d)
    assert (tmp_path / "g.bin").read_bytes() == (tmp_path / "w.bin").read_bytes()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["k4_noise", "k8_1based", "sparse_ids", "ba_n4096_m4_s7",
                                  "rmat_s12_ef16_s1", "matching_only"])
def test_bs_tc_and_rt_tc(tmp_path, name):
    rec = tc_golden()[name]
    s, d = golden_edges(rec)
    rtg.edges_write_bin(str(tmp_path / "g.edge"), s, d)
    out = run("bs_tc", tmp_path / "g.edge", 0)
    assert int(re.search(r"counting result = (\d+)", out).group(1)) == rec["triangles"]
    out = run("rt_tc", tmp_path / "g.edge", 0)
    assert int(re.search(r"Triangle Counting = (\d+)", out).group(1)) == rec["triangles"]
    nodes, edges = map(int, re.search(r"After preprocessing: nodes = (\d+), edges = (\d+)",
                                      out).groups())
    assert (nodes, edges) == (rec["nodes"], rec["edges"])


@pytest.mark.gpu
@pytest.mark.parametrize("tool", ["bs", "hi", "ip", "bi_naive", "bi_dynamic", "rt_intersection"])
def test_si_tools_accept_reference_datasets(tool):
    for name in si_golden():
        extra = ["--buckets", "97", "--bucket_size", "64"] if tool == "hi" else []
        extra += ["--chunk_length", "1000"] if tool == "rt_intersection" else []
        out = run(tool, "--device", "0", "--dataset", GOLDEN / "si" / f"{name}.s_data", *extra)
        assert "Check: accepted" in out, (tool, name, out[-500:])
        assert "kernel time" in out or "RT counting time" in out
