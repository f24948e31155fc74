"""Generate the golden vectors that pin the CPU oracle to the reference's own code.

Runs oracle/_ref/ref_driver (built by oracle/build_ref.sh from the reference sources:
tc/graph/graph.cpp, the host Preprocessing of tc/bs_tc/bs_tc.cu and
set_intersection/data_generator/data.cpp) and records:

  tc_golden.json  – per input graph: the reference's CSR after ReadBinaryEdges +
                    TCPreprocessing + ConvertToCSR (nodes, edges, sha256 of offsets/adjs as
                    little-endian int32, full arrays for small graphs) and the triangle count
                    of its two-hop Preprocessing + HashmapKernel rule.
  si/*.s_data     – dataset files written by the reference's Data::Generator/Writer; the
                    known answer of every A x B pair is the header's `intersection` field.

Inputs are either inline edge lists or librtg's seeded generators (the sha256 of the
generated edge list is stored so a changed generator is detected).

Usage: python tests/golden/make_golden.py   (needs the reference checkout; run here only)
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path.insert(0, str(REPO / "rt-graph_gb300"))
import rtg  # noqa: E402

DRIVER = REPO / "oracle" / "_ref" / "ref_driver"

INLINE = {
    "k4_noise": [(1, 2), (2, 3), (3, 1), (3, 4), (4, 1), (1, 2), (5, 5), (2, 4), (6, 7)],
    "triangle": [(0, 1), (1, 2), (2, 0)],
    "triangle_1based": [(1, 2), (2, 3), (3, 1)],
    "two_triangles_shared_edge": [(0, 1), (1, 2), (2, 0), (1, 3), (3, 2)],
    "bowtie": [(0, 1), (1, 2), (2, 0), (2, 3), (3, 4), (4, 2)],
    "star": [(0, i) for i in range(1, 9)],
    "path": [(i, i + 1) for i in range(10)],
    "matching_only": [(0, 1), (2, 3), (4, 5)],
    "self_loops_only": [(0, 0), (1, 1), (2, 2)],
    "dups_both_directions": [(0, 1), (1, 0), (1, 2), (2, 1), (2, 0), (0, 2), (0, 1), (2, 2)],
    "sparse_ids": [(100, 5000), (5000, 70000), (70000, 100), (70000, 123456), (123456, 100),
                   (9, 9), (42, 100)],
    "k5": [(i, j) for i in range(5) for j in range(i + 1, 5)],
    "k6_reversed": [(j, i) for i in range(6) for j in range(i + 1, 6)],
    "k8_1based": [(i, j) for i in range(1, 9) for j in range(i + 1, 9)],
    "wheel": [(0, i) for i in range(1, 9)] + [(i, i % 8 + 1) for i in range(1, 9)],
}

GENERATED = {
    "ba_n32768_m8_s1": ("ba", dict(n=32768, m=8, seed=1)),
    "ba_n4096_m4_s7": ("ba", dict(n=4096, m=4, seed=7)),
    "hk_n8192_m16_p0.3_s1": ("hk", dict(n=8192, m=16, p=0.3, seed=1)),
    "hk_n20000_m6_p0.9_s3": ("hk", dict(n=20000, m=6, p=0.9, seed=3)),
    "rmat_s12_ef16_s1": ("rmat", dict(scale=12, edge_factor=16, seed=1)),
    "rmat_s14_ef16_s42": ("rmat", dict(scale=14, edge_factor=16, seed=42)),
    "rmat_s10_ef8_s5_skewed": ("rmat", dict(scale=10, edge_factor=8, a=0.7, b=0.1, c=0.1, seed=5)),
}

SI_CASES = {
    # name: (mode, args) for ref_driver
    "single_len1000_skew1_sel0.3_d0.1_a8": ("si_single", ["1000", "1", "0.3", "0.1", "8"]),
    "single_len2048_skew4_sel0.2_d0.05_a4": ("si_single", ["2048", "4", "0.2", "0.05", "4"]),
    "single_len64_skew1_sel1.0_d0.5_a16": ("si_single", ["64", "1", "1.0", "0.5", "16"]),
    "single_len500_skew1_sel0_d0.2_a4": ("si_single", ["500", "1", "0", "0.2", "4"]),
    "multi_len300_uniform_a100_b3": ("si_multi", ["300", "1", "0.4", "0", "1", "100", "3"]),
    "multi_len200_normal_skew2_a100_b2": ("si_multi", ["200", "2", "0.25", "1", "1", "100", "2"]),
    "multi_len128_exp_a100_b2": ("si_multi", ["128", "1", "0.5", "2", "4", "100", "2"]),
}


def gen_edges(kind: str, kw: dict):
    if kind == "ba":
        return rtg.gen_ba(kw["n"], kw["m"], kw["seed"])
    if kind == "hk":
        return rtg.gen_hk(kw["n"], kw["m"], kw["p"], kw["seed"])
    if kind == "rmat":
        return rtg.gen_rmat(kw["scale"], kw.get("edge_factor", 16), kw.get("a", 0.57),
                            kw.get("b", 0.19), kw.get("c", 0.19), kw["seed"])
    raise ValueError(kind)


def edges_sha(s: np.ndarray, d: np.ndarray) -> str:
    pairs = np.stack([s.astype("<i4"), d.astype("<i4")], axis=1)
    return hashlib.sha256(pairs.tobytes()).hexdigest()


def run_tc(edge_file: Path, csr_file: Path):
    out = subprocess.run([str(DRIVER), "tc", str(edge_file), str(csr_file)], check=True,
                         capture_output=True, text=True).stdout
    line = [l for l in out.splitlines() if l.startswith("REF_TC")][-1]
    _, nodes, edges, count = line.split()
    raw = np.fromfile(csr_file, dtype="<i4")
    n, e = int(raw[0]), int(raw[1])
    assert (n, e) == (int(nodes), int(edges))
    off = raw[2:2 + n + 1]
    adj = raw[2 + n + 1:2 + n + 1 + e]
    return n, e, int(count), off, adj


def main() -> None:
    if not DRIVER.exists():
        subprocess.run([str(REPO / "oracle" / "build_ref.sh")], check=True)
    tc = {}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        cases = []
        for name, edges in INLINE.items():
            a = np.array(edges, dtype=np.int64).reshape(-1, 2)
            cases.append((name, {"edge_list": edges}, a[:, 0].astype(np.uint32),
                          a[:, 1].astype(np.uint32)))
        for name, (kind, kw) in GENERATED.items():
            s, d = gen_edges(kind, kw)
            cases.append((name, {"generator": kind, "params": kw, "edges_sha256": edges_sha(s, d),
                                 "m_input": int(len(s))}, s, d))
        for name, src, s, d in cases:
            ef = td / f"{name}.edge"
            rtg.edges_write_bin(str(ef), s, d)
            n, e, count, off, adj = run_tc(ef, td / f"{name}.csr")
            rec = dict(src)
            rec.update(nodes=n, edges=e, triangles=count,
                       offsets_sha256=hashlib.sha256(off.astype("<i4").tobytes()).hexdigest(),
                       adjs_sha256=hashlib.sha256(adj.astype("<i4").tobytes()).hexdigest())
            if e <= 64:
                rec["offsets"] = off.tolist()
                rec["adjs"] = adj.tolist()
            tc[name] = rec
            print(f"tc {name}: nodes={n} edges={e} triangles={count}")
    (HERE / "tc_golden.json").write_text(json.dumps(tc, indent=1) + "\n")

    si_dir = HERE / "si"
    if si_dir.exists():
        shutil.rmtree(si_dir)
    si_dir.mkdir()
    si = {}
    for name, (mode, args) in SI_CASES.items():
        with tempfile.TemporaryDirectory() as td:
            subprocess.run([str(DRIVER), mode, *args, td + os.sep], check=True,
                           capture_output=True, text=True)
            files = list(Path(td).iterdir())
            assert len(files) == 1, files
            dst = si_dir / f"{name}.s_data"
            shutil.copy(files[0], dst)
        info, off, el = rtg.dataset_read(str(dst))
        si[name] = dict(mode=mode, args=args, num_a=info.num_a, num_b=info.num_b,
                        max_element=info.max_element, intersection=info.intersection,
                        elems=int(info.elems),
                        sha256=hashlib.sha256(dst.read_bytes()).hexdigest())
        print(f"si {name}: A={info.num_a} B={info.num_b} |A∩B|={info.intersection} "
              f"elems={info.elems} bytes={dst.stat().st_size}")
    (HERE / "si_golden.json").write_text(json.dumps(si, indent=1) + "\n")


if __name__ == "__main__":
    main()
