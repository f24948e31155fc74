"""The C++ snippets of INTEGRATION.md, compiled against the reference's own headers.

Every ```cpp block of INTEGRATION.md is a complete function that a maintainer would paste
into the reference's code. This test puts them in one translation unit after the
reference's tc/graph/include/graph.h, tc/utils/model.h and set_intersection/utils/util.h
and include/rtg.h, compiles it and links it against librtg.so with no undefined symbols
(compile and link only: nothing runs). The reference checkout is looked up at
$RTG_REFERENCE, else next to the repository; without it the test is skipped.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent
REF = Path(os.environ.get("RTG_REFERENCE", REPO.parent / "reference"))
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _snippets() -> list[str]:
    text = (REPO / "INTEGRATION.md").read_text()
    return re.findall(r"```cpp\n(.*?)```", text, flags=re.S)


def test_integration_has_snippets():
    assert len(_snippets()) >= 4


@pytest.mark.skipif(not (REF / "tc" / "graph" / "include" / "graph.h").exists(),
                    reason="reference checkout not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_integration_snippets_compile_and_link(tmp_path):
    src = tmp_path / "snippets.cpp"
    body = "\n".join(_snippets())
    src.write_text("#include <cstdio>\n#include <cstdint>\n#include <vector>\n"
                   '#include "graph.h"\n#include "util.h"\n#include "rtg.h"\n\n' + body)
    lib = REPO / "rt-graph_gb300" / "lib"
    out = tmp_path / "snippets.so"
    cmd = ["g++", "-std=c++17", "-fPIC", "-shared", "-Wl,--no-undefined",
           f"-I{REF / 'tc' / 'graph' / 'include'}", f"-I{REF / 'tc' / 'utils'}",
           f"-I{REF / 'set_intersection' / 'utils'}", f"-I{REPO / 'include'}",
           f"-I{CUDA / 'include'}", str(src), "-o", str(out), f"-L{lib}", "-lrtg",
           f"-Wl,-rpath,{lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    nm = subprocess.run(["nm", "-D", "--undefined-only", str(out)], capture_output=True,
                        text=True).stdout
    for sym in ("rtg_tc_count_host_csr", "rtg_graph_from_host_pairs", "rtg_si_count_dense",
                "rtg_tc_list"):
        assert sym in nm
