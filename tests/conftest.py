"""Shared test setup.

`-m "not gpu"` runs the oracle-vs-golden checks, host logic and C-ABI checks on CPU;
`-m gpu` runs the parity tests, which call librtg through its C ABI on a real GPU and
fail (never skip) when no device or no library is present.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "rt-graph_gb300"))
sys.path.insert(0, str(REPO))

GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; calls librtg kernels")
    lib = REPO / "rt-graph_gb300" / "lib" / "librtg.so"
    tools = REPO / "rt-graph_gb300" / "bin" / "s_generator"
    if not lib.exists() or not tools.exists():
        import importlib.util
        spec = importlib.util.spec_from_file_location("rtg_build", REPO / "rt-graph_gb300" / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build_all(cli=True, oracle=True)


def tc_golden() -> dict:
    return json.loads((GOLDEN / "tc_golden.json").read_text())


def si_golden() -> dict:
    return json.loads((GOLDEN / "si_golden.json").read_text())


def golden_edges(rec: dict):
    """Edge arrays of a tc_golden record (inline or regenerated with librtg's generator)."""
    import rtg
    if "edge_list" in rec:
        a = np.array(rec["edge_list"], dtype=np.int64).reshape(-1, 2)
        return a[:, 0].astype(np.uint32), a[:, 1].astype(np.uint32)
    kw = rec["params"]
    kind = rec["generator"]
    if kind == "ba":
        return rtg.gen_ba(kw["n"], kw["m"], kw["seed"])
    if kind == "hk":
        return rtg.gen_hk(kw["n"], kw["m"], kw["p"], kw["seed"])
    return rtg.gen_rmat(kw["scale"], kw.get("edge_factor", 16), kw.get("a", 0.57),
                        kw.get("b", 0.19), kw.get("c", 0.19), kw["seed"])


def edges_sha(s, d) -> str:
    import hashlib
    pairs = np.stack([np.asarray(s).astype("<i4"), np.asarray(d).astype("<i4")], axis=1)
    return hashlib.sha256(pairs.tobytes()).hexdigest()


def sha_i32(a) -> str:
    import hashlib
    return hashlib.sha256(np.asarray(a).astype("<i4").tobytes()).hexdigest()


@pytest.fixture(scope="session")
def ctx():
    import rtg
    c = rtg.Context(0)   # raises on a machine without a GPU: gpu tests fail, never skip
    yield c
    c.close()
