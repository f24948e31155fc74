"""The checked build (librtg_checked.so, RTG_CHECKED): every CSR and counting form is
validated on the device before a count reads it and the counting kernels check the indexes
they derive from it, reporting violations through the device status word. Each case runs
in a child process bound to that library (tests/checked_child.py).

No input here can fault the GPU: the forged forms break structure only (sizes and
checksum stay valid, so every array has the length its header states), the device checks
read only at loop counters or at values already checked against their array's size, and
no count kernel runs on a form the checks refused.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parent.parent
CHECKED = REPO / "rt-graph_gb300" / "lib" / "librtg_checked.so"


def _child(what: str) -> None:
    assert CHECKED.exists(), "checked build missing (rt-graph_gb300/build.py)"
    r = subprocess.run([sys.executable, str(REPO / "tests" / "checked_child.py"), what],
                       env=dict(os.environ, RTG_LIB=str(CHECKED)), capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and f"ok {what}" in r.stdout, r.stdout + r.stderr


def test_checked_build_counts_exactly():
    _child("parity")


def test_checked_build_refuses_forged_forms_on_the_device():
    _child("forged")
