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
