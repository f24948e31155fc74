"""CSR cache files checked on the host (no GPU): rtg_graph_file_check runs the checks that
rtg_graph_load(RTG_FMT_RTG_CSR) applies before anything reaches the device.

A valid counting form is written here in the file layout of csrc/csr_cache.cpp (header,
counting part, block-chained FNV-1a-64 checksum of the payload), then forged so that it
would lead the batched kernel out of its bitmap (an element at or below its vertex, rows out
of order, a suffix range crossing into the next row or reaching below its head); every
forgery, a flipped byte and a truncated file are refused with RTG_ERR_FORMAT.
"""
from __future__ import annotations

import pytest

import rtg
from cache_forms import cache_file, counting_form, forgeries


def _check(tmp_path, data: bytes) -> int:
    p = tmp_path / "g.rtgcsr"
    p.write_bytes(data)
    return rtg.lib.rtg_graph_file_check(str(p).encode())


@pytest.fixture(scope="module")
def form():
    s, d = rtg.gen_rmat(9, 8, seed=4)
    return counting_form(s, d)


def test_valid_counting_form_accepted(tmp_path, form):
    assert _check(tmp_path, cache_file(*form)) == rtg.OK


def test_missing_file_is_io_error(tmp_path):
    assert rtg.lib.rtg_graph_file_check(str(tmp_path / "none").encode()) == rtg.ERR_IO


def test_damaged_files_refused(tmp_path, form):
    good = cache_file(*form)
    flipped = bytearray(good)
    flipped[40] ^= 1
    assert _check(tmp_path, bytes(flipped)) == rtg.ERR_FORMAT
    assert _check(tmp_path, good[:-9]) == rtg.ERR_FORMAT
    assert _check(tmp_path, good[:12]) == rtg.ERR_FORMAT
    assert _check(tmp_path, b"NOTACSR!" + good[8:]) == rtg.ERR_FORMAT


def test_forged_counting_forms_refused(tmp_path, form):
    for name, forged in forgeries(form).items():
        assert _check(tmp_path, cache_file(*forged)) == rtg.ERR_FORMAT, name
    # the unforged form still passes
    assert _check(tmp_path, cache_file(*form)) == rtg.OK
