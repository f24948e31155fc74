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


def test_directory_and_empty_file(tmp_path):
    assert rtg.lib.rtg_graph_file_check(str(tmp_path).encode()) == rtg.ERR_IO
    assert _check(tmp_path, b"") == rtg.ERR_FORMAT


def test_file_read_in_pieces(tmp_path):
    """A file of several read pieces (8 MiB each) and copy pieces (4 MiB each): accepted
    whole, refused with one byte flipped in its last piece or one forged range in its last
    in-edges."""
    s, d = rtg.gen_rmat(17, 16, seed=11)
    big = counting_form(s, d)
    good = cache_file(*big)
    assert len(good) > 2 * (8 << 20)
    assert _check(tmp_path, good) == rtg.OK
    flipped = bytearray(good)
    flipped[len(good) - 100] ^= 4
    assert _check(tmp_path, bytes(flipped)) == rtg.ERR_FORMAT
    n, off, adj, in_off, rng = big
    r = rng.copy()
    k = len(r) - 1
    while r[k, 0] == r[k, 1]:
        k -= 1
    r[k, 1] = min(int(r[k, 1]) + 1, len(adj))
    if int(r[k, 1]) <= int(rng[k, 1]):
        r[k, 0] = r[k, 1] + 1
    assert _check(tmp_path, cache_file(n, off, adj, in_off, r)) == rtg.ERR_FORMAT


def test_other_versions_and_parts_refused(tmp_path, form):
    """A file of another format version, with no part or an unknown part bit, is refused."""
    import struct

    from cache_forms import MAGIC, payload_sum
    good = cache_file(*form)
    body = bytearray(good[8:-8])
    for version, parts in ((1, 2), (3, 2), (2, 0), (2, 8 | 2)):
        b = bytearray(body)
        b[0:8] = struct.pack("<II", version, parts)
        data = MAGIC + bytes(b) + struct.pack("<Q", payload_sum(bytes(b)))
        assert _check(tmp_path, data) == rtg.ERR_FORMAT, (version, parts)
