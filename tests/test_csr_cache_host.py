"""CSR cache files checked on the host (no GPU): rtg_graph_file_check runs the checks that
rtg_graph_load(RTG_FMT_RTG_CSR) applies before anything reaches the device.

A valid counting form is written here in the file layout of csrc/csr_cache.cpp (header,
counting part, FNV-1a-64 checksum of every byte after the magic), then forged so that it
would lead the batched kernel out of its bitmap (an element at or below its vertex, rows out
of order, a suffix range crossing into the next row or reaching below its head); every
forgery, a flipped byte and a truncated file are refused with RTG_ERR_FORMAT.
"""
from __future__ import annotations

import struct

import numpy as np
import pytest

import oracle
import rtg

MAGIC = b"RTGCSR01"


def _fnv(data: bytes) -> int:
    h = 1469598103934665603
    for b in data:
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def _counting_form(s: np.ndarray, d: np.ndarray):
    """Counting form of a small graph: ranks by (degree, id), edges low -> high rank, rows
    ascending, in-edges grouped by head with their suffix ranges [e + 1, row end)."""
    off, adj = oracle.degree_csr(s, d)
    n = len(off) - 1
    src = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
    deg = np.bincount(src, minlength=n) + np.bincount(adj.astype(np.int64), minlength=n)
    rank = np.empty(n, np.int64)
    rank[np.lexsort((np.arange(n), deg))] = np.arange(n)
    a, b = rank[src], rank[adj.astype(np.int64)]
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    order = np.lexsort((hi, lo))
    lo, hi = lo[order], hi[order]
    coff = np.zeros(n + 1, np.uint64)
    np.add.at(coff, lo + 1, 1)
    coff = np.cumsum(coff).astype(np.uint64)
    m = len(hi)
    pos = np.arange(m)
    rend = coff[lo + 1].astype(np.int64)
    ino = np.lexsort((pos, hi))
    in_off = np.zeros(n + 1, np.uint64)
    np.add.at(in_off, hi + 1, 1)
    in_off = np.cumsum(in_off).astype(np.uint64)
    rng = np.stack([pos[ino] + 1, rend[ino]], axis=1).astype(np.uint32)
    return n, coff, hi.astype(np.uint32), in_off, rng


def _file(n, off, adj, in_off, rng, m_input=0) -> bytes:
    body = struct.pack("<IIQiI", 1, 2, m_input, 0, 0)
    body += struct.pack("<IIQ", n, int(np.diff(off.astype(np.int64)).max(initial=0)), len(adj))
    body += off.astype("<u8").tobytes() + adj.astype("<u4").tobytes()
    body += in_off.astype("<u8").tobytes() + rng.astype("<u4").tobytes()
    return MAGIC + body + struct.pack("<Q", _fnv(body))


def _check(tmp_path, data: bytes) -> int:
    p = tmp_path / "g.rtgcsr"
    p.write_bytes(data)
    return rtg.lib.rtg_graph_file_check(str(p).encode())


@pytest.fixture(scope="module")
def form():
    s, d = rtg.gen_rmat(9, 8, seed=4)
    return _counting_form(s, d)


def test_valid_counting_form_accepted(tmp_path, form):
    assert _check(tmp_path, _file(*form)) == rtg.OK


def test_missing_file_is_io_error(tmp_path):
    assert rtg.lib.rtg_graph_file_check(str(tmp_path / "none").encode()) == rtg.ERR_IO


def test_damaged_files_refused(tmp_path, form):
    good = _file(*form)
    flipped = bytearray(good)
    flipped[40] ^= 1
    assert _check(tmp_path, bytes(flipped)) == rtg.ERR_FORMAT
    assert _check(tmp_path, good[:-9]) == rtg.ERR_FORMAT
    assert _check(tmp_path, good[:12]) == rtg.ERR_FORMAT
    assert _check(tmp_path, b"NOTACSR!" + good[8:]) == rtg.ERR_FORMAT


def _row_with(off, k):
    """A vertex whose row has at least k entries."""
    lens = np.diff(off.astype(np.int64))
    return int(np.nonzero(lens >= k)[0][0])


def test_forged_counting_forms_refused(tmp_path, form):
    n, off, adj, in_off, rng = form
    # an element at or below its own vertex
    v = _row_with(off, 1)
    a = adj.copy()
    a[int(off[v])] = v
    assert _check(tmp_path, _file(n, off, a, in_off, rng)) == rtg.ERR_FORMAT
    # a row out of order
    v = _row_with(off, 2)
    a = adj.copy()
    q = int(off[v])
    a[q], a[q + 1] = a[q + 1], a[q]
    assert _check(tmp_path, _file(n, off, a, in_off, rng)) == rtg.ERR_FORMAT
    # a suffix range that runs into the next row
    r = rng.copy()
    k = int(np.nonzero((r[:, 0] < r[:, 1]) & (r[:, 1] < len(adj)))[0][0])
    r[k, 1] += 1
    assert _check(tmp_path, _file(n, off, adj, in_off, r)) == rtg.ERR_FORMAT
    # a suffix range that starts at or below its head (first element of the head's row
    # position, moved back to the row start)
    r = rng.copy()
    heads = np.repeat(np.arange(n), np.diff(in_off.astype(np.int64)))
    for k in range(len(r)):
        u_row = int(np.searchsorted(off, r[k, 0], side="right")) - 1
        start = int(off[u_row])
        if adj[start] <= heads[k] < adj[r[k, 0]] if r[k, 0] < r[k, 1] else False:
            r[k, 0] = start
            break
    else:
        pytest.skip("no suffix range to move below its head")
    assert _check(tmp_path, _file(n, off, adj, in_off, r)) == rtg.ERR_FORMAT
    # a range beyond the edge count
    r = rng.copy()
    r[0, 1] = len(adj) + 5
    assert _check(tmp_path, _file(n, off, adj, in_off, r)) == rtg.ERR_FORMAT
    # the unforged form still passes
    assert _check(tmp_path, _file(n, off, adj, in_off, rng)) == rtg.OK
