"""Counting forms written in the CSR cache file layout of csrc/csr_cache.cpp (header,
counting part, checksum of the payload: FNV-1a-64 over the 64-bit words of each 1 MiB block,
the block values chained by FNV-1a-64 seeded with the payload length), and forged variants
of them: shared by the host-side file checks and the checked build's device-side checks."""
from __future__ import annotations

import struct

import numpy as np

import oracle

MAGIC = b"RTGCSR01"


MASK = 0xFFFFFFFFFFFFFFFF
PRIME = 1099511628211
BASIS = 1469598103934665603
BLOCK = 1 << 20


def _block_sum(data: bytes) -> int:
    h = BASIS
    k = len(data) // 8 * 8
    for w in np.frombuffer(data[:k], "<u8").tolist():
        h = ((h ^ w) * PRIME) & MASK
    for b in data[k:]:
        h = ((h ^ b) * PRIME) & MASK
    return h


def payload_sum(data: bytes) -> int:
    h = ((BASIS ^ len(data)) * PRIME) & MASK
    for i in range(0, len(data), BLOCK):
        h = ((h ^ _block_sum(data[i:i + BLOCK])) * PRIME) & MASK
    return h


def counting_form(s: np.ndarray, d: np.ndarray):
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


def cache_file(n, off, adj, in_off, rng, m_input=0) -> bytes:
    body = struct.pack("<IIQiI", 2, 2, m_input, 0, 0)
    body += struct.pack("<IIQ", n, int(np.diff(off.astype(np.int64)).max(initial=0)), len(adj))
    body += off.astype("<u8").tobytes() + adj.astype("<u4").tobytes()
    body += in_off.astype("<u8").tobytes() + rng.astype("<u4").tobytes()
    return MAGIC + body + struct.pack("<Q", payload_sum(body))



def _row_with(off, k):
    """A vertex whose row has at least k entries."""
    lens = np.diff(off.astype(np.int64))
    return int(np.nonzero(lens >= k)[0][0])


def forgeries(form) -> dict:
    """Forged copies of a counting form, each breaking one invariant the batched kernel
    relies on (name -> (n, off, adj, in_off, rng))."""
    n, off, adj, in_off, rng = form
    out = {}
    v = _row_with(off, 1)
    a = adj.copy()
    a[int(off[v])] = v
    out["element at its vertex"] = (n, off, a, in_off, rng)
    v = _row_with(off, 2)
    a = adj.copy()
    q = int(off[v])
    a[q], a[q + 1] = a[q + 1], a[q]
    out["row out of order"] = (n, off, a, in_off, rng)
    r = rng.copy()
    k = int(np.nonzero((r[:, 0] < r[:, 1]) & (r[:, 1] < len(adj)))[0][0])
    r[k, 1] += 1
    out["range into the next row"] = (n, off, adj, in_off, r)
    r = rng.copy()
    heads = np.repeat(np.arange(n), np.diff(in_off.astype(np.int64)))
    for k in range(len(r)):
        u_row = int(np.searchsorted(off, r[k, 0], side="right")) - 1
        start = int(off[u_row])
        if adj[start] <= heads[k] < adj[r[k, 0]] if r[k, 0] < r[k, 1] else False:
            r[k, 0] = start
            out["range below its head"] = (n, off, adj, in_off, r)
            break
    r = rng.copy()
    r[0, 1] = len(adj) + 5
    out["range past the edges"] = (n, off, adj, in_off, r)
    r = rng.copy()
    k = int(np.nonzero(r[:, 0] < r[:, 1])[0][0])
    r[k] = r[k][::-1]
    out["range reversed"] = (n, off, adj, in_off, r)
    a = adj.copy()
    a[len(a) // 2] = n + 7
    out["id beyond the vertices"] = (n, off, a, in_off, rng)
    o = off.copy()
    v = _row_with(off, 1)
    o[v], o[v + 1] = o[v + 1], o[v]
    out["offsets out of order"] = (n, o, adj, in_off, rng)
    io = in_off.copy()
    v = _row_with(in_off, 1)
    io[v], io[v + 1] = io[v + 1], io[v]
    out["in-edge offsets out of order"] = (n, off, adj, io, rng)
    # two in-edges of one head swapped: every range still valid, the source order broken
    r = rng.copy()
    first = in_off[:-1].astype(np.int64)
    k = int(np.nonzero((np.diff(in_off.astype(np.int64)) >= 2) &
                       (r[np.minimum(first + 1, len(r) - 1), 0] > r[first, 0]))[0][0])
    e = int(in_off[k])
    r[[e, e + 1]] = r[[e + 1, e]]
    out["in-edges out of source order"] = (n, off, adj, in_off, r)
    return out
