"""Text edge-list and MatrixMarket readers: the semantics of the reference's line-by-line
stream extraction (`std::istringstream(line) >> a >> b`, tc/graph/graph.cpp:179-214;
bfs/graph/graph.cpp:17-117) on lines that stress it: blank and comment lines, signs, junk
after or between the numbers, CRLF, values past int32 and past long long, missing final
newlines, MatrixMarket headers, sizes, comments, symmetric expansion and short files. The
expected results were produced by the stream-based readers these replace; no GPU."""
from __future__ import annotations

import pytest

import rtg

TXT = {
    "basic": "0 1\n1 2\n2 0\n",
    "comments_blank": "# c\n\n% x\n0 1\n   \n3\t4\n",
    "crlf": "0 1\r\n2 3\r\n",
    "trailing_tokens": "0 1 7 8\n2 3 x\n",
    "junk_after_second": "1 2abc\n5 6\n",
    "junk_after_first": "1abc 2\n7 8\n",
    "no_space": "1-2\n",
    "plus_sign": "+3 +4\n",
    "minus_zero": "-0 5\n",
    "float": "1.5 2\n3 4\n",
    "single_token": "12\n3 4\n",
    "leading_ws": "   9    10   \n",
    "tabs_vt": "\t11\u000b12\f\n",
    "no_trailing_newline": "13 14",
    "big_ok": "2147483647 0\n",
    "too_big": "2147483648 0\n",
    "negative": "-1 2\n",
    "overflow_ll": "99999999999999999999 1\n3 4\n",
    "comma": "1,2\n3 4\n",
    "unicode": "5 6\n\u00e2\u0080\u008b7 8\n"
}

MTX = {
    "general": "%%MatrixMarket matrix coordinate pattern general\n% c\n3 3 2\n1 2\n3 1\n",
    "symmetric": "%%MatrixMarket matrix coordinate pattern symmetric\n3 3 3\n1 2\n2 2\n3 1\n",
    "values": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 2 0.5\n2 3 1e3\n",
    "extra_lines": "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 2\n2 1\n",
    "too_few": "%%MatrixMarket matrix coordinate pattern general\n2 2 3\n1 2\n",
    "out_of_range": "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n3 1\n",
    "zero_index": "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n0 1\n",
    "bad_header": "%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 2\n",
    "array_format": "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
    "caps": "%%MatrixMarket MATRIX Coordinate Pattern SYMMETRIC\n2 2 1\n1 2\n",
    "comment_in_body": "%%MatrixMarket matrix coordinate pattern general\n3 3 2\n1 2\n% mid\n\n2 3\n",
    "malformed_entry": "%%MatrixMarket matrix coordinate pattern general\n3 3 2\n1 x\n2 3\n",
    "malformed_after_nnz": "%%MatrixMarket matrix coordinate pattern general\n3 3 1\n1 2\nfoo bar\n",
    "crlf": "%%MatrixMarket matrix coordinate pattern general\r\n2 2 1\r\n1 2\r\n",
    "indented_comment": "%%MatrixMarket matrix coordinate pattern general\n2 2 1\n  % not a comment\n1 2\n",
    "size_missing": "%%MatrixMarket matrix coordinate pattern general\n% only comments\n",
    "nnz_zero": "%%MatrixMarket matrix coordinate pattern general\n2 2 0\n",
    "crlf_size": "%%MatrixMarket matrix coordinate pattern general\n2 2 1\r\n2 1\r\n"
}

EXPECT = {
    "txt/basic": [
        [
            0,
            1,
            2
        ],
        [
            1,
            2,
            0
        ]
    ],
    "txt/comments_blank": [
        [
            0,
            3
        ],
        [
            1,
            4
        ]
    ],
    "txt/crlf": [
        [
            0,
            2
        ],
        [
            1,
            3
        ]
    ],
    "txt/trailing_tokens": [
        [
            0,
            2
        ],
        [
            1,
            3
        ]
    ],
    "txt/junk_after_second": [
        [
            1,
            5
        ],
        [
            2,
            6
        ]
    ],
    "txt/junk_after_first": [
        [
            7
        ],
        [
            8
        ]
    ],
    "txt/no_space": "status 4",
    "txt/plus_sign": [
        [
            3
        ],
        [
            4
        ]
    ],
    "txt/minus_zero": [
        [
            0
        ],
        [
            5
        ]
    ],
    "txt/float": [
        [
            3
        ],
        [
            4
        ]
    ],
    "txt/single_token": [
        [
            3
        ],
        [
            4
        ]
    ],
    "txt/leading_ws": [
        [
            9
        ],
        [
            10
        ]
    ],
    "txt/tabs_vt": [
        [
            11
        ],
        [
            12
        ]
    ],
    "txt/no_trailing_newline": [
        [
            13
        ],
        [
            14
        ]
    ],
    "txt/big_ok": [
        [
            2147483647
        ],
        [
            0
        ]
    ],
    "txt/too_big": "status 4",
    "txt/negative": "status 4",
    "txt/overflow_ll": [
        [
            3
        ],
        [
            4
        ]
    ],
    "txt/comma": [
        [
            3
        ],
        [
            4
        ]
    ],
    "txt/unicode": [
        [
            5
        ],
        [
            6
        ]
    ],
    "mtx/general": [
        [
            0,
            2
        ],
        [
            1,
            0
        ]
    ],
    "mtx/symmetric": [
        [
            0,
            1,
            1,
            2,
            0
        ],
        [
            1,
            0,
            1,
            0,
            2
        ]
    ],
    "mtx/values": [
        [
            0,
            1
        ],
        [
            1,
            2
        ]
    ],
    "mtx/extra_lines": [
        [
            0
        ],
        [
            1
        ]
    ],
    "mtx/too_few": "status 4",
    "mtx/out_of_range": "status 4",
    "mtx/zero_index": "status 4",
    "mtx/bad_header": "status 4",
    "mtx/array_format": "status 4",
    "mtx/caps": [
        [
            0,
            1
        ],
        [
            1,
            0
        ]
    ],
    "mtx/comment_in_body": [
        [
            0,
            1
        ],
        [
            1,
            2
        ]
    ],
    "mtx/malformed_entry": "status 4",
    "mtx/malformed_after_nnz": [
        [
            0
        ],
        [
            1
        ]
    ],
    "mtx/crlf": [
        [
            0
        ],
        [
            1
        ]
    ],
    "mtx/indented_comment": "status 4",
    "mtx/size_missing": "status 4",
    "mtx/nnz_zero": [
        [],
        []
    ],
    "mtx/crlf_size": [
        [
            1
        ],
        [
            0
        ]
    ]
}


@pytest.mark.parametrize("kind,name", [("txt", k) for k in TXT] + [("mtx", k) for k in MTX])
def test_reader_edge_cases(tmp_path, kind, name):
    text = (TXT if kind == "txt" else MTX)[name]
    path = tmp_path / f"{name}.{kind}"
    path.write_bytes(text.encode("latin-1"))
    fmt = rtg.FMT_EDGE_TXT if kind == "txt" else rtg.FMT_MTX
    want = EXPECT[f"{kind}/{name}"]
    if isinstance(want, str):
        with pytest.raises(rtg.RtgError) as e:
            rtg.edges_read(str(path), fmt)
        assert e.value.status == int(want.split()[1])
    else:
        s, d = rtg.edges_read(str(path), fmt)
        assert [s.tolist(), d.tolist()] == want


def test_large_text_file_parses_in_parallel_pieces(tmp_path):
    """A file of many pieces (several MB, cut into per-thread pieces at newlines) gives the
    edges in file order, comment lines skipped wherever the cuts fall."""
    import numpy as np
    rng = np.random.default_rng(7)
    s = rng.integers(0, 2**31 - 1, 600_000, dtype=np.int64)
    d = rng.integers(0, 2**31 - 1, 600_000, dtype=np.int64)
    rows = [f"{a} {b}" if i % 97 else f"# {a} {b}" for i, (a, b) in enumerate(zip(s, d))]
    path = tmp_path / "big.txt"
    path.write_text("\n".join(rows) + "\n")
    keep = np.arange(len(s)) % 97 != 0
    gs, gd = rtg.edges_read(str(path), rtg.FMT_EDGE_TXT)
    assert np.array_equal(gs, s[keep].astype(np.uint32))
    assert np.array_equal(gd, d[keep].astype(np.uint32))


def test_large_mtx_file_in_parallel_pieces(tmp_path):
    """A symmetric MatrixMarket file of several MB (entry lines cut into per-thread pieces):
    comments anywhere, mirrored off-diagonal entries in file order, a malformed line after
    the nnz entries ignored, one before the last of them a format error."""
    import numpy as np
    rng = np.random.default_rng(8)
    n, nnz = 5000, 400_000
    r = rng.integers(1, n + 1, nnz)
    c = rng.integers(1, n + 1, nnz)
    rows = []
    for i, (a, b) in enumerate(zip(r, c)):
        if i % 101 == 0:
            rows.append("% a comment")
        rows.append(f"{a} {b}")
    head = f"%%MatrixMarket matrix coordinate pattern symmetric\n{n} {n} {nnz}\n"
    want_s, want_d = [], []
    for a, b in zip(r, c):
        want_s.append(a - 1)
        want_d.append(b - 1)
        if a != b:
            want_s.append(b - 1)
            want_d.append(a - 1)
    path = tmp_path / "big.mtx"
    path.write_text(head + "\n".join(rows) + "\nnot an entry\n1 1\n")
    gs, gd = rtg.edges_read(str(path), rtg.FMT_MTX)
    assert np.array_equal(gs, np.array(want_s, np.uint32))
    assert np.array_equal(gd, np.array(want_d, np.uint32))
    rows[-2] = "1 x"  # the next-to-last entry line malformed: fewer than nnz entries
    path.write_text(head + "\n".join(rows) + "\n")
    with pytest.raises(rtg.RtgError) as e:
        rtg.edges_read(str(path), rtg.FMT_MTX)
    assert e.value.status == rtg.ERR_FORMAT


_LIMITED_CHILD = r"""
import ctypes as C, os, resource, sys
import rtg
path, fmt, share = sys.argv[1], int(sys.argv[2]), float(sys.argv[3])
vm = [int(l.split()[1]) for l in open('/proc/self/status') if l.startswith('VmSize:')][0] * 1024
# share 1: room for the file itself, not for the parsed edges beside it; share 0.5: not
# even for the file
room = int(os.path.getsize(path) * share) + (24 << 20 if share >= 1 else 0)
resource.setrlimit(resource.RLIMIT_AS, (vm + room, vm + room))
m = C.c_uint64(0)
if fmt < 0:
    print(rtg.lib.rtg_graph_file_check(path.encode()))
else:
    print(rtg.lib.rtg_edges_read(path.encode(), fmt, C.byref(m), None, None))
"""


def test_host_allocation_failure_is_a_status(tmp_path):
    """A reader or the cache check that runs out of host memory returns RTG_ERR_OOM (the
    child limits its own address space to the file plus a little), rather than ending the
    process with an exception through the C boundary."""
    import os
    import subprocess
    import sys

    import numpy as np

    rng = np.random.default_rng(2)
    e = rng.integers(0, 1 << 20, size=(3_000_000, 2))
    txt = tmp_path / "big.txt"
    np.savetxt(txt, e, fmt="%d")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    pkg = os.path.dirname(os.path.dirname(rtg.__file__))
    env["PYTHONPATH"] = pkg + os.pathsep + env.get("PYTHONPATH", "")

    def limited(path, fmt, share):
        r = subprocess.run([sys.executable, "-c", _LIMITED_CHILD, str(path), str(fmt), str(share)],
                           env=env, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        return int(r.stdout.split()[-1])

    # the parse pieces fail (inside the parallel region), then the file buffer itself
    assert limited(txt, rtg.FMT_EDGE_TXT, 1.0) == rtg.ERR_OOM
    assert limited(txt, rtg.FMT_EDGE_TXT, 0.5) == rtg.ERR_OOM
    # a cache file larger than the room left
    from cache_forms import cache_file, counting_form
    s, d = rtg.gen_rmat(17, 16, seed=3)
    cf = tmp_path / "g.rtgcsr"
    cf.write_bytes(cache_file(*counting_form(s, d)))
    assert rtg.lib.rtg_graph_file_check(str(cf).encode()) == rtg.OK
    assert limited(cf, -1, 0.5) == rtg.ERR_OOM
    # the same file without the limit reads
    assert len(rtg.edges_read(str(txt), rtg.FMT_EDGE_TXT)[0]) == len(e)
