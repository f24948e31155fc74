"""C ABI and host logic, on CPU: the library loads and exports every declared symbol, status
codes, seeded generators, file formats. No kernel is launched here."""
from __future__ import annotations

import re
import subprocess

import numpy as np
import pytest

import oracle
import rtg
from conftest import REPO


def declared_symbols() -> set[str]:
    text = (REPO / "include" / "rtg.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(rtg_[a-z0-9_]+)\s*\(", text))


def test_every_declared_symbol_is_exported():
    out = subprocess.run(["nm", "-D", "--defined-only", str(rtg.LIB_PATH)], check=True,
                         capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    declared = declared_symbols()
    assert declared, "no declarations parsed"
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    unbound = declared - set(rtg.EXPORTED)
    assert not unbound, f"declared but not bound in rtg: {sorted(unbound)}"


def test_status_strings_and_version():
    assert rtg.lib.rtg_abi_version() == 3
    for s in range(10):
        assert rtg.lib.rtg_status_str(s)
    assert rtg.lib.rtg_status_str(99) == b"unknown status"


def test_init_reports_device_status_without_gpu():
    import ctypes as C
    h = C.c_void_p()
    st = rtg.lib.rtg_init(0, C.byref(h))
    if st == rtg.OK:
        rtg.lib.rtg_destroy(h)
        pytest.skip("a GPU is present")
    assert st == rtg.ERR_DEVICE
    assert rtg.lib.rtg_init(-1, C.byref(h)) in (rtg.ERR_INVALID_ARG, rtg.ERR_DEVICE)


def test_null_arguments_are_rejected():
    assert rtg.lib.rtg_init(0, None) == rtg.ERR_INVALID_ARG
    assert rtg.lib.rtg_set_config(None, None) == rtg.ERR_INVALID_ARG
    assert rtg.lib.rtg_tc_count(None, None, 0, None, None) == rtg.ERR_INVALID_ARG
    assert rtg.lib.rtg_si_count(None, None, None, None, 0, None, 0, None) == rtg.ERR_INVALID_ARG
    assert rtg.lib.rtg_gen_rmat(0, 16, 0.57, 0.19, 0.19, 1, None, None) == rtg.ERR_INVALID_ARG


def test_rmat_deterministic_and_distributed():
    s1, d1 = rtg.gen_rmat(12, 16, seed=9)
    s2, d2 = rtg.gen_rmat(12, 16, seed=9)
    s3, _ = rtg.gen_rmat(12, 16, seed=10)
    assert np.array_equal(s1, s2) and np.array_equal(d1, d2)
    assert not np.array_equal(s1, s3)
    assert len(s1) == 16 << 12 and s1.max() < (1 << 12) and d1.max() < (1 << 12)
    # quadrant a=0.57: the top bit of both endpoints is 0 for ~57% of samples
    top = ((s1 >> 11) == 0) & ((d1 >> 11) == 0)
    assert abs(top.mean() - 0.57) < 0.02


def test_ba_and_hk_shapes():
    s, d = rtg.gen_ba(2000, 5, seed=1)
    assert len(s) == 5 * (2000 - 5)
    assert (s != d).all()
    key = np.minimum(s, d).astype(np.uint64) << 32 | np.maximum(s, d)
    assert len(np.unique(key)) == len(key)
    s, d = rtg.gen_hk(3000, 6, 0.5, seed=2)
    assert len(s) <= 6 * (3000 - 6)
    assert (s != d).all()
    key = np.minimum(s, d).astype(np.uint64) << 32 | np.maximum(s, d)
    assert len(np.unique(key)) == len(key)
    # triad closure raises clustering above plain preferential attachment
    sb, db = rtg.gen_ba(3000, 6, seed=2)
    off_hk, adj_hk = oracle.degree_csr(s, d)
    off_ba, adj_ba = oracle.degree_csr(sb, db)
    assert oracle.tc_merge(off_hk, adj_hk) > 2 * oracle.tc_merge(off_ba, adj_ba)


def test_si_generator_known_answers():
    off, el, pa, pb, exp = rtg.gen_si_pairs(3000, seed=3)
    lens = np.diff(off.astype(np.int64))
    assert lens.min() >= 1 and lens.max() <= 65536
    assert el.max() < (1 << 26)
    for i in range(0, 6000, 7):
        seg = el[off[i]:off[i + 1]]
        assert (np.diff(seg.astype(np.int64)) > 0).all()
    got = oracle.si_pairs(off, el, pa, pb)
    assert np.array_equal(got, exp)
    short = np.minimum(lens[0::2], lens[1::2])
    assert (exp <= short // 2).all()
    # lognormal median ~64
    assert 50 < np.median(lens) < 80


def test_edge_file_roundtrips(tmp_path):
    s = np.array([0, 1, 2, 7], np.uint32)
    d = np.array([1, 2, 0, 7], np.uint32)
    rtg.edges_write_bin(str(tmp_path / "e.bin"), s, d)
    s2, d2 = rtg.edges_read(str(tmp_path / "e.bin"), rtg.FMT_EDGE_BIN)
    assert np.array_equal(s, s2) and np.array_equal(d, d2)
    (tmp_path / "e.txt").write_text("# snap header\n0 1\n1 2\nbad line\n2 0\n7 7\n")
    s2, d2 = rtg.edges_read(str(tmp_path / "e.txt"), rtg.FMT_EDGE_TXT)
    assert np.array_equal(s, s2) and np.array_equal(d, d2)
    (tmp_path / "e.mtx").write_text("%%MatrixMarket matrix coordinate pattern symmetric\n"
                                    "% x\n8 8 3\n2 1\n3 2\n8 8\n")
    s2, d2 = rtg.edges_read(str(tmp_path / "e.mtx"), rtg.FMT_MTX)
    assert list(zip(s2, d2)) == [(1, 0), (0, 1), (2, 1), (1, 2), (7, 7)]


def test_bad_files_are_reported(tmp_path):
    (tmp_path / "odd.bin").write_bytes(b"\x01\x02\x03")
    with pytest.raises(rtg.RtgError) as e:
        rtg.edges_read(str(tmp_path / "odd.bin"))
    assert e.value.status == rtg.ERR_FORMAT
    with pytest.raises(rtg.RtgError) as e:
        rtg.edges_read(str(tmp_path / "missing.bin"))
    assert e.value.status == rtg.ERR_IO
    (tmp_path / "zero.mtx").write_text("%%MatrixMarket matrix coordinate pattern general\n3 3 1\n0 1\n")
    with pytest.raises(rtg.RtgError) as e:
        rtg.edges_read(str(tmp_path / "zero.mtx"), rtg.FMT_MTX)
    assert e.value.status == rtg.ERR_FORMAT
    (tmp_path / "short.s_data").write_bytes(np.array([2, 1, 10], np.uint32).tobytes())
    with pytest.raises(rtg.RtgError) as e:
        rtg.dataset_read(str(tmp_path / "short.s_data"))
    assert e.value.status == rtg.ERR_FORMAT


def test_dataset_header_beyond_the_file(tmp_path):
    """A header that claims more sets than the file holds is refused before the offsets are
    allocated (2^33 sets would take 34 GB), and a header alone is a format error too."""
    for hdr in ([0xFFFFFFFF, 0xFFFFFFFF, 10, 0], [1 << 30, 0, 10, 0], [3, 2, 10, 0]):
        p = tmp_path / "big.s_data"
        p.write_bytes(np.array(hdr + [0, 1, 2], np.uint32).tobytes())
        with pytest.raises(rtg.RtgError) as e:
            rtg.dataset_read(str(p))
        assert e.value.status == rtg.ERR_FORMAT, hdr
    p.write_bytes(np.array([1, 1, 10, 0], np.uint32).tobytes())
    with pytest.raises(rtg.RtgError) as e:
        rtg.dataset_read(str(p))
    assert e.value.status == rtg.ERR_FORMAT
    # exactly the offsets and no elements: two empty sets
    p.write_bytes(np.array([1, 1, 10, 0, 0, 0, 0], np.uint32).tobytes())
    info, off, el = rtg.dataset_read(str(p))
    assert (info.num_a, info.num_b, info.elems) == (1, 1, 0) and list(off) == [0, 0, 0]


def test_dataset_roundtrip(tmp_path):
    info = rtg.DatasetInfo(2, 1, 100, 1, 5)
    off = np.array([0, 2, 4, 5], np.uint32)
    el = np.array([1, 5, 1, 6, 1], np.uint32)
    rtg.dataset_write(str(tmp_path / "x.s_data"), info, off, el)
    i2, o2, e2 = rtg.dataset_read(str(tmp_path / "x.s_data"))
    assert (i2.num_a, i2.num_b, i2.max_element, i2.intersection, i2.elems) == (2, 1, 100, 1, 5)
    assert np.array_equal(o2, off) and np.array_equal(e2, el)


def test_checked_build_variant_loads_and_flags_itself():
    """The checked library is a separate build: it reports itself and accepts the
    file-check test hook, which the product library refuses (no GPU call)."""
    import ctypes as C
    from pathlib import Path
    assert rtg.lib.rtg_checked_build() == 0
    assert rtg.lib.rtg_debug_skip_file_checks(1) == rtg.ERR_STATE
    checked = C.CDLL(str(Path(rtg.LIB_PATH).parent / "librtg_checked.so"))
    checked.rtg_debug_skip_file_checks.argtypes = [C.c_int]
    assert checked.rtg_checked_build() == 1
    assert checked.rtg_debug_skip_file_checks(1) == rtg.OK
    assert checked.rtg_debug_skip_file_checks(0) == rtg.OK


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of the public structs have the header's size and field offsets
    (a C program built with gcc against include/rtg.h prints them)."""
    import ctypes as C
    structs = {"rtg_config": rtg.Config, "rtg_timing": rtg.Timing,
               "rtg_graph_info": rtg.GraphInfo, "rtg_tune_result": rtg.TuneResult}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "rtg.h"', 'int main(void) {']
    for cname, py in structs.items():
        lines.append(f'printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(REPO / "include"), str(src), "-o", str(exe)],
                   check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True,
                               text=True).stdout.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_core_config_constants():
    assert rtg.TC_CORE_NONE == 0xFFFFFFFF
    assert rtg.TC_CORE_MAX_RANKS == 32768
    text = (REPO / "include" / "rtg.h").read_text()
    assert "#define RTG_TC_CORE_NONE 0xFFFFFFFFu" in text
    assert "#define RTG_TC_CORE_MAX_RANKS 32768u" in text
