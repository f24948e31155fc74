"""ctypes binding of librtg (include/rtg.h) for tests, benchmarks and scripting.

The library is loaded from rt-graph_gb300/lib/librtg.so (built in-tree by
rt-graph_gb300/build.py). There is no fallback: if the library is missing, importing this
module raises, and every counting call goes through the CUDA kernels of librtg.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent.parent
LIB_PATH = Path(os.environ.get("RTG_LIB", PKG / "lib" / "librtg.so"))

if not LIB_PATH.exists():
    raise ImportError(f"librtg not built: {LIB_PATH} is missing (run rt-graph_gb300/build.py)")

lib = C.CDLL(str(LIB_PATH))

# ---------------------------------------------------------------- constants
OK, ERR_INVALID_ARG, ERR_OOM, ERR_IO, ERR_FORMAT, ERR_DEVICE, ERR_TIMEOUT, ERR_CANCELLED, \
    ERR_STATE, ERR_BUSY = range(10)
FMT_EDGE_BIN, FMT_EDGE_TXT, FMT_MTX, FMT_RTG_CSR = 0, 1, 2, 3
ORIENT_DEGREE, ORIENT_DEGREE_RAW_REF, ORIENT_SYMMETRIC = 0, 1, 2
TC_PLAIN, TC_BATCHED, TC_BUCKETED = 0, 1, 2
TC_CORE_NONE = 0xFFFFFFFF     # rtg_config.tc_core_ranks: no dense core
TC_CORE_MAX_RANKS = 32768
SI_AUTO, SI_MERGE, SI_SEARCH, SI_BITMAP, SI_PLAIN = 0, 1, 2, 3, 4
PAIRS_DEVICE, OUT_DEVICE = 0x100, 0x200


class Timing(C.Structure):
    _fields_ = [("h2d_ms", C.c_double), ("build_ms", C.c_double), ("count_ms", C.c_double),
                ("main_kernel_ms", C.c_double), ("d2h_ms", C.c_double),
                ("total_ms", C.c_double), ("kernel_launches", C.c_uint64),
                ("algo_bytes", C.c_uint64), ("h2d_bytes", C.c_uint64),
                ("d2h_bytes", C.c_uint64), ("core_ms", C.c_double),
                ("core_ranks", C.c_uint32), ("reserved", C.c_uint32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class GraphInfo(C.Structure):
    _fields_ = [("n", C.c_uint32), ("m_input", C.c_uint64), ("m", C.c_uint64),
                ("max_out_degree", C.c_uint32), ("work_elems", C.c_uint64),
                ("orient", C.c_int32), ("has_symmetric", C.c_int32), ("n_sym", C.c_uint32),
                ("m_sym", C.c_uint64)]


class Config(C.Structure):
    _fields_ = [(k, C.c_uint32) for k in (
        "tc_block_warps", "tc_item_edges", "tc_region_words", "tc_blocks_per_sm",
        "si_block_warps", "si_search_ratio", "si_stage_slots", "si_stage_bytes",
        "si_blocks_per_sm", "si_skew_stream", "si_form", "tc_core_ranks")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class DatasetInfo(C.Structure):
    _fields_ = [("num_a", C.c_uint32), ("num_b", C.c_uint32), ("max_element", C.c_uint32),
                ("intersection", C.c_uint32), ("elems", C.c_uint64)]


class TuneResult(C.Structure):
    _fields_ = [("best", Config), ("best_ms", C.c_double), ("default_ms", C.c_double),
                ("candidates", C.c_uint32), ("rejected", C.c_uint32),
                ("from_cache", C.c_uint32), ("reserved", C.c_uint32)]

    def as_dict(self) -> dict:
        return {"best": self.best.as_dict(), "best_ms": self.best_ms,
                "default_ms": self.default_ms, "candidates": self.candidates,
                "rejected": self.rejected, "from_cache": bool(self.from_cache)}


class ServeConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_batch_pairs", C.c_uint32),
                ("si_slots", C.c_uint32), ("max_graphs", C.c_uint32), ("flags", C.c_uint32),
                ("inject_fail_launch", C.c_uint32), ("reserved", C.c_uint32)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("kind", C.c_uint32), ("graph", C.c_uint32),
                ("launches", C.c_uint32), ("batch_requests", C.c_uint32),
                ("reserved", C.c_uint32), ("npairs", C.c_uint64), ("triangles", C.c_uint64),
                ("latency_ms", C.c_double), ("queue_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class ServeStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in (
        "submitted", "completed", "failed", "cancelled", "tc_launches", "tc_coalesced",
        "si_launches", "si_pairs", "max_requests_per_launch", "max_inflight_launches",
        "resident_graphs", "resident_bytes", "plan_bytes", "buffer_bytes", "budget_bytes",
        "plan_evictions", "admission_waits", "tc_direct")]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


P = C.c_void_p
u32p = C.POINTER(C.c_uint32)
u64p = C.POINTER(C.c_uint64)
i32p = C.POINTER(C.c_int32)

_SIGS = {
    "rtg_init": (C.c_int, [C.c_int, C.POINTER(P)]),
    "rtg_destroy": (None, [P]),
    "rtg_last_error": (C.c_char_p, [P]),
    "rtg_status_str": (C.c_char_p, [C.c_int]),
    "rtg_abi_version": (C.c_int, []),
    "rtg_set_config": (C.c_int, [P, C.POINTER(Config)]),
    "rtg_get_config": (C.c_int, [P, C.POINTER(Config)]),
    "rtg_kernel_launches": (C.c_uint64, [P]),
    "rtg_synchronize": (C.c_int, [P]),
    "rtg_flush_l2": (C.c_int, [P]),
    "rtg_device_info": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "rtg_host_alloc": (C.c_int, [P, C.c_size_t, C.POINTER(P)]),
    "rtg_host_free": (None, [P]),
    "rtg_graph_from_host_edges": (C.c_int, [P, P, P, C.c_uint64, C.POINTER(P)]),
    "rtg_graph_from_host_pairs": (C.c_int, [P, P, C.c_uint64, C.POINTER(P)]),
    "rtg_graph_from_device_edges": (C.c_int, [P, P, P, C.c_uint64, C.POINTER(P)]),
    "rtg_graph_load": (C.c_int, [P, C.c_char_p, C.c_int, C.POINTER(P)]),
    "rtg_csr_build": (C.c_int, [P, P, C.c_int]),
    "rtg_graph_from_host_csr": (C.c_int, [P, P, P, C.c_int32, C.c_int64, C.POINTER(P)]),
    "rtg_graph_info_get": (C.c_int, [P, C.POINTER(GraphInfo)]),
    "rtg_csr_view": (C.c_int, [P, C.c_int, C.POINTER(P), C.POINTER(P), u32p, u64p]),
    "rtg_csr_to_host": (C.c_int, [P, P, C.c_int, P, P]),
    "rtg_graph_release_edges": (C.c_int, [P]),
    "rtg_graph_device_bytes": (C.c_uint64, [P]),
    "rtg_graph_file_check": (C.c_int, [C.c_char_p]),
    "rtg_graph_save": (C.c_int, [P, P, C.c_char_p]),
    "rtg_graph_destroy": (None, [P]),
    "rtg_tc_count": (C.c_int, [P, P, C.c_int, u64p, C.POINTER(Timing)]),
    "rtg_tc_count_host_edges": (C.c_int, [P, P, P, C.c_uint64, C.c_int, C.c_int, u64p,
                                          C.POINTER(Timing)]),
    "rtg_tc_count_host_csr": (C.c_int, [P, P, P, C.c_int32, C.c_int64, C.c_int, u64p,
                                        C.POINTER(Timing)]),
    "rtg_graph_pair_count": (C.c_int, [P, P, P, P, C.c_uint64, P, C.c_uint32,
                                       C.POINTER(Timing)]),
    "rtg_debug_si_wait_limit": (C.c_int, [P, C.c_uint32, C.c_uint32]),
    "rtg_checked_build": (C.c_int, []),
    "rtg_debug_skip_file_checks": (C.c_int, [C.c_int]),
    "rtg_tc_count_device_csr_noalloc": (C.c_int, [P, P, C.c_uint32, C.c_uint64, u64p, P]),
    "rtg_sets_from_host": (C.c_int, [P, P, C.c_uint64, P, C.POINTER(P)]),
    "rtg_sets_from_host_u32": (C.c_int, [P, P, C.c_uint32, P, C.POINTER(P)]),
    "rtg_sets_count": (C.c_uint64, [P]),
    "rtg_sets_elems": (C.c_uint64, [P]),
    "rtg_sets_destroy": (None, [P]),
    "rtg_si_count": (C.c_int, [P, P, P, P, C.c_uint64, P, C.c_uint32, C.POINTER(Timing)]),
    "rtg_si_count_dense": (C.c_int, [P, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, P,
                                     C.c_uint32, C.POINTER(Timing)]),
    "rtg_si_materialize": (C.c_int, [P, P, P, P, C.c_uint64, P, P, C.c_uint64,
                                     C.POINTER(Timing)]),
    "rtg_tc_list": (C.c_int, [P, P, P, P, C.c_uint64, C.POINTER(Timing)]),
    "rtg_tune_tc": (C.c_int, [P, P, C.c_char_p, C.POINTER(TuneResult)]),
    "rtg_tune_si": (C.c_int, [P, P, P, P, C.c_uint64, C.c_char_p, C.POINTER(TuneResult)]),
    "rtg_serve_start": (C.c_int, [C.c_int, C.POINTER(ServeConfig), C.POINTER(P)]),
    "rtg_serve_stop": (None, [P]),
    "rtg_serve_last_error": (C.c_char_p, [P]),
    "rtg_serve_add_graph": (C.c_int, [P, P, P, C.c_uint64, u32p]),
    "rtg_serve_add_graph_file": (C.c_int, [P, C.c_char_p, C.c_int, u32p]),
    "rtg_serve_remove_graph": (C.c_int, [P, C.c_uint32]),
    "rtg_serve_save_graph": (C.c_int, [P, C.c_uint32, C.c_char_p]),
    "rtg_serve_graph_info": (C.c_int, [P, C.c_uint32, C.POINTER(GraphInfo)]),
    "rtg_serve_submit_tc": (C.c_int, [P, C.c_uint32, u64p]),
    "rtg_serve_submit_pairs": (C.c_int, [P, C.c_uint32, P, P, C.c_uint64, P, u64p]),
    "rtg_serve_poll": (C.c_int, [P, C.c_uint64, C.c_int32, C.POINTER(RequestInfo)]),
    "rtg_serve_wait_any": (C.c_int, [P, C.c_int32, u64p, C.POINTER(RequestInfo)]),
    "rtg_serve_cancel": (C.c_int, [P, C.c_uint64]),
    "rtg_serve_release": (C.c_int, [P]),
    "rtg_serve_drain": (C.c_int, [P, C.c_int32]),
    "rtg_serve_stats_get": (C.c_int, [P, C.POINTER(ServeStats)]),
    "rtg_dataset_read": (C.c_int, [C.c_char_p, C.POINTER(DatasetInfo), P, P]),
    "rtg_dataset_write": (C.c_int, [C.c_char_p, C.POINTER(DatasetInfo), P, P]),
    "rtg_edges_write_bin": (C.c_int, [C.c_char_p, P, P, C.c_uint64]),
    "rtg_edges_read": (C.c_int, [C.c_char_p, C.c_int, u64p, P, P]),
    "rtg_gen_rmat": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                               C.c_uint64, P, P]),
    "rtg_gen_ba": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint64, P, P, u64p]),
    "rtg_gen_hk": (C.c_int, [C.c_uint32, C.c_uint32, C.c_double, C.c_uint64, P, P, u64p]),
    "rtg_gen_si_pairs": (C.c_int, [C.c_uint64, C.c_double, C.c_double, C.c_uint32, C.c_uint32,
                                   C.c_uint32, C.c_double, C.c_uint64, P, u64p, P, P, P]),
}

for _name, (_res, _args) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args

EXPORTED = tuple(_SIGS)


class RtgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{lib.rtg_status_str(status).decode()} ({status}): {msg}")
        self.status = status


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(P)


def _check(status: int, ctx=None, what: str = "") -> None:
    if status != OK:
        msg = lib.rtg_last_error(ctx).decode() if ctx is not None else ""
        raise RtgError(status, f"{what}: {msg}" if what else msg)


# ---------------------------------------------------------------- generators

def gen_rmat(scale: int, edge_factor: int = 16, a=0.57, b=0.19, c=0.19, seed: int = 1):
    m = edge_factor << scale
    s = np.empty(m, np.uint32)
    d = np.empty(m, np.uint32)
    _check(lib.rtg_gen_rmat(scale, edge_factor, a, b, c, seed, _ptr(s), _ptr(d)), what="gen_rmat")
    return s, d


def gen_ba(n: int, m: int, seed: int = 1):
    cap = m * (n - m)
    s = np.empty(cap, np.uint32)
    d = np.empty(cap, np.uint32)
    out = C.c_uint64(0)
    _check(lib.rtg_gen_ba(n, m, seed, _ptr(s), _ptr(d), C.byref(out)), what="gen_ba")
    return s[: out.value].copy(), d[: out.value].copy()


def gen_hk(n: int, m: int, p: float, seed: int = 1):
    cap = m * (n - m)
    s = np.empty(cap, np.uint32)
    d = np.empty(cap, np.uint32)
    out = C.c_uint64(0)
    _check(lib.rtg_gen_hk(n, m, p, seed, _ptr(s), _ptr(d), C.byref(out)), what="gen_hk")
    return s[: out.value].copy(), d[: out.value].copy()


def gen_si_pairs(npairs: int, median=64.0, sigma=1.5, min_len=1, max_len=65536,
                 universe_log2=26, overlap_max=0.5, seed: int = 1):
    """Returns (offsets u64[2n+1], elems u32, pair_a, pair_b, expected u32[n])."""
    lens = np.empty(2 * npairs, np.uint32)
    total = C.c_uint64(0)
    _check(lib.rtg_gen_si_pairs(npairs, median, sigma, min_len, max_len, universe_log2,
                                overlap_max, seed, _ptr(lens), C.byref(total), None, None, None),
           what="gen_si_pairs(lengths)")
    off = np.empty(2 * npairs + 1, np.uint64)
    elems = np.empty(max(total.value, 1), np.uint32)
    exp = np.empty(npairs, np.uint32)
    _check(lib.rtg_gen_si_pairs(npairs, median, sigma, min_len, max_len, universe_log2,
                                overlap_max, seed, _ptr(lens), C.byref(total), _ptr(off),
                                _ptr(elems), _ptr(exp)), what="gen_si_pairs")
    pa = np.arange(0, 2 * npairs, 2, dtype=np.uint32)
    pb = pa + 1
    return off, elems[: total.value], pa, pb, exp


# ------------------------------------------------------------------- files

def edges_write_bin(path: str, s: np.ndarray, d: np.ndarray) -> None:
    s = np.ascontiguousarray(s, np.uint32)
    d = np.ascontiguousarray(d, np.uint32)
    _check(lib.rtg_edges_write_bin(str(path).encode(), _ptr(s), _ptr(d), len(s)),
           what="edges_write_bin")


def edges_read(path: str, fmt: int = FMT_EDGE_BIN):
    """One read: the arrays are sized from the file (8 bytes per binary edge; a text or
    MatrixMarket edge takes at least 3 bytes, two edges per symmetric MatrixMarket entry);
    a file that grows between the sizing and the read falls back to the two-call form."""
    try:
        size = os.path.getsize(path)
    except OSError:
        size = -1
    if size >= 0:
        cap = size // 8 if fmt == FMT_EDGE_BIN else (size // 3 + 1) * (2 if fmt == FMT_MTX else 1)
        s = np.empty(max(cap, 1), np.uint32)
        d = np.empty(max(cap, 1), np.uint32)
        m = C.c_uint64(cap)
        st = lib.rtg_edges_read(str(path).encode(), fmt, C.byref(m), _ptr(s), _ptr(d))
        if st == OK:
            return s[: m.value].copy(), d[: m.value].copy()
        if st != ERR_INVALID_ARG:
            _check(st, what="edges_read")
    m = C.c_uint64(0)
    _check(lib.rtg_edges_read(str(path).encode(), fmt, C.byref(m), None, None), what="edges_read")
    s = np.empty(max(m.value, 1), np.uint32)
    d = np.empty(max(m.value, 1), np.uint32)
    _check(lib.rtg_edges_read(str(path).encode(), fmt, C.byref(m), _ptr(s), _ptr(d)),
           what="edges_read")
    return s[: m.value], d[: m.value]


def dataset_read(path: str):
    info = DatasetInfo()
    _check(lib.rtg_dataset_read(str(path).encode(), C.byref(info), None, None), what="dataset_read")
    off = np.empty(info.num_a + info.num_b + 1, np.uint32)
    el = np.empty(max(info.elems, 1), np.uint32)
    _check(lib.rtg_dataset_read(str(path).encode(), C.byref(info), _ptr(off), _ptr(el)),
           what="dataset_read")
    return info, off, el[: info.elems]


def dataset_write(path: str, info: DatasetInfo, off: np.ndarray, el: np.ndarray) -> None:
    off = np.ascontiguousarray(off, np.uint32)
    el = np.ascontiguousarray(el, np.uint32)
    _check(lib.rtg_dataset_write(str(path).encode(), C.byref(info), _ptr(off), _ptr(el)),
           what="dataset_write")


# ---------------------------------------------------------------- context

def device_available() -> bool:
    ctx = P()
    st = lib.rtg_init(0, C.byref(ctx))
    if st == OK:
        lib.rtg_destroy(ctx)
        return True
    return False


class Context:
    def __init__(self, device: int = 0):
        self.h = P()
        self.children = weakref.WeakSet()   # graphs / set collections made on this context
        st = lib.rtg_init(device, C.byref(self.h))
        if st != OK:
            raise RtgError(st, f"rtg_init(device={device}) failed")

    def close(self) -> None:
        if self.h:
            for ch in list(self.children):
                ch.close()
            lib.rtg_destroy(self.h)
            self.h = P()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st: int, what: str = "") -> None:
        _check(st, self.h, what)

    @property
    def launches(self) -> int:
        return lib.rtg_kernel_launches(self.h)

    def config(self) -> Config:
        c = Config()
        self.check(lib.rtg_get_config(self.h, C.byref(c)))
        return c

    def set_config(self, **kw) -> None:
        c = self.config()
        for k, v in kw.items():
            setattr(c, k, int(v))
        self.check(lib.rtg_set_config(self.h, C.byref(c)), "set_config")

    def sync(self) -> None:
        self.check(lib.rtg_synchronize(self.h), "synchronize")

    def flush_l2(self) -> None:
        self.check(lib.rtg_flush_l2(self.h), "flush_l2")

    def device_info(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        self.check(lib.rtg_device_info(self.h, *[C.byref(x) for x in v]))
        return dict(sm_count=v[0].value, smem_optin=v[1].value, cc=(v[2].value, v[3].value))

    def host_array(self, n: int, dtype) -> np.ndarray:
        """Pinned host array (freed with the returned array's owner object)."""
        dtype = np.dtype(dtype)
        p = P()
        self.check(lib.rtg_host_alloc(self.h, max(n, 1) * dtype.itemsize, C.byref(p)),
                   "host_alloc")
        buf = (C.c_char * (max(n, 1) * dtype.itemsize)).from_address(p.value)
        arr = np.frombuffer(buf, dtype=dtype, count=n)
        _Pinned.keep[id(arr)] = p
        return arr

    # graphs
    def graph_from_edges(self, s: np.ndarray, d: np.ndarray) -> "Graph":
        s = np.ascontiguousarray(s, np.uint32)
        d = np.ascontiguousarray(d, np.uint32)
        g = P()
        self.check(lib.rtg_graph_from_host_edges(self.h, _ptr(s), _ptr(d), len(s), C.byref(g)),
                   "graph_from_host_edges")
        self.sync()
        return Graph(self, g)

    def graph_from_pairs(self, pairs: np.ndarray) -> "Graph":
        pairs = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        g = P()
        self.check(lib.rtg_graph_from_host_pairs(self.h, _ptr(pairs), len(pairs), C.byref(g)),
                   "graph_from_host_pairs")
        return Graph(self, g)

    def graph_load(self, path: str, fmt: int = FMT_EDGE_BIN) -> "Graph":
        g = P()
        self.check(lib.rtg_graph_load(self.h, str(path).encode(), fmt, C.byref(g)), "graph_load")
        return Graph(self, g)

    def graph_from_csr(self, offsets: np.ndarray, adjs: np.ndarray) -> "Graph":
        offsets = np.ascontiguousarray(offsets, np.int32)
        adjs = np.ascontiguousarray(adjs, np.int32)
        g = P()
        self.check(lib.rtg_graph_from_host_csr(self.h, _ptr(offsets), _ptr(adjs),
                                               len(offsets) - 1, len(adjs), C.byref(g)),
                   "graph_from_host_csr")
        return Graph(self, g)

    def tc_count_host_edges(self, s, d, orient=ORIENT_DEGREE, mode=TC_BATCHED):
        s = np.ascontiguousarray(s, np.uint32)
        d = np.ascontiguousarray(d, np.uint32)
        out = C.c_uint64(0)
        t = Timing()
        self.check(lib.rtg_tc_count_host_edges(self.h, _ptr(s), _ptr(d), len(s), orient, mode,
                                               C.byref(out), C.byref(t)), "tc_count_host_edges")
        return out.value, t

    def tc_count_host_csr(self, offsets, adjs, mode=TC_BATCHED):
        offsets = np.ascontiguousarray(offsets, np.int32)
        adjs = np.ascontiguousarray(adjs, np.int32)
        out = C.c_uint64(0)
        t = Timing()
        self.check(lib.rtg_tc_count_host_csr(self.h, _ptr(offsets), _ptr(adjs),
                                             len(offsets) - 1, len(adjs), mode, C.byref(out),
                                             C.byref(t)), "tc_count_host_csr")
        return out.value, t

    # sets
    def sets(self, offsets: np.ndarray, elems: np.ndarray) -> "Sets":
        h = P()
        if offsets.dtype == np.uint32:
            offsets = np.ascontiguousarray(offsets)
            self.check(lib.rtg_sets_from_host_u32(self.h, _ptr(offsets), len(offsets) - 1,
                                                  _ptr(np.ascontiguousarray(elems, np.uint32)),
                                                  C.byref(h)), "sets_from_host_u32")
        else:
            offsets = np.ascontiguousarray(offsets, np.uint64)
            elems = np.ascontiguousarray(elems, np.uint32)
            self.check(lib.rtg_sets_from_host(self.h, _ptr(offsets), len(offsets) - 1,
                                              _ptr(elems), C.byref(h)), "sets_from_host")
        return Sets(self, h)


class _Pinned:
    keep: dict = {}


class Graph:
    def __init__(self, ctx: Context, h):
        self.ctx = ctx
        self.h = h
        ctx.children.add(self)

    def close(self) -> None:
        if self.h:
            if self.ctx.h:   # a closed context has already released its graphs
                lib.rtg_graph_destroy(self.h)
            self.h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, orient: int = ORIENT_DEGREE) -> "Graph":
        self.ctx.check(lib.rtg_csr_build(self.ctx.h, self.h, orient), "csr_build")
        return self

    def info(self) -> GraphInfo:
        i = GraphInfo()
        self.ctx.check(lib.rtg_graph_info_get(self.h, C.byref(i)))
        return i

    def save(self, path: str) -> None:
        """Write the graph's CSRs to a cache file (read back with FMT_RTG_CSR)."""
        self.ctx.check(lib.rtg_graph_save(self.ctx.h, self.h, str(path).encode()), "graph_save")

    def tune(self, cache: str | None = None) -> dict:
        """Autotune the batched count's schedule for this graph (set on the context)."""
        r = TuneResult()
        self.ctx.check(lib.rtg_tune_tc(self.ctx.h, self.h, cache.encode() if cache else None,
                                       C.byref(r)), "tune_tc")
        return r.as_dict()

    def csr(self, symmetric: bool = False):
        i = self.info()
        n, m = (i.n_sym, i.m_sym) if symmetric else (i.n, i.m)
        off = np.empty(n + 1, np.uint64)
        adj = np.empty(max(m, 1), np.uint32)
        self.ctx.check(lib.rtg_csr_to_host(self.ctx.h, self.h, int(symmetric), _ptr(off),
                                           _ptr(adj)), "csr_to_host")
        return off, adj[:m]

    def release_edges(self) -> None:
        self.ctx.check(lib.rtg_graph_release_edges(self.h))

    def device_bytes(self) -> int:
        return lib.rtg_graph_device_bytes(self.h)

    def tc_list(self, capacity: int | None = None):
        """Per-edge triangle lists on the oriented CSR: (offsets u64[m+1], w u32[T], timing);
        the triangles of edge e = (u -> v) of csr() are (u, v, w[offsets[e]:offsets[e+1]])."""
        m = self.info().m
        off = np.empty(m + 1, np.uint64)
        if capacity is None:
            st = lib.rtg_tc_list(self.ctx.h, self.h, _ptr(off), None, 0, None)
            if st not in (OK, ERR_INVALID_ARG):
                self.ctx.check(st, "tc_list")
            capacity = int(off[-1])
        w = np.empty(max(capacity, 1), np.uint32)
        t = Timing()
        self.ctx.check(lib.rtg_tc_list(self.ctx.h, self.h, _ptr(off), _ptr(w), capacity,
                                       C.byref(t)), "tc_list")
        return off, w[: int(off[-1])], t

    def tc(self, mode: int = TC_BATCHED):
        out = C.c_uint64(0)
        t = Timing()
        self.ctx.check(lib.rtg_tc_count(self.ctx.h, self.h, mode, C.byref(out), C.byref(t)),
                       "tc_count")
        return out.value, t

    def pair_count(self, u: np.ndarray, v: np.ndarray, flags: int = 0):
        u = np.ascontiguousarray(u, np.uint32)
        v = np.ascontiguousarray(v, np.uint32)
        out = np.empty(max(len(u), 1), np.uint32)
        t = Timing()
        self.ctx.check(lib.rtg_graph_pair_count(self.ctx.h, self.h, _ptr(u), _ptr(v), len(u),
                                                _ptr(out), flags, C.byref(t)), "pair_count")
        return out[: len(u)], t


class Sets:
    def __init__(self, ctx: Context, h):
        self.ctx = ctx
        self.h = h
        ctx.children.add(self)

    def close(self) -> None:
        if self.h:
            if self.ctx.h:   # a closed context has already released its set collections
                lib.rtg_sets_destroy(self.h)
            self.h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nsets(self) -> int:
        return lib.rtg_sets_count(self.h)

    def count(self, pa: np.ndarray, pb: np.ndarray, family: int = SI_AUTO,
              out: np.ndarray | None = None):
        """Per-pair intersection sizes; `out` (uint32, len(pa)) may be a pinned host array."""
        pa = np.ascontiguousarray(pa, np.uint32)
        pb = np.ascontiguousarray(pb, np.uint32)
        if out is None:
            out = np.empty(max(len(pa), 1), np.uint32)
        elif out.dtype != np.uint32 or not out.flags.c_contiguous or len(out) < len(pa):
            raise ValueError("out must be a contiguous uint32 array of len(pa) elements")
        t = Timing()
        self.ctx.check(lib.rtg_si_count(self.ctx.h, self.h, _ptr(pa), _ptr(pb), len(pa),
                                        _ptr(out), family, C.byref(t)), "si_count")
        return out[: len(pa)], t

    def count_dense(self, a0: int, a1: int, b0: int, b1: int, family: int = SI_AUTO):
        out = np.empty(max((a1 - a0) * (b1 - b0), 1), np.uint32)
        t = Timing()
        self.ctx.check(lib.rtg_si_count_dense(self.ctx.h, self.h, a0, a1, b0, b1, _ptr(out),
                                              family, C.byref(t)), "si_count_dense")
        return out[: (a1 - a0) * (b1 - b0)], t

    def tune(self, pa: np.ndarray, pb: np.ndarray, cache: str | None = None) -> dict:
        """Autotune the batched SI schedule on these pairs (set on the context)."""
        pa = np.ascontiguousarray(pa, np.uint32)
        pb = np.ascontiguousarray(pb, np.uint32)
        r = TuneResult()
        self.ctx.check(lib.rtg_tune_si(self.ctx.h, self.h, _ptr(pa), _ptr(pb), len(pa),
                                       cache.encode() if cache else None, C.byref(r)),
                       "tune_si")
        return r.as_dict()

    def materialize(self, pa: np.ndarray, pb: np.ndarray, capacity: int | None = None):
        pa = np.ascontiguousarray(pa, np.uint32)
        pb = np.ascontiguousarray(pb, np.uint32)
        off = np.empty(len(pa) + 1, np.uint64)
        if capacity is None:
            # first call sizes the output (fails with INVALID_ARG, offsets filled)
            st = lib.rtg_si_materialize(self.ctx.h, self.h, _ptr(pa), _ptr(pb), len(pa),
                                        _ptr(off), None, 0, None)
            if st not in (OK, ERR_INVALID_ARG):
                self.ctx.check(st, "si_materialize")
            capacity = int(off[-1])
        el = np.empty(max(capacity, 1), np.uint32)
        t = Timing()
        self.ctx.check(lib.rtg_si_materialize(self.ctx.h, self.h, _ptr(pa), _ptr(pb), len(pa),
                                              _ptr(off), _ptr(el), capacity, C.byref(t)),
                       "si_materialize")
        return off, el[: int(off[-1])], t


# ---------------------------------------------------------------- serving

REQ_TC, REQ_PAIRS = 0, 1
SERVE_START_HELD = 0x1


class Server:
    """Request loop over resident graphs (rtg_serve_*). Pair arrays and output arrays of
    submitted requests are kept alive here until their request is collected."""

    def __init__(self, device: int = 0, budget_bytes: int = 0, max_batch_pairs: int = 0,
                 si_slots: int = 0, max_graphs: int = 0, held: bool = False,
                 inject_fail_launch: int = 0):
        cfg = ServeConfig(budget_bytes, max_batch_pairs, si_slots, max_graphs,
                          SERVE_START_HELD if held else 0, inject_fail_launch, 0)
        self.h = P()
        st = lib.rtg_serve_start(device, C.byref(cfg), C.byref(self.h))
        if st != OK:
            raise RtgError(st, "serve_start")
        self._keep: dict[int, tuple] = {}

    def _check(self, st: int, what: str) -> None:
        if st != OK:
            raise RtgError(st, f"{what}: {lib.rtg_serve_last_error(self.h).decode()}")

    def close(self) -> None:
        if self.h:
            lib.rtg_serve_stop(self.h)
            self.h = P()
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_graph(self, src: np.ndarray, dst: np.ndarray) -> int:
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        gid = C.c_uint32(0)
        self._check(lib.rtg_serve_add_graph(self.h, _ptr(src), _ptr(dst), len(src),
                                            C.byref(gid)), "serve_add_graph")
        return gid.value

    def add_graph_file(self, path: str, fmt: int = FMT_EDGE_BIN) -> int:
        gid = C.c_uint32(0)
        self._check(lib.rtg_serve_add_graph_file(self.h, str(path).encode(), fmt, C.byref(gid)),
                    "serve_add_graph_file")
        return gid.value

    def save_graph(self, gid: int, path: str) -> None:
        self._check(lib.rtg_serve_save_graph(self.h, gid, str(path).encode()), "serve_save_graph")

    def remove_graph(self, gid: int) -> None:
        self._check(lib.rtg_serve_remove_graph(self.h, gid), "serve_remove_graph")

    def graph_info(self, gid: int) -> GraphInfo:
        info = GraphInfo()
        self._check(lib.rtg_serve_graph_info(self.h, gid, C.byref(info)), "serve_graph_info")
        return info

    def submit_tc(self, gid: int) -> int:
        rid = C.c_uint64(0)
        self._check(lib.rtg_serve_submit_tc(self.h, gid, C.byref(rid)), "serve_submit_tc")
        return rid.value

    def submit_pairs(self, gid: int, u: np.ndarray, v: np.ndarray,
                     out: np.ndarray | None = None) -> tuple[int, np.ndarray]:
        u = np.ascontiguousarray(u, np.uint32)
        v = np.ascontiguousarray(v, np.uint32)
        if len(u) != len(v):
            raise ValueError("u and v differ in length")
        if out is None:
            out = np.empty(max(len(u), 1), np.uint32)
        rid = C.c_uint64(0)
        self._check(lib.rtg_serve_submit_pairs(self.h, gid, _ptr(u), _ptr(v), len(u), _ptr(out),
                                               C.byref(rid)), "serve_submit_pairs")
        self._keep[rid.value] = (u, v, out)
        return rid.value, out[: len(u)]

    def poll(self, rid: int, wait_ms: int = -1) -> dict | None:
        """Info of a completed request, or None while it runs (wait_ms 0 polls)."""
        info = RequestInfo()
        st = lib.rtg_serve_poll(self.h, rid, wait_ms, C.byref(info))
        if st == ERR_BUSY:
            return None
        self._check(st, "serve_poll")
        self._keep.pop(rid, None)
        return info.as_dict()

    def wait_any(self, wait_ms: int = -1) -> tuple[int, dict] | None:
        rid = C.c_uint64(0)
        info = RequestInfo()
        st = lib.rtg_serve_wait_any(self.h, wait_ms, C.byref(rid), C.byref(info))
        if st == ERR_BUSY:
            return None
        self._check(st, "serve_wait_any")
        self._keep.pop(rid.value, None)
        return rid.value, info.as_dict()

    def cancel(self, rid: int) -> None:
        self._check(lib.rtg_serve_cancel(self.h, rid), "serve_cancel")

    def release(self) -> None:
        self._check(lib.rtg_serve_release(self.h), "serve_release")

    def drain(self, wait_ms: int = -1) -> bool:
        st = lib.rtg_serve_drain(self.h, wait_ms)
        if st == ERR_BUSY:
            return False
        self._check(st, "serve_drain")
        return True

    def stats(self) -> dict:
        s = ServeStats()
        self._check(lib.rtg_serve_stats_get(self.h, C.byref(s)), "serve_stats")
        return s.as_dict()
