"""The reference's own GPU triangle count as a same-box data point — TEST INFRASTRUCTURE.

oracle/build_ref.sh compiles the reference's tc/bs_tc/bs_tc.cu, unmodified, with its method
0 selected (oracle/ref_method0.h), into oracle/_ref/bs_tc_method0.cubin (device code only).
This module loads that cubin through the CUDA driver API (ctypes on libcuda, no other
library) and launches ListIntersectionKernel (bs_tc.cu:120-148) the way the reference's
CountOnGPU does (bs_tc.cu:309-317: 256 threads per block, at most 65,535 blocks, one thread
per oriented edge, uint32 counter), on an int32 oriented CSR. Used by bench.py's reference
arm; the library under test is not involved.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

CUBIN = Path(__file__).resolve().parent / "_ref" / "bs_tc_method0.cubin"
KERNEL = b"_Z22ListIntersectionKernelPiS_iiPj"  # ListIntersectionKernel(int*, int*, int, int, uint*)
BLOCK_SIZE, MAX_BLOCKS = 256, 65535         # bs_tc.cu:11-12


def available() -> tuple[bool, str]:
    if not CUBIN.exists():
        return False, ("the reference's GPU kernel was not built on this host (its sources are "
                       "not here; oracle/build_ref.sh builds it where they are)")
    try:
        C.CDLL("libcuda.so.1")
    except OSError:
        return False, "no CUDA driver library"
    return True, ""


class _Driver:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")

    def __call__(self, name: str, *args):
        r = getattr(self.cu, name)(*args)
        if r != 0:
            raise RuntimeError(f"{name} failed with CUDA driver error {r}")


def count(offsets: np.ndarray, adjs: np.ndarray, runs: int = 3, device: int = 0):
    """(triangles as the reference's uint32 counter, kernel milliseconds per run) of the
    reference's ListIntersectionKernel on the oriented CSR (offsets: nodes+1, adjs: edges)."""
    d = _Driver()
    off = np.ascontiguousarray(offsets, np.int32)
    adj = np.ascontiguousarray(adjs, np.int32)
    nodes, edges = len(off) - 1, len(adj)
    d("cuInit", 0)
    dev, ctx = C.c_int(), C.c_void_p()
    d("cuDeviceGet", C.byref(dev), device)
    d("cuDevicePrimaryCtxRetain", C.byref(ctx), dev)
    d("cuCtxPushCurrent_v2", ctx)
    mod, fn = C.c_void_p(), C.c_void_p()
    bufs = []
    try:
        d("cuModuleLoad", C.byref(mod), str(CUBIN).encode())
        d("cuModuleGetFunction", C.byref(fn), mod, KERNEL)

        def alloc(nbytes):
            p = C.c_uint64()
            d("cuMemAlloc_v2", C.byref(p), C.c_size_t(max(nbytes, 4)))
            bufs.append(p)
            return p

        d_adj, d_off, d_cnt = alloc(adj.nbytes), alloc(off.nbytes), alloc(4)
        d("cuMemcpyHtoD_v2", d_adj, adj.ctypes.data_as(C.c_void_p), C.c_size_t(adj.nbytes))
        d("cuMemcpyHtoD_v2", d_off, off.ctypes.data_as(C.c_void_p), C.c_size_t(off.nbytes))
        blocks = min((edges + BLOCK_SIZE - 1) // BLOCK_SIZE, MAX_BLOCKS) or 1
        a_nodes, a_threads = C.c_int(nodes), C.c_int(edges)
        params = (C.c_void_p * 5)(*[C.cast(C.byref(x), C.c_void_p)
                                    for x in (d_adj, d_off, a_nodes, a_threads, d_cnt)])
        e0, e1 = C.c_void_p(), C.c_void_p()
        d("cuEventCreate", C.byref(e0), 0)
        d("cuEventCreate", C.byref(e1), 0)
        times, total = [], 0
        for _ in range(1 + runs):  # the first launch is a warm-up
            d("cuMemsetD32_v2", d_cnt, 0, C.c_size_t(1))
            d("cuEventRecord", e0, None)
            d("cuLaunchKernel", fn, blocks, 1, 1, BLOCK_SIZE, 1, 1, 0, None, params, None)
            d("cuEventRecord", e1, None)
            d("cuEventSynchronize", e1)
            ms = C.c_float()
            d("cuEventElapsedTime", C.byref(ms), e0, e1)
            times.append(ms.value)
            h = np.zeros(1, np.uint32)
            d("cuMemcpyDtoH_v2", h.ctypes.data_as(C.c_void_p), d_cnt, C.c_size_t(4))
            total = int(h[0])
        d("cuEventDestroy_v2", e0)
        d("cuEventDestroy_v2", e1)
        return total, times[1:]
    finally:
        for p in bufs:
            d.cu.cuMemFree_v2(p)
        if mod.value:
            d.cu.cuModuleUnload(mod)
        d.cu.cuCtxPopCurrent_v2(C.byref(C.c_void_p()))
        d.cu.cuDevicePrimaryCtxRelease_v2(dev)
