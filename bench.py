#!/usr/bin/env python3
"""Benchmark: exact triangle count of an R-MAT scale-21 graph on one GB300.

Workload (the batched-TC configuration): R-MAT scale 21, edge factor 16 (2^25 samples),
(a,b,c,d) = (0.57,0.19,0.19,0.05), seed 42, symmetrised, deduplicated, self loops removed,
oriented by degree. A step is one exact uint64 count of the resident CSR:

  value   – edges/s = m / device time of the BATCHED count (dense-core stage + persistent
            streaming kernel in one CUDA graph), CSR resident in HBM, L2 flushed before
            every step (CUDA events).
  e2e     – the same metric through the public C ABI with host buffers:
            rtg_tc_count_host_edges (pinned host edges -> H2D -> GPU CSR build -> count ->
            D2H of the total), wall time per call.
  plain   – the PLAIN form (one launch per bucket, one warp per oriented edge, the
            reference's per-edge formulation) on the same CSR, for the batched/plain ratio.
  roofline– the persistent streaming kernel's own algorithmic bytes per launch (4 B per
            streamed suffix element, 8 B per streamed in-edge range, 4 B per out-list element
            marked, 16 B of offsets per vertex; only in-edges whose source lies below the
            dense core are streamed) over its CUDA-event duration against the measured HBM
            copy peak; beside it the per-edge work formula of the measurement plan
            (4 x sum over oriented edges of (d+(u) + d+(v)) + 8 m) over the whole count as a
            work-equivalent rate, and the DRAM traffic, issue activity and instructions per
            element from the committed ncu summary of the same kernel.
  core    – the dense-core stage of the same count: its top ranks, device time (matrix
            build + word-AND count), core edges, matrix bytes, and the 16-byte groups the
            core count sweeps (each read from L2 and ANDed with the staged row).
  cpu_baseline – the oracle's restatement of the reference's ListIntersectionKernel
            (bs_tc.cu:120-148) on the host cores, on a stride sample of source vertices.
  si      – summary of the batched set-intersection workload (1e6 pairs of sorted unique
            u32 lists, lengths lognormal with median 64 and sigma 1.5 clamped to [1, 65536],
            universe [0, 2^26), overlap uniform in [0, 0.5] of the shorter list, seed 1):
            pairs/s of the persistent staged kernel vs the PLAIN per-pair form, end to end
            through rtg_si_count, and its roofline. `--workload si` prints that workload
            alone as a full line (with its CPU baseline).

`--impl reference` times the reference's counting logic on the host cores: the oracle's
restatement of ListIntersectionKernel, on a stride sample of the same workload, which it
generates with the oracle's copy of the seeded generator, so that the library under test is
not loaded in that process. Beside it (`reference_gpu`) it times the reference's own GPU
kernel for the same count (ListIntersectionKernel, its method 0, compiled unmodified from
its sources by oracle/build_ref.sh into a cubin, launched through the CUDA driver API by
oracle/ref_gpu.py), when that cubin was built.
With torchrun (N>1) every rank runs an independent replica on its own GPU (the count does
not shard across GPUs here); rank 0 prints one line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "rt-graph_gb300"))
sys.path.insert(0, str(REPO))

WORKLOAD = dict(workload="rmat21_ef16_tc", scale=21, edge_factor=16, abcd=[0.57, 0.19, 0.19, 0.05],
                seed=42, orientation="degree (post-dedup)", counter="uint64")
METRIC = "TC edges/s"
UNIT = "edges/s"

SI_WORKLOAD = dict(workload="si_lognormal_1e6_pairs", npairs=1_000_000, length_median=64,
                   length_sigma=1.5, length_clamp=[1, 65536], universe="[0, 2^26)",
                   overlap="uniform [0, 0.5] of the shorter list", seed=1,
                   storage="CSR (u64 offsets, u32 elements) resident in HBM")
SI_METRIC = "batched intersections/s"
SI_UNIT = "pairs/s"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier / max / sum across ranks (torch.distributed when WORLD_SIZE > 1)."""

    def __init__(self, backend: str | None = None):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            td.init_process_group(backend=backend or "gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def reduce(self, x: float, op: str) -> float:
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX if op == "max" else self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


def aggregate(dist: Dist, units_local: float, ms_local: float) -> tuple[float, float]:
    """Whole-job throughput: units of all ranks / the slowest rank's time."""
    ms = dist.reduce(ms_local, "max")
    units = dist.reduce(units_local, "sum")
    return units / (ms / 1e3), ms


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes ~0.1 s to print its first sample: wait for it (at most 5 s)
            # so that the samples kept below fall inside the timed region
            t_end = time.monotonic() + 5.0
            while not self.lines and time.monotonic() < t_end and self.proc.poll() is None:
                time.sleep(0.005)
        except (FileNotFoundError, OSError):
            self.proc = None
        self.first = len(self.lines)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # samples taken after the timed region began; all of them when it was too short
        lines = self.lines[self.first:] or self.lines
        for line in lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for name, flag in zip(names, p[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        loaded = [x for x in sm if mx and x > 0.5 * mx] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_fields(name: str) -> dict:
    """Machine-readable `key: value` lines of a committed ncu summary (profiles/NAME.txt):
    dram_bytes_per_full_launch, issue_active, warp_instructions, ..."""
    p = REPO / "profiles" / f"{name}.txt"
    out = {}
    if not p.exists():
        return out
    for line in p.read_text().splitlines():
        if ":" not in line or line.startswith(" "):
            continue
        k, v = line.split(":", 1)
        try:
            out[k.strip()] = float(v.split()[0])
        except (ValueError, IndexError):
            continue
    return out


def profile_traffic(name: str):
    """DRAM bytes per launch of the dominant kernel from a committed ncu summary."""
    v = profile_fields(name).get("dram_bytes_per_full_launch")
    return int(v) if v else None


def gen_workload(with_library: bool = True):
    """The seeded R-MAT edge list: the library's generator, or the oracle's copy of the same
    stream (identical arrays) for the reference arm, which does not load the library."""
    if with_library:
        import rtg
        gen = rtg.gen_rmat
    else:
        import oracle
        gen = oracle.gen_rmat
    return gen(WORKLOAD["scale"], WORKLOAD["edge_factor"], *WORKLOAD["abcd"][:3],
               seed=WORKLOAD["seed"])


def tc_config(n: int, m: int, m_input: int, max_out: int) -> dict:
    """The workload identity both arms report (same keys, same values)."""
    return dict(WORKLOAD, n=int(n), m=int(m), m_input=int(m_input), max_out_degree=int(max_out))


def tc_split(off: np.ndarray, adj: np.ndarray, K: int) -> dict:
    """How the batched count of the oriented CSR (kept ids) splits its work when the top K
    ranks form the dense core. Ranks order vertices by (degree, id), the orientation's own
    order, so the counting form is this CSR relabelled by rank and c0 = n - K.

    Streaming kernel: the in-edges u->v with u below the core and d+(v) >= 1 (heads without
    out-edges get no work item); each streams the suffix of N+(u) after v (4 B per element)
    and reads its range (8 B); every head with streamed in-edges marks its out-list once
    (4 B per element); two u64 offsets per vertex. Core stage: the edges u->v of core rows
    except the last of each row, each sweeping the 16-byte groups of N+(v)'s rank span up to
    u's last group (kernel k_tc_core)."""
    off = off.astype(np.int64)
    n = len(off) - 1
    dplus = np.diff(off)
    m = int(off[-1])
    src = np.repeat(np.arange(n, dtype=np.int64), dplus)
    dst = adj[:m].astype(np.int64)
    deg = dplus + np.bincount(dst, minlength=n)
    rank = np.empty(n, np.int64)
    rank[np.lexsort((np.arange(n), deg))] = np.arange(n)
    # rows in rank order (the counting form's rows, still indexed by kept source ids)
    dst = dst[np.lexsort((rank[dst], src))]
    c0 = n - K
    pos = np.arange(m, dtype=np.int64)
    suffix = off[src + 1] - pos - 1
    head_ok = dplus[dst] >= 1
    streamed = (rank[src] < c0) & head_ok
    sdeg = np.bincount(dst[streamed], minlength=n)
    out = {"stream_elems": int(suffix[streamed].sum()), "stream_inedges": int(streamed.sum()),
           "mark_elems": int(dplus[(sdeg >= 1) & (dplus >= 1)].sum())}
    out["stream_bytes"] = (4 * out["stream_elems"] + 8 * out["stream_inedges"] +
                           4 * out["mark_elems"] + 16 * n)
    out["core_edges"] = int((rank[src] >= c0).sum())
    rw = 4
    while rw * 32 < K:
        rw <<= 1
    out["matrix_bytes"] = K * rw * 4 if K else 0
    if K:
        rdst = rank[dst]
        # rank span of every out-list: its first and last element in rank order
        nz = dplus > 0
        lo = np.full(n, -1, np.int64)
        hi = np.full(n, -1, np.int64)
        lo[nz] = rdst[off[:-1][nz]]
        hi[nz] = rdst[off[1:][nz] - 1]
        sel = (rank[src] >= c0) & (pos != off[src + 1] - 1) & head_ok
        u, v = src[sel], dst[sel]
        g0 = ((lo[v] - c0) >> 5) >> 2
        g1 = np.minimum(((hi[v] - c0) >> 5) >> 2, ((hi[u] - c0) >> 5) >> 2)
        out["core_groups"] = int(np.where(g1 >= g0, g1 - g0 + 1, 0).sum())
    else:
        out["core_groups"] = 0
    return out


def cpu_baseline_tc(off: np.ndarray, adj: np.ndarray, target_s: float = 15.0) -> dict:
    """The oracle's ListIntersectionKernel restatement on a stride sample of source
    vertices, all host threads. Returns edges/s on the sampled oriented edges."""
    import oracle
    n = len(off) - 1
    threads = os.cpu_count() or 1
    off32 = off.astype(np.int32)
    adj32 = adj.astype(np.int32)
    stride = 256
    while True:
        rows = np.arange(0, n, stride, dtype=np.int32)
        edges = int((off32[rows + 1] - off32[rows]).sum())
        t0 = time.perf_counter()
        oracle.tc_bsearch_rows(off32, adj32, rows, threads)
        dt = time.perf_counter() - t0
        if dt * 4 > target_s or stride == 1:
            break
        stride = max(1, stride // 4)
    return {"value": edges / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"every {stride}-th source vertex ({edges} oriented edges, {dt:.1f} s), "
                      "ListIntersectionKernel restatement (per edge x binary search), OpenMP"}


def gen_si_workload(with_library: bool = True):
    if with_library:
        import rtg
        gen = rtg.gen_si_pairs
    else:
        import oracle
        gen = oracle.gen_si_pairs
    return gen(SI_WORKLOAD["npairs"], median=64.0, sigma=1.5, min_len=1, max_len=65536,
               universe_log2=26, overlap_max=0.5, seed=SI_WORKLOAD["seed"])


def dram_view(traffic, kernel_ms: float, peak_gbs: float, note: str) -> dict:
    """The dominant kernel's measured DRAM traffic (from its ncu summary) per live launch
    time, beside the algorithmic-bytes figure."""
    if not traffic or not kernel_ms:
        return {"note": note}
    gbs = traffic / (kernel_ms / 1e3) / 1e9
    return {"dram_gbs": gbs, "dram_frac": gbs / peak_gbs, "note": note}


def si_algo_bytes(off: np.ndarray, pa: np.ndarray, pb: np.ndarray) -> int:
    """4 bytes per element of both lists of every pair + 16 B of pair ids + 4 B of count."""
    lens = np.diff(off.astype(np.int64))
    return int(4 * (lens[pa].sum() + lens[pb].sum()) + 20 * len(pa))


def cpu_baseline_si(off, el, pa, pb, target_s: float = 10.0) -> dict:
    """The oracle's per-pair merge (the reference's SerialIntersection, ip.cu:266-287) on a
    prefix sample of the pairs, split over all host threads."""
    import oracle
    threads = os.cpu_count() or 1
    k = 4096
    while True:
        t0 = time.perf_counter()
        oracle.si_pairs(off, el, pa[:k], pb[:k], threads)
        dt = time.perf_counter() - t0
        if dt * 4 > target_s or k >= len(pa):
            break
        k = min(len(pa), k * 4)
    return {"value": k / dt, "unit": SI_UNIT, "cores": threads, "kind": "port",
            "sample": f"first {k} pairs ({dt:.1f} s), per-pair merge restatement, OpenMP"}


def run_reference_si(args, dist: Dist) -> None:
    if dist.rank != 0:
        return
    import oracle
    off, el, pa, pb, exp = gen_si_workload(with_library=False)
    threads = os.cpu_count() or 1
    k = max(1, len(pa) // args.ref_stride)
    sel = np.arange(0, len(pa), len(pa) // k, dtype=np.int64)[:k]
    spa, spb = pa[sel], pb[sel]
    for _ in range(args.warmup):
        oracle.si_pairs(off, el, spa[: max(1, k // 50)], spb[: max(1, k // 50)], threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        got = oracle.si_pairs(off, el, spa, spb, threads)
        times.append(time.perf_counter() - t0)
    if not np.array_equal(got, exp[sel]):
        raise RuntimeError("oracle counts differ from the generator's expected counts")
    ms = 1e3 * sum(times) / len(times)
    value = k / (ms / 1e3)
    line = {"metric": SI_METRIC, "value": value, "unit": SI_UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded lognormal pair lists)", "impl": "reference",
            "config": dict(SI_WORKLOAD, sample_stride=args.ref_stride, sampled_pairs=k),
            "cpu_baseline": {"value": value, "unit": SI_UNIT, "cores": threads, "kind": "port",
                             "sample": f"every {args.ref_stride}-th pair, {k} pairs per step; "
                                       "restatement of the reference's SerialIntersection "
                                       "(set_intersection/baseline/ip.cu:266-287)"},
            "e2e": {"value": value, "unit": SI_UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def measure_si(args, dist: Dist, ctx, cpu: bool) -> dict:
    """Batched SI on the 1e6-pair workload: device throughput of the persistent kernel,
    the PLAIN per-pair form, end-to-end through rtg_si_count with pinned host buffers."""
    import rtg
    off, el, pa, pb, exp = gen_si_workload()
    sets = ctx.sets(off, el)
    np_ = len(pa)
    tune = None if args.no_tune else sets.tune(pa, pb)  # autotuned schedule (set on the context)
    algo = si_algo_bytes(off, pa, pb)
    for _ in range(args.warmup):
        ctx.flush_l2()
        sets.count(pa, pb, rtg.SI_AUTO)
        sets.count(pa, pb, rtg.SI_PLAIN)
    l0 = ctx.launches
    ms_steps, kms_steps = [], []
    dist.barrier()
    ctx.sync()
    with ClockSampler(dist.local) as clk:
        for _ in range(args.steps):
            ctx.flush_l2()
            got, t = sets.count(pa, pb, rtg.SI_AUTO)
            ms_steps.append(t.count_ms)
            kms_steps.append(t.main_kernel_ms)
            if not np.array_equal(got, exp):
                raise RuntimeError("batched SI counts differ from the expected counts")
        ctx.sync()
    dist.barrier()
    launches = ctx.launches - l0  # kernels only: the L2 flush is a memset
    value, ms = aggregate(dist, np_, sum(ms_steps) / len(ms_steps))
    # the PLAIN form runs with the library's fixed default schedule, not the tuned one
    tuned = ctx.config().as_dict()
    ctx.set_config(**dict(tuned, si_block_warps=0, si_search_ratio=0, si_stage_slots=0,
                          si_stage_bytes=0, si_blocks_per_sm=0))
    plain_ms = []
    for _ in range(args.steps):
        ctx.flush_l2()
        got, t = sets.count(pa, pb, rtg.SI_PLAIN)
        plain_ms.append(t.count_ms)
        if not np.array_equal(got, exp):
            raise RuntimeError("plain SI counts differ from the expected counts")
    ctx.set_config(**tuned)
    plain_value, _ = aggregate(dist, np_, sum(plain_ms) / len(plain_ms))
    hpa = ctx.host_array(np_, np.uint32)
    hpb = ctx.host_array(np_, np.uint32)
    hout = ctx.host_array(np_, np.uint32)
    hpa[:] = pa
    hpb[:] = pb
    sets.count(hpa, hpb, rtg.SI_AUTO, out=hout)
    e2e_ms = []
    for _ in range(max(1, min(args.steps, 5))):
        t0 = time.perf_counter()
        _, te = sets.count(hpa, hpb, rtg.SI_AUTO, out=hout)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        if not np.array_equal(hout, exp):
            raise RuntimeError("end-to-end SI counts differ")
    e2e_value, _ = aggregate(dist, np_, sum(e2e_ms) / len(e2e_ms))
    # materialised intersections of the same pairs: count -> scan -> write, elements to the
    # host; checked against the expected counts
    moff, mel, _ = sets.materialize(pa, pb)  # sizes the output
    mat_dev, mat_wall = [], []
    for _ in range(3):
        ctx.flush_l2()
        t0 = time.perf_counter()
        moff, mel, tm = sets.materialize(pa, pb, capacity=len(mel))
        mat_wall.append((time.perf_counter() - t0) * 1e3)
        mat_dev.append(tm.count_ms)
    if not np.array_equal(np.diff(moff.astype(np.int64)), exp.astype(np.int64)):
        raise RuntimeError("materialised intersections differ from the expected counts")
    materialize = {"pairs_per_s": np_ / (statistics.median(mat_dev) / 1e3),
                   "device_ms": statistics.median(mat_dev), "wall_ms": statistics.median(mat_wall),
                   "elements_out": int(len(mel)), "d2h_bytes": int(tm.d2h_bytes),
                   "api": "rtg_si_materialize (count -> scan -> write, offsets and elements "
                          "copied to the host; device_ms excludes the copy)"}
    kms = sum(kms_steps) / len(kms_steps)
    peaks = measured_peaks()
    achieved = algo / (kms / 1e3) / 1e9
    # the kernel of the batched form the context ran (si_form 0 is the library default, the
    # producer/consumer form) and its committed ncu summary
    pc_form = tuned.get("si_form", 0) in (0, 2)
    kernel = "k_si_pc" if pc_form else "k_si_stream"
    prof = "si_pc_lognormal_1e6" if pc_form else "si_stream_lognormal_1e6"
    res = {
        "value": value, "unit": SI_UNIT, "ms_per_step": ms, "launches": int(launches),
        "config": dict(SI_WORKLOAD, mode="batched (persistent staged kernel)",
                       l2="flushed before every step", elements=int(len(el))),
        "plain": {"value": plain_value, "unit": SI_UNIT,
                  "ms_per_step": sum(plain_ms) / len(plain_ms)},
        "batched_over_plain": value / plain_value,
        "e2e": {"value": e2e_value, "unit": SI_UNIT, "h2d_bytes_per_step": int(te.h2d_bytes),
                "d2h_bytes_per_step": int(te.d2h_bytes), "ms_per_step": sum(e2e_ms) / len(e2e_ms),
                "api": "rtg_si_count (pinned host pair ids and counts, sets resident)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                     "traffic": profile_traffic(prof),
                     "peak_source": peaks["source"], "kernel": kernel, "kernel_ms": kms,
                     "algo_bytes_per_launch": algo,
                     **dram_view(profile_traffic(prof), kms,
                                 peaks["hbm_gbs"], "pairs longer than a slot with |B| > 8 |A| "
                                 "are searched in global memory, not streamed")},
        "clocks": clk.summary(),
        "cpu_baseline": None,
        "schedule": tune,
        "materialize": materialize,
    }
    if cpu and dist.rank == 0 and dist.ws == 1:
        res["cpu_baseline"] = cpu_baseline_si(off, el, pa, pb)
    sets.close()
    return res


def run_gpu_si(args, dist: Dist) -> None:
    import rtg
    ctx = rtg.Context(dist.local if dist.ws > 1 else 0)
    r = measure_si(args, dist, ctx, cpu=not args.no_cpu_baseline)
    if dist.rank == 0:
        line = {"metric": SI_METRIC, "value": r["value"], "unit": SI_UNIT, "n_gpus": dist.ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic (seeded lognormal pair lists, generated on the host)",
                "config": dict(r["config"], parallelism="replicas" if dist.ws > 1 else "single GPU"),
                "e2e": r["e2e"], "plain": r["plain"], "batched_over_plain": r["batched_over_plain"],
                "roofline": r["roofline"], "cpu_baseline": r["cpu_baseline"],
                "clocks": r["clocks"], "gpu_launches": r["launches"],
                "schedule": r["schedule"], "materialize": r["materialize"]}
        print(json.dumps(line), flush=True)
    ctx.close()


SERVE_WORKLOAD = dict(workload="serve_rmat14to20_x64", graphs=64, scales=[14, 20],
                      edge_factor=16, abcd=[0.57, 0.19, 0.19, 0.05], requests=10_000,
                      p_tc=0.2, pairs_per_request=[1000, 100_000], arrivals="Poisson",
                      load_levels=[0.5, 0.8, 0.95], seed=5,
                      pair_query="|N(u) ∩ N(v)| on the symmetric adjacency, u, v uniform")


def serve_setup(seed: int):
    """64 seeded R-MAT graphs (scales uniform over 14..20) and per-graph pools of random
    vertex pairs; requests take windows of a pool."""
    import rtg
    rng = np.random.default_rng(seed)
    scales = rng.integers(14, 21, SERVE_WORKLOAD["graphs"])
    graphs = []
    for i, sc in enumerate(scales):
        s, d = rtg.gen_rmat(int(sc), 16, 0.57, 0.19, 0.19, seed=1000 + i)
        graphs.append((int(sc), s, d))
    return graphs


def serve_requests(rng, ngraphs: int, n_sym: list[int], count: int, pools):
    lo, hi = SERVE_WORKLOAD["pairs_per_request"]
    reqs = []
    for _ in range(count):
        g = int(rng.integers(ngraphs))
        if rng.random() < SERVE_WORKLOAD["p_tc"]:
            reqs.append((g, 0, 0))
        else:
            k = int(rng.integers(lo, hi + 1))
            o = int(rng.integers(0, len(pools[g][0]) - k + 1))
            reqs.append((g, o, k))
    return reqs


def serve_run(srv, gids, pools, reqs, rate: float | None, m_of: list[int]) -> dict:
    """Submit `reqs` (all at once when rate is None, else Poisson arrivals at `rate`
    requests/s) from one thread while another collects completions."""
    done: list[dict] = []
    n = len(reqs)

    def collect():
        while len(done) < n:
            r = srv.wait_any(1000)
            if r is not None:
                done.append(r[1])

    col = threading.Thread(target=collect, daemon=True)
    rng = np.random.default_rng(17)
    gaps = rng.exponential(1.0 / rate, n) if rate else np.zeros(n)
    col.start()
    t0 = time.perf_counter()
    due = t0
    for (g, o, k), gap in zip(reqs, gaps):
        due += gap
        while True:
            now = time.perf_counter()
            if now >= due:
                break
            time.sleep(min(due - now, 0.0005))
        if k == 0:
            srv.submit_tc(gids[g])
        else:
            u, v = pools[g]
            srv.submit_pairs(gids[g], u[o:o + k], v[o:o + k])
    col.join()
    wall = time.perf_counter() - t0
    lat = np.array([x["latency_ms"] for x in done])
    bad = [x for x in done if x["status"] != 0]
    if bad:
        raise RuntimeError(f"{len(bad)} serving requests failed: {bad[:3]}")
    pairs = sum(x["npairs"] for x in done)
    edges = sum(m_of[x["graph"]] for x in done if x["kind"] == 0)
    return {"offered_rate": rate, "wall_s": wall, "requests_per_s": n / wall,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "intersections_per_s": pairs / wall, "tc_edges_per_s": edges / wall,
            "max_requests_per_launch": max(x["batch_requests"] for x in done)}


def measure_serve(args) -> dict:
    """Serving workload: saturation throughput from a burst of all requests, then Poisson
    arrivals at 0.5 / 0.8 / 0.95 of it; an HBM budget below the graphs' full footprint
    (graphs + a quarter of all counting plans, as the library sizes them: one count of every
    graph on a server without a budget) forces plan eviction and admission waits."""
    import rtg
    graphs = serve_setup(SERVE_WORKLOAD["seed"])
    srv = rtg.Server(0)
    gids = [srv.add_graph(s, d) for _, s, d in graphs]
    infos = [srv.graph_info(x) for x in gids]
    rng = np.random.default_rng(SERVE_WORKLOAD["seed"])
    pools = []
    for i in infos:
        pools.append((rng.integers(0, i.n_sym, 250_000, dtype=np.uint32),
                      rng.integers(0, i.n_sym, 250_000, dtype=np.uint32)))
    m_of = [int(i.m) for i in infos]
    serve_run(srv, gids, pools, [(g, 0, 0) for g in range(len(gids))], None, m_of)
    st0 = srv.stats()
    srv.close()
    plans = st0["plan_bytes"]
    budget = st0["resident_bytes"] + st0["buffer_bytes"] + plans // 4
    srv = rtg.Server(0, budget_bytes=budget)
    gids = [srv.add_graph(s, d) for _, s, d in graphs]
    nreq = SERVE_WORKLOAD["requests"]
    # warm-up: every graph's counting plan and both SI slots once
    warm = serve_requests(np.random.default_rng(1), len(gids), None, 200, pools)
    serve_run(srv, gids, pools, warm, None, m_of)
    sat = serve_run(srv, gids, pools, serve_requests(np.random.default_rng(2), len(gids), None,
                                                     nreq, pools), None, m_of)
    levels = []
    for k, f in enumerate(SERVE_WORKLOAD["load_levels"]):
        reqs = serve_requests(np.random.default_rng(10 + k), len(gids), None, nreq, pools)
        r = serve_run(srv, gids, pools, reqs, f * sat["requests_per_s"], m_of)
        r["load"] = f
        levels.append(r)
    st = srv.stats()
    srv.close()
    return {"saturation": sat, "levels": levels, "budget_bytes": budget,
            "resident_bytes": st0["resident_bytes"], "plan_bytes_all": plans,
            "plan_evictions": st["plan_evictions"], "admission_waits": st["admission_waits"],
            "max_requests_per_launch": st["max_requests_per_launch"],
            "max_inflight_launches": st["max_inflight_launches"],
            "tc_coalesced": st["tc_coalesced"], "si_launches": st["si_launches"],
            "tc_launches": st["tc_launches"]}


def run_gpu_serve(args, dist: Dist) -> None:
    r = measure_serve(args)
    if dist.rank == 0:
        mid = next(x for x in r["levels"] if x["load"] == 0.8)
        line = {"metric": "serving p99 latency", "value": mid["p99_ms"], "unit": "ms",
                "n_gpus": dist.ws, "steps": SERVE_WORKLOAD["requests"], "warmup": 200,
                "ms_per_step": 1e3 / mid["requests_per_s"], "higher_is_better": False,
                "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic (seeded R-MAT graphs and uniform vertex pairs)",
                "config": dict(SERVE_WORKLOAD, parallelism="single GPU",
                               value_at="load 0.8 of saturation"),
                "serving": r}
        print(json.dumps(line), flush=True)


def run_reference(args, dist: Dist) -> None:
    if dist.rank != 0:
        return
    import oracle
    s, d = gen_workload(with_library=False)
    off, adj = oracle.degree_csr(s, d)
    m = len(adj)
    off32, adj32 = off.astype(np.int32), adj.astype(np.int32)
    n = len(off) - 1
    threads = os.cpu_count() or 1
    stride = args.ref_stride
    rows = np.arange(0, n, stride).astype(np.int32)
    sampled_edges = int((off32[rows + 1] - off32[rows]).sum())
    for _ in range(args.warmup):
        oracle.tc_bsearch_rows(off32, adj32, rows[: max(1, len(rows) // 50)], threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.tc_bsearch_rows(off32, adj32, rows, threads)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = sampled_edges / (ms / 1e3)
    sample = (f"every {stride}-th source vertex of the oriented CSR ({sampled_edges} of {m} "
              f"oriented edges per step, {ms / 1e3:.2f} s); restatement of the reference's "
              "ListIntersectionKernel (tc/bs_tc/bs_tc.cu:120-148), per edge x binary search, "
              f"OpenMP on {threads} threads; edges/s = sampled edges / step time")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded R-MAT, the oracle's copy of the generator)",
            "impl": "reference",
            "config": tc_config(n, m, len(s), int(np.diff(off).max()) if m else 0),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "reference_gpu": reference_gpu_point(off, adj, m, args)}
    print(json.dumps(line), flush=True)


def reference_gpu_point(off: np.ndarray, adj: np.ndarray, m: int, args) -> dict:
    """The reference's own GPU count on the same oriented CSR, beside the CPU arm: its
    ListIntersectionKernel (tc/bs_tc/bs_tc.cu:120-148, method 0, compiled unmodified by
    oracle/build_ref.sh where the reference's sources are) launched as its CountOnGPU does,
    timed with CUDA events; its count is checked against the oracle's merge counter."""
    from oracle import ref_gpu
    ok, why = ref_gpu.available()
    if not ok:
        return {"unavailable": why}
    import oracle
    total, times = ref_gpu.count(off, adj, runs=max(1, min(args.steps, 5)))
    ms = sum(times) / len(times)
    return {"value": m / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": len(times),
            "triangles": total, "exact": total == oracle.tc_merge(off, adj),
            "kernel": "ListIntersectionKernel (tc/bs_tc/bs_tc.cu:120-148), the reference's "
                      "method 0, 256 threads per block, at most 65,535 blocks, uint32 counter",
            "timing": "CUDA events around each launch, kernel only (CSR resident)"}


def run_gpu(args, dist: Dist) -> None:
    import rtg
    ctx = rtg.Context(dist.local if dist.ws > 1 else 0)
    s, d = gen_workload()
    g = ctx.graph_from_edges(s, d).build(rtg.ORIENT_DEGREE)
    g.release_edges()
    info = g.info()
    m = info.m
    # autotuned schedule of the batched count (set on the context); --no-tune keeps the
    # library default (for profiling runs: fewer launches before the timed one)
    tune = None if args.no_tune else g.tune()
    # warm-up (also builds and captures the CUDA graph of the batched count)
    for _ in range(args.warmup):
        ctx.flush_l2()
        g.tc(rtg.TC_BATCHED)
        g.tc(rtg.TC_PLAIN)
    want = g.tc(rtg.TC_BATCHED)[0]
    # ---- timed region: batched count, L2 flushed between steps
    launches0 = ctx.launches
    ms_steps, kms_steps, core_steps = [], [], []
    dist.barrier()
    ctx.sync()
    with ClockSampler(dist.local) as clk:
        for _ in range(args.steps):
            ctx.flush_l2()
            total, t = g.tc(rtg.TC_BATCHED)
            if total != want:
                raise RuntimeError(f"count changed between steps: {total} != {want}")
            ms_steps.append(t.count_ms)
            kms_steps.append(t.main_kernel_ms)
            core_steps.append(t.core_ms)
        ctx.sync()
    core_ranks = int(t.core_ranks)
    dist.barrier()
    launches = ctx.launches - launches0  # kernels only: the L2 flush is a memset
    algo_bytes = t.algo_bytes
    ms_local = sum(ms_steps) / len(ms_steps)
    value, ms = aggregate(dist, m, ms_local)
    # ---- plain form on the same CSR
    plain_ms = []
    for _ in range(args.steps):
        ctx.flush_l2()
        tp, t2 = g.tc(rtg.TC_PLAIN)
        if tp != want:
            raise RuntimeError("plain count differs from batched count")
        plain_ms.append(t2.count_ms)
    plain_value, _ = aggregate(dist, m, sum(plain_ms) / len(plain_ms))
    # ---- the counting-form kernel without persistence, graph or tuning (one launch per
    # item bucket, items built on every call): separates algorithm from scheduling
    buck_ms, buck_kms = [], []
    for _ in range(args.steps):
        ctx.flush_l2()
        tb, t3 = g.tc(rtg.TC_BUCKETED)
        if tb != want:
            raise RuntimeError("bucketed count differs from batched count")
        buck_ms.append(t3.count_ms)
        buck_kms.append(t3.main_kernel_ms)
    buck_value, _ = aggregate(dist, m, sum(buck_ms) / len(buck_ms))
    # ---- end to end through the C ABI with pinned host buffers
    hs = ctx.host_array(len(s), np.uint32)
    hd = ctx.host_array(len(d), np.uint32)
    hs[:] = s
    hd[:] = d
    ctx.tc_count_host_edges(hs, hd, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)  # warm
    e2e_ms, e2e_stages = [], []
    for _ in range(max(1, min(args.steps, 5))):
        t0 = time.perf_counter()
        tot, te = ctx.tc_count_host_edges(hs, hd, rtg.ORIENT_DEGREE, rtg.TC_BATCHED)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_stages.append((te.h2d_ms, te.build_ms, te.count_ms))
        if tot != want:
            raise RuntimeError("end-to-end count differs")
    e2e_value, _ = aggregate(dist, m, sum(e2e_ms) / len(e2e_ms))
    kms = sum(kms_steps) / len(kms_steps)
    core_ms = sum(core_steps) / len(core_steps)
    peaks = measured_peaks()
    off, adj = g.csr()
    split = tc_split(off, adj, core_ranks)
    elems, kbytes = split["stream_elems"], split["stream_bytes"]
    prof = profile_fields("tc_batched_rmat21")
    achieved = kbytes / (kms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": profile_traffic("tc_batched_rmat21"),
                "peak_source": peaks["source"], "kernel": "k_tc_warp", "kernel_ms": kms,
                "algo_bytes_per_launch": kbytes, "streamed_elements": elems,
                "algo_bytes_basis": "4 B per streamed suffix element + 8 B per streamed in-edge "
                                    "range + 4 B per out-list element marked + 16 B of offsets "
                                    "per vertex (in-edges from sources below the dense core)",
                "work_equiv_bytes": algo_bytes,
                "work_equiv_gbs": algo_bytes / (ms_local / 1e3) / 1e9,
                "work_equiv_basis": "4 x sum over oriented edges of (d+(u) + d+(v)) + 8 m over "
                                    "the whole count's device time: both full out-lists per "
                                    "edge, which the count never streams"}
    core = {"ranks": core_ranks, "ms": core_ms, "edges": split["core_edges"],
            "matrix_bytes": split["matrix_bytes"], "groups_swept": split["core_groups"],
            "l2_gbs": (16 * split["core_groups"] / (core_ms / 1e3) / 1e9) if core_ms else None,
            "kernels": "k_core_rows (matrix rows) + k_tc_core (word-AND count)",
            "rule": "library choice: largest of 32768 .. 1024 top ranks with edge density >= 2.5 %"}
    if "issue_active" in prof:
        roofline["issue_active"] = prof["issue_active"]
    if "warp_instructions" in prof:
        roofline["inst_per_elem"] = 32 * prof["warp_instructions"] / elems
        roofline["inst_per_elem_basis"] = "32 x ncu warp instructions / streamed elements"
    roofline.update(dram_view(roofline["traffic"], kms, peaks["hbm_gbs"],
                              "most of the algorithmic bytes are served from L2; the limiter "
                              "is instruction issue (issue_active), not DRAM (dram_frac)"))
    # per-edge triangle lists of the same graph (count -> scan -> write over the oriented
    # CSR's edges, lists copied to the host): every triangle once
    tl_dev, tl_wall = [], []
    for _ in range(2):
        t0 = time.perf_counter()
        loff, lw, tl = g.tc_list()
        tl_wall.append((time.perf_counter() - t0) * 1e3)
        tl_dev.append(tl.count_ms)
    if int(loff[-1]) != want:
        raise RuntimeError("triangle lists do not hold every triangle once")
    tc_list = {"triangles_per_s": want / (min(tl_dev) / 1e3), "device_ms": min(tl_dev),
               "wall_ms": min(tl_wall), "elements_out": int(loff[-1]),
               "d2h_bytes": int(tl.d2h_bytes),
               "api": "rtg_tc_list (count -> scan -> write per oriented edge, offsets and "
                      "third vertices copied to the host; device_ms excludes the copy)"}
    del loff, lw
    cpu = None
    if dist.rank == 0 and dist.ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_tc(off, adj)
    g.close()
    si = None
    if not args.tc_only:
        r = measure_si(args, dist, ctx, cpu=False)
        si = {"metric": SI_METRIC, "value": r["value"], "unit": SI_UNIT,
              "ms_per_step": r["ms_per_step"], "workload": r["config"]["workload"],
              "plain": r["plain"], "batched_over_plain": r["batched_over_plain"],
              "e2e": {k: r["e2e"][k] for k in ("value", "unit", "h2d_bytes_per_step",
                                               "d2h_bytes_per_step")},
              "roofline": {k: r["roofline"][k] for k in ("achieved", "peak", "unit", "frac",
                                                         "traffic", "kernel", "dram_gbs",
                                                         "dram_frac") if k in r["roofline"]},
              "gpu_launches": r["launches"], "materialize": r["materialize"],
              "schedule": r["schedule"]["best"] if r["schedule"] else "library default"}
    serving = None
    if not args.tc_only and not args.no_serve and dist.rank == 0:
        r = measure_serve(args)
        mid = next(x for x in r["levels"] if x["load"] == 0.8)
        serving = {"metric": "serving p99 latency", "value": mid["p99_ms"], "unit": "ms",
                   "p50_ms": mid["p50_ms"], "at": "load 0.8 of saturation",
                   "workload": SERVE_WORKLOAD["workload"],
                   "saturation_requests_per_s": r["saturation"]["requests_per_s"],
                   "intersections_per_s": mid["intersections_per_s"],
                   "tc_edges_per_s": mid["tc_edges_per_s"],
                   "levels": [{k: x[k] for k in ("load", "requests_per_s", "p50_ms", "p99_ms")}
                              for x in r["levels"]],
                   "max_requests_per_launch": r["max_requests_per_launch"],
                   "max_inflight_launches": r["max_inflight_launches"]}
    if dist.rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic (seeded R-MAT, generated on the host)",
                "config": tc_config(info.n, m, info.m_input, info.max_out_degree),
                "triangles": want,
                "run": {"mode": "batched", "l2": "flushed before every step",
                        "timing": "CUDA events around each count on the context stream",
                        "parallelism": "replicas" if dist.ws > 1 else "single GPU"},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(te.h2d_bytes),
                        "d2h_bytes_per_step": int(te.d2h_bytes),
                        "ms_per_step": sum(e2e_ms) / len(e2e_ms),
                        "stages_ms": {k: statistics.median(x[i] for x in e2e_stages)
                                      for i, k in enumerate(("h2d", "build", "count"))},
                        "stages_basis": "device time per stage (CUDA events): edge pull over "
                                        "the host link, counting-form build, batched count",
                        "api": "rtg_tc_count_host_edges (pinned host edges, CSR build included)"},
                "plain": {"value": plain_value, "unit": UNIT,
                          "ms_per_step": sum(plain_ms) / len(plain_ms)},
                "batched_over_plain": value / plain_value,
                "bucketed": {"value": buck_value, "unit": UNIT,
                             "ms_per_step": sum(buck_ms) / len(buck_ms),
                             "kernel_ms": sum(buck_kms) / len(buck_kms),
                             "form": "the batched kernel's algorithm (counting form, suffix "
                                     "streaming) launched once per item bucket, no persistence, "
                                     "no CUDA graph, default schedule, items built every call"},
                "bucketed_over_plain": buck_value / plain_value,
                "batched_over_bucketed": value / buck_value,
                "roofline": roofline, "core": core, "tc_list": tc_list, "cpu_baseline": cpu,
                "clocks": clk.summary(),
                "gpu_launches": int(launches), "schedule": tune, "si": si,
                "serving": serving}
        print(json.dumps(line), flush=True)
    ctx.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="rtg", choices=["rtg", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-stride", type=int, default=32)
    ap.add_argument("--workload", default="tc", choices=["tc", "si", "serve"],
                    help="tc: R-MAT-21 triangle count (with a batched-SI summary); "
                         "si: the 1e6-pair batched set intersection alone")
    ap.add_argument("--tc-only", action="store_true",
                    help="skip the batched-SI and serving summaries")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving summary")
    ap.add_argument("--no-tune", action="store_true",
                    help="time the library's default schedules instead of autotuning first")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("at least 3 warm-up steps")
    dist = Dist("gloo" if args.impl == "reference" else None)
    try:
        if args.impl == "reference":
            if args.workload == "serve":
                if dist.rank == 0:
                    print(json.dumps({"impl": "reference", "unavailable":
                                      "the reference has no serving loop: its mains count one "
                                      "graph or one dataset per process"}), flush=True)
            else:
                (run_reference_si if args.workload == "si" else run_reference)(args, dist)
        else:
            {"tc": run_gpu, "si": run_gpu_si, "serve": run_gpu_serve}[args.workload](args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
