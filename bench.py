"""Benchmark of the Fast-APSP hot path on GB300.

Workload (default): a directed 3-nearest-neighbour geometric graph of 65,536
uniform points in the unit square with integer weights U[1,1000] (seeded),
split into K=64 parts by the engine's partitioner, all parts solved (the rows
of solveSubGraph(1..64)), int32 distances + predecessors.  Inputs are synthetic;
there is no public dataset in this workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:      one JSON line: device-resident throughput (value), the end-to-end
           number through the public C ABI with host buffers (e2e), the
           min-plus kernel's add-min roofline, the SSSP kernel's HBM roofline,
           the plain-form comparison, clocks and the CPU baseline.
reference: the reference's CPU algorithm (the oracle restatement of its
           fapGraph::run CPU branch, pinned bit-for-bit to the reference's own
           fap.cpp) on a bounded sample of the same workload, on all host cores.
Under torchrun (N>1) every rank solves its own instance (seed + rank), no
collective on the data path; rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

MP_TRAFFIC_PER_OUTPUT_BYTE = 1.136  # DRAM read+write per algorithmic byte of the min-plus launch (ncu)
METRIC = "APSP distances/s"
UNIT = "distances/s"
HBM_PEAK_FALLBACK = 6800.0


N_DEFAULT, K_DEFAULT = 65536, 64


def workload(seed_offset=0, n=N_DEFAULT, K=K_DEFAULT):
    from fastapsp_gb300 import graphs

    return graphs.geometric_knn(n, 3, 1, 1000, seed=20261205 + seed_offset), K


def read_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text()), "measured"
        except Exception:
            pass
    return {"hbm_gbs": HBM_PEAK_FALLBACK}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.file:
            return None
        self.file.flush()
        rows = []
        try:
            for line in Path(self.file.name).read_text().splitlines():
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            try:
                os.unlink(self.file.name)
            except OSError:
                pass
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def part_stats(eng, K, n):
    subs, bdys = [], []
    for p in range(1, K + 1):
        s, b, _ = eng.part_info(p)
        subs.append(s)
        bdys.append(b)
    subs = np.array(subs, np.int64)
    bdys = np.array(bdys, np.int64)
    addmin_mp = int(((subs - bdys) * bdys).sum() * n)
    ld = ((subs + 63) // 64) * 64
    addmin_fw = int((ld.astype(np.float64) ** 3).sum())
    rounds = int(ld.max() // 64)
    return subs, bdys, addmin_mp, addmin_fw, rounds


def run_ours(args, rank, world, local_rank):
    import torch

    import fastapsp_gb300 as fap

    torch.cuda.set_device(local_rank)
    dev = local_rank
    g, K = workload(seed_offset=rank, n=args.n, K=args.K)
    gid, cut = fap.partition(g.row_offset, g.col_val, K)
    n = g.n
    eng = fap.Engine(n, g.row_offset, g.col_val, g.weight, K, graph_id=gid, dtype=fap.DTYPE_I32, device=dev)
    subs, bdys, addmin_mp, addmin_fw, rounds = part_stats(eng, K, n)
    dist = torch.empty((n, n), dtype=torch.int32, device="cuda")
    pred = torch.empty((n, n), dtype=torch.int32, device="cuda")
    flush = torch.empty(64 << 20, dtype=torch.int32, device="cuda")  # 256 MiB > L2
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step():
        eng.solve(dist, pred, fap.MODE_BATCHED, stream=sptr)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # the first solve tuned the SSSP near-far step; later engines on the same
    # graph (the e2e loop) reuse it instead of tuning again
    tuned_delta = eng.get_option(fap._lib.OPT_SSSP_DELTA)
    tuned_lanes = eng.get_option(fap._lib.OPT_SSSP_LANES)
    step_ms, phase = [], []
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            flush.fill_(1)  # untimed L2 flush between timed steps
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            step()
            b.record(stream)
            b.synchronize()
            step_ms.append(a.elapsed_time(b))
            phase.append(eng.last_times())
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = clk.summary()
    total_ms = float(sum(step_ms))
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * float(n) * n / (ms_per_step / 1e3)

    # phase times (device events inside the captured graph)
    ph = {k: statistics.mean(p[k] for p in phase) for k in phase[0]}
    sssp_stats = eng.sssp_stats()
    launches_per_step = eng.last_launches()  # kernels of one solve (counted by the engine)
    # roofline of the dominant kernel (min-plus) against the add-min issue peak
    peak_dpx = eng_ctx_peak(fap, dev, 0)
    peak_arg = eng_ctx_peak(fap, dev, 2)
    def rate(x, ms):
        return x / (ms / 1e3) if ms and ms > 0 else float("nan")

    mp_rate = rate(addmin_mp, ph["min_plus"])
    fw_rate = rate(addmin_fw, ph["floyd"])
    peaks, peak_src = read_peaks()
    hbm = float(peaks.get("hbm_gbs", HBM_PEAK_FALLBACK))
    srcs = int(bdys.sum())
    sssp_bytes = srcs * (4 * (n + 1) + 8 * g.m + 8 * n)
    sssp_gbs = rate(sssp_bytes, ph["sssp"]) / 1e9
    mp_bytes = int(((subs - bdys) * n * 8).sum() + (bdys * n * 8).sum())  # C written + B read once
    mp_gbs = rate(mp_bytes, ph["min_plus"]) / 1e9
    # add-min steps the strip kernel actually ran (it skips the k-steps whose B
    # row or A column is unreached over a tile): one more solve with counters
    eng.minplus_counters(reset=True)
    eng.solve(dist, pred, fap.MODE_BATCHED, stream=sptr)
    torch.cuda.synchronize()
    mpc = eng.minplus_counters(reset=True)
    executed = mpc["active_steps"] * 128 * 128  # upper bound: full 128x128 tiles

    # plain form (per-part launches) on the same graph, for batched-vs-plain
    plain_ms = []
    for _ in range(2 if args.plain else 0):
        eng.solve(dist, pred, fap.MODE_PLAIN, stream=sptr)
    for _ in range(2 if args.plain else 0):
        flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.solve(dist, pred, fap.MODE_PLAIN, stream=sptr)
        b.record(stream)
        b.synchronize()
        plain_ms.append(a.elapsed_time(b))
    plain_ms = statistics.mean(plain_ms) if plain_ms else float("nan")
    eng.close()
    del dist, pred
    torch.cuda.empty_cache()

    # end to end through the public C ABI with host buffers: per step the CSR
    # goes host->device (fap_create from pinned arrays) and the full result
    # rows come back device->host into pinned buffers.
    ro_h = torch.from_numpy(g.row_offset).pin_memory()
    col_h = torch.from_numpy(g.col_val).pin_memory()
    w_h = torch.from_numpy(g.weight).pin_memory()
    gid_h = torch.from_numpy(gid).pin_memory()
    shape = (n, n) if args.e2e_steps > 0 else (1, 1)
    dist_h = torch.empty(shape, dtype=torch.int32, pin_memory=True)
    pred_h = torch.empty(shape, dtype=torch.int32, pin_memory=True)
    e2e_ms = []
    for i in range((1 + args.e2e_steps) if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e = fap.Engine(n, ro_h.numpy(), col_h.numpy(), w_h.numpy(), K, graph_id=gid_h.numpy(),
                       dtype=fap.DTYPE_I32, device=dev)
        e.set_option(fap._lib.OPT_SSSP_DELTA, tuned_delta)
        e.set_option(fap._lib.OPT_SSSP_LANES, tuned_lanes)
        e.solve(dist_h, pred_h, fap.MODE_BATCHED)
        e.close()
        t1 = time.perf_counter()
        if i > 0:
            e2e_ms.append((t1 - t0) * 1e3)
    e2e_ms_step = statistics.mean(e2e_ms) if e2e_ms else float("nan")
    h2d = int(g.row_offset.nbytes + g.col_val.nbytes + g.weight.nbytes + gid.nbytes)
    d2h = int(n) * n * 8

    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {
            "workload": f"directed 3-NN geometric graph, n={n}, int weights U[1,1000], K={K} parts, "
                        f"all parts solved (solveSubGraph 1..{K} rows), int32 dist + pred",
            "n": n, "m": int(g.m), "K": K, "edge_cut": cut, "boundary_vertices": srcs,
            "mode": "batched (one launch per phase, CUDA graph)",
            "sssp_delta": tuned_delta,
            "sssp_lanes": int(tuned_lanes),
            "l2": f"L2 flushed (256 MiB write) before every timed step; outputs {n * n * 8 / 1e9:.1f} GB",
            "parallelism": f"replicas x{world}",
        },
        "e2e": {"value": world * float(n) * n / (e2e_ms_step / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms_step,
                "what": "fap_create (CSR from pinned host) + fap_solve into pinned host rows + fap_destroy"
                    " (SSSP step set to the value tuned on this graph)"},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {
            # The min-plus skips the k-steps that cannot change a tile (unreached B row
            # or A column), so on this graph its add-min count is data-dependent and
            # small; what it must always do is write the n x n rows: HBM-bound.
            "kernel": "mp_strip_kernel (min-plus of the inner rows and decode of their own-part columns)",
            "bound": "hbm",
            "achieved": mp_gbs, "peak": hbm, "unit": "GB/s", "frac": mp_gbs / hbm,
            "peak_source": peak_src,
            "algorithmic_bytes_per_launch": mp_bytes,
            # DRAM bytes per launch: an ncu capture of the same launch at n=24,576 read + wrote
            # this many bytes per output byte; output and work grow with n^2, so the full
            # launch is scaled by its output bytes.
            "traffic": MP_TRAFFIC_PER_OUTPUT_BYTE * mp_bytes,
            "traffic_source": f"ncu capture at n=24,576 ({MP_TRAFFIC_PER_OUTPUT_BYTE} DRAM bytes per "
                              "algorithmic byte), scaled",
            "alu_view": {
                "executed_addmins_per_launch": executed,
                "achieved": rate(executed, ph["min_plus"]) / 1e9, "peak": peak_dpx / 1e9,
                "unit": "Gaddmin/s", "frac": rate(executed, ph["min_plus"]) / peak_dpx,
                "dense_addmins_per_launch": addmin_mp,
                "dense_equivalent_rate": mp_rate / 1e9,
                "strip_tiles": mpc["tiles"], "tiles_without_active_step": mpc["empty_tiles"],
                "peak_source": "fap_addmin_peak mode 0 (int32 DPX add-min from registers), measured in this run",
                "peak_with_argmin": peak_arg / 1e9,
            },
        },
        "roofline_fw": {"achieved": fw_rate / 1e9, "peak": peak_dpx / 1e9, "unit": "Gaddmin/s",
                        "frac": fw_rate / peak_dpx, "algorithmic_addmins": addmin_fw,
                        "note": "dense count (sum of ld^3); the remaining-tile kernel skips unreached "
                                "steps, so this is a dense-equivalent rate"},
        "roofline_sssp": {"bound": "hbm", "achieved": sssp_gbs, "peak": hbm, "unit": "GB/s",
                          "frac": sssp_gbs / hbm, "algorithmic_bytes": sssp_bytes, "peak_source": peak_src},
        "phase_ms": ph,
        "sssp_stats": sssp_stats,
        "plain_form": {"ms_per_step": plain_ms, "batched_speedup": plain_ms / ms_per_step},
        "clocks": clocks,
    }
    return res


_PEAK_CACHE = {}


def eng_ctx_peak(fap, dev, mode):
    if mode not in _PEAK_CACHE:
        ctx = fap.Context(dev)
        _PEAK_CACHE[mode] = ctx.addmin_peak(mode)
        ctx.close()
    return _PEAK_CACHE[mode]


def cpu_sample(part, g, K, gid, pre, rows):
    """The reference's CPU algorithm on one part with the min-plus limited to
    `rows` inner rows; returns (extrapolated part seconds, measured seconds)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    n = g.n
    sub = int(pre["ver_num"][part])
    bdy = int(pre["bdy_num"][part])
    inner = sub - bdy
    r = min(rows, inner)
    t0 = time.perf_counter()
    _, _, t = oracle.run_part(part, g.row_offset, g.col_val, g.weight, gid, pre, mp_rows=r)
    measured = time.perf_counter() - t0
    scale = inner / max(r, 1)
    est = t["sssp"] + t["floyd"] + t["data"] + t["min_plus"] * scale
    return est, measured, sub


def run_reference(args):
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    import fastapsp_gb300 as fap

    oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    g, K = workload()
    gid, _ = fap.partition(g.row_offset, g.col_val, K)
    pre = oracle.preprocess(K, gid, g.row_offset, g.col_val)
    rates, meas = [], []
    for i in range(args.warmup + args.steps):
        part = 1 + (i % K)
        est, m, sub = cpu_sample(part, g, K, gid, pre, args.ref_rows)
        if i >= args.warmup:
            rates.append(sub * g.n / est)
            meas.append(m)
    value = statistics.mean(rates)
    sample = (f"per step one part of the 64: SSSP from all its boundary vertices (OpenMP), its full "
              f"Floyd-Warshall, and the min-plus on the first {args.ref_rows} inner rows; the part's "
              f"time is extrapolated per add-min to all its inner rows; distances/s = part rows x n "
              f"/ part time")
    res = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(meas) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (reference arithmetic; integer weights exact)",
        "data": "synthetic",
        "config": {"workload": f"directed 3-NN geometric graph, n={g.n}, int weights U[1,1000], K={K} parts",
                   "n": g.n, "m": int(g.m), "K": K},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return res


def _device_solve_rate(fap, torch, g, K, dtype, steps, warmup, mode=None, options=None):
    """Device-resident solve of a whole graph: (ms per solve, engine, dist, pred)."""
    mode = fap.MODE_BATCHED if mode is None else mode
    gid, cut = fap.partition(g.row_offset, g.col_val, K)
    eng = fap.Engine(g.n, g.row_offset, g.col_val, g.weight, K, graph_id=gid, dtype=dtype)
    for opt, val in (options or {}).items():
        eng.set_option(opt, val)
    tdt = torch.int32 if dtype == fap.DTYPE_I32 else torch.float32
    dist = torch.empty((g.n, g.n), dtype=tdt, device="cuda")
    pred = torch.empty((g.n, g.n), dtype=torch.int32, device="cuda")
    flush = torch.empty(64 << 20, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        eng.solve(dist, pred, mode, stream=stream.cuda_stream)
    times = []
    for _ in range(steps):
        flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.solve(dist, pred, mode, stream=stream.cuda_stream)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return statistics.mean(times), eng, dist, pred, gid, cut


def run_c1(args):
    """128x128 grid (spanning tree + p=0.6 edges), unweighted, K=16, int32,
    full solve(); distances checked bit for bit against the oracle's
    Dijkstra (the reference's dijkstra_path) on sampled rows."""
    import torch

    import fastapsp_gb300 as fap
    from fastapsp_gb300 import graphs

    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    g = graphs.grid_graph()
    ms, eng, dist, pred, gid, cut = _device_solve_rate(fap, torch, g, 16, fap.DTYPE_I32, args.steps, args.warmup)
    plain_ms, *_ = _device_solve_rate(fap, torch, g, 16, fap.DTYPE_I32, 2, 1, mode=fap.MODE_PLAIN)
    mapping = eng.mapping()
    rows = np.random.default_rng(0).choice(g.n, size=64, replace=False)
    d = dist[torch.from_numpy(rows).cuda()].cpu().numpy()
    exact = True
    for i, r in enumerate(rows):
        rd, _ = oracle.dijkstra_path(int(mapping[r]), g.row_offset, g.col_val, g.weight)
        ref = np.where(rd >= 1e8, 1 << 30, rd).astype(np.int64)
        exact = exact and np.array_equal(d[i].astype(np.int64), ref)
    return {"config": "c1", "metric": METRIC, "value": g.n * g.n / (ms / 1e3), "unit": UNIT,
            "ms_per_step": ms, "dtype": "int32", "n": g.n, "m": g.m, "K": 16, "edge_cut": cut,
            "plain_ms": plain_ms, "batched_speedup": plain_ms / ms,
            "parity": f"64 sampled rows bit-exact vs the reference's Dijkstra: {exact}",
            "phase_ms": eng.last_times(), "sssp_stats": eng.sssp_stats(),
            "sssp_delta": eng.get_option(fap._lib.OPT_SSSP_DELTA),
            "sssp_lanes": int(eng.get_option(fap._lib.OPT_SSSP_LANES))}


def run_c3(args):
    """512 dense int32 instances, sizes log-uniform in [32, 2048], 5% edges,
    weights U[1,100]: all instances in one launch per FW phase (batched) vs
    one launch sequence per instance."""
    import torch

    import fastapsp_gb300 as fap
    from fastapsp_gb300 import graphs

    mats = graphs.dense_instances()
    ctx = fap.Context(0)
    work = float(sum(float(m.shape[0]) ** 3 for m in mats))
    host = [torch.from_numpy(m) for m in mats]
    dev = [h.cuda() for h in host]
    preds = [torch.where(h < (1 << 30), torch.arange(h.shape[0], dtype=torch.int32)[:, None],
                         torch.full((1, 1), -1, dtype=torch.int32)).contiguous().cuda() for h in host]
    pinit = [p.clone() for p in preds]
    stream = torch.cuda.current_stream()

    def reset():
        for d_, h in zip(dev, host):
            d_.copy_(h, non_blocking=True)
        for p_, p0 in zip(preds, pinit):
            p_.copy_(p0)

    def timed(fn, steps):
        out = []
        for _ in range(steps):
            reset()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            out.append(a.elapsed_time(b))
        return statistics.mean(out)

    batched = lambda: ctx.floyd_batched(1, dev, preds, stream=stream.cuda_stream)  # noqa: E731

    def per_instance():
        for d_, p_ in zip(dev, preds):
            ctx.floyd_batched(1, [d_], [p_], stream=stream.cuda_stream)

    for _ in range(args.warmup):
        reset()
        batched()
    ms_b = timed(batched, args.steps)
    per_instance()
    ms_p = timed(per_instance, max(1, args.steps // 2))
    peak = ctx.addmin_peak(0)
    ctx.close()
    return {"config": "c3", "metric": "add-min Gop/s (batched Floyd-Warshall, 512 instances)",
            "value": work / (ms_b / 1e3) / 1e9, "unit": "Gaddmin/s", "ms_per_step": ms_b,
            "per_instance_ms": ms_p, "batched_speedup": ms_p / ms_b, "dtype": "int32",
            "instances": len(mats), "addmins": work, "frac_of_dpx_peak": work / (ms_b / 1e3) / peak}


def run_c4(args):
    """Road-like FP32 graph, 114,599 vertices, K=128, full batched APSP;
    error against FP64 Dijkstra on 4,096 sampled sources."""
    import torch

    import fastapsp_gb300 as fap
    from fastapsp_gb300 import graphs

    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    g = graphs.road_like()
    fp64 = 0 if args.c4_faithful else 1
    ms, eng, dist, pred, gid, cut = _device_solve_rate(
        fap, torch, g, 128, fap.DTYPE_F32, args.steps, args.warmup,
        options={fap._lib.OPT_SSSP_FP64: fp64})
    phase = eng.last_times()
    stats = eng.sssp_stats()
    delta = eng.get_option(fap._lib.OPT_SSSP_DELTA)
    mapping = eng.mapping()
    inv = np.empty_like(mapping)
    inv[mapping] = np.arange(g.n)
    srcs = np.random.default_rng(4).choice(g.n, size=args.c4_sources, replace=False)
    rows = torch.from_numpy(inv[srcs].astype(np.int64)).cuda()
    d = dist[rows].cpu().numpy()
    eng.close()
    del dist, pred
    torch.cuda.empty_cache()
    from concurrent.futures import ThreadPoolExecutor

    def err(i):
        d64 = oracle.dijkstra_f64(int(srcs[i]), g.row_offset, g.col_val, g.weight)
        f = d64 < 1e299
        if not np.array_equal(f, d[i] < 1e8):
            return float("inf")
        return float(np.max(np.abs(d[i][f] - d64[f]) / np.maximum(d64[f], 1e-30)))

    with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        errs = list(ex.map(err, range(len(srcs))))
    return {"config": "c4", "metric": METRIC, "value": g.n * g.n / (ms / 1e3), "unit": UNIT,
            "ms_per_step": ms, "dtype": "f32", "n": g.n, "m": g.m, "K": 128, "edge_cut": cut,
            "sssp": "FP64 search, rounded once" if fp64 else "FP32 (reference arithmetic)",
            "sampled_sources": len(srcs), "max_rel_err_vs_fp64": max(errs),
            "mean_of_row_max_rel_err": float(np.mean(errs)), "phase_ms": phase,
            "sssp_stats": stats, "sssp_delta": delta}


def run_c5(args):
    """256 random 4-regular digraphs (n U[256,1024], FP32 w U(0.5,2)): batched
    FW with predecessors (forward), loss = sum of D[s,t] over 10,000 pairs,
    adjoint onto the weights (backward); backward/forward time ratio."""
    import torch

    import fastapsp_gb300 as fap
    from fastapsp_gb300 import graphs

    gs = graphs.regular_digraphs()
    rng = np.random.default_rng(5)
    npairs = 10000
    b = rng.integers(0, len(gs), size=npairs)
    s = np.array([rng.integers(0, gs[i].n) for i in b])
    t = np.array([rng.integers(0, gs[i].n) for i in b])
    ctx = fap.Context(0)
    host = []
    for g in gs:
        W = np.full((g.n, g.n), 1e8, np.float32)
        src = np.repeat(np.arange(g.n), np.diff(g.row_offset))
        W[src, g.col_val] = g.weight
        np.fill_diagonal(W, 0)
        P = np.where(W < 1e8, np.arange(g.n)[:, None], -1).astype(np.int32)
        host.append((torch.from_numpy(W), torch.from_numpy(P)))
    D = [h[0].cuda() for h in host]
    P = [h[1].cuda() for h in host]
    dW = [torch.zeros_like(d_) for d_ in D]
    bt, st_, tt = (torch.from_numpy(x.astype(np.int32)).cuda() for x in (b, s, t))
    gg = torch.ones(npairs, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    fw, bw = [], []
    for i in range(args.warmup + args.steps):
        for d_, p_, h in zip(D, P, host):
            d_.copy_(h[0])
            p_.copy_(h[1])
        for w_ in dW:
            w_.zero_()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        ctx.floyd_batched(0, D, P, stream=stream.cuda_stream)
        e1.record(stream)
        ctx.backward_dense(P, dW, bt, st_, tt, gg, stream=stream.cuda_stream)
        e2.record(stream)
        e2.synchronize()
        if i >= args.warmup:
            fw.append(e0.elapsed_time(e1))
            bw.append(e1.elapsed_time(e2))
    ctx.close()
    work = float(sum(float(g.n) ** 3 for g in gs))
    return {"config": "c5", "metric": "backward / forward time", "value": statistics.mean(bw) / statistics.mean(fw),
            "unit": "ratio", "forward_ms": statistics.mean(fw), "backward_ms": statistics.mean(bw),
            "forward_gaddmin_s": work / (statistics.mean(fw) / 1e3) / 1e9, "graphs": len(gs),
            "pairs": npairs, "dtype": "f32"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--ref-rows", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="host work of the cpu_baseline sample (whole parts until this is reached)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n", type=int, default=N_DEFAULT, help="vertices (profiling cases only)")
    ap.add_argument("--K", type=int, default=K_DEFAULT, help="parts (profiling cases only)")
    ap.add_argument("--no-plain", dest="plain", action="store_false")
    ap.add_argument("--config", choices=["c1", "c2", "c3", "c4", "c5"], default="c2",
                    help="c2 (default) is the headline workload; the others print their own line")
    ap.add_argument("--c4-sources", type=int, default=4096)
    ap.add_argument("--c4-faithful", action="store_true",
                    help="c4 with FP32 SSSP arithmetic (the reference's) instead of FP64")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if args.config != "c2":
        import torch

        torch.cuda.set_device(local_rank)
        fn = {"c1": run_c1, "c3": run_c3, "c4": run_c4, "c5": run_c5}[args.config]
        print(json.dumps(fn(args)))
        return

    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res = run_ours(args, rank, world, local_rank)
    if rank == 0:
        if not args.no_cpu_baseline:
            sys.path.insert(0, str(ROOT / "oracle"))
            import oracle

            import fastapsp_gb300 as fap

            oracle.build()
            cores = os.cpu_count() or 1
            oracle.set_threads(cores)
            g, K = workload()
            gid, _ = fap.partition(g.row_offset, g.col_val, K)
            pre = oracle.preprocess(K, gid, g.row_offset, g.col_val)
            # parts in order until about --cpu-seconds of host work
            rows = est = meas = 0.0
            parts = 0
            for part in range(1, K + 1):
                e_p, m_p, sub = cpu_sample(part, g, K, gid, pre, args.ref_rows)
                rows, est, meas, parts = rows + sub, est + e_p, meas + m_p, parts + 1
                if meas >= args.cpu_seconds:
                    break
            res["cpu_baseline"] = {
                "value": rows * g.n / est, "unit": UNIT, "cores": cores, "kind": "port",
                "sample": f"parts 1..{parts} of {K}: SSSP (all boundary sources, OpenMP), full FW, "
                          f"min-plus on {args.ref_rows} inner rows per part extrapolated per add-min; "
                          f"{meas:.1f} s measured",
            }
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
