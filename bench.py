"""Benchmark of the Fast-APSP hot path on GB300.

Workload (default, --config c4): the road-like graph of 114,599 vertices
(perturbed planar grid thinned to a near-tree and subdivided by degree-2
chains, ~239k directed entries, FP32 weights U[0.1,10], seeded), split into
K=128 parts, full all-pairs solve with FP32 distances and int32 predecessors,
the boundary SSSP in exact arithmetic (the FP64 option), so results are within
1e-6 of FP64 Dijkstra.  Inputs are synthetic; no dataset is involved.  The
parts come from a committed partition (tests/golden/partitions/partition_*.npz) that both
arms use.  --config c1 / c2 print the same line for the 128x128 grid and the
65,536-vertex geometric graph; c3 / c5 print their own lines.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config c4]

ours:      one JSON line: device-resident throughput (value), the end-to-end
           number through the public C ABI with host buffers (e2e), the
           min-plus kernel's roofline, the FW and SSSP rates, the plain-form
           comparison, clocks and the CPU baseline.
reference: the reference's CPU algorithm (the oracle restatement of its
           fapGraph::run CPU branch, pinned bit-for-bit to the reference's own
           fap.cpp) on a bounded sample of the same workload, on all host
           cores, without loading the engine's library.
Under torchrun (N>1) every rank solves its own copy of the graph, no
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

METRIC = "APSP distances/s"
UNIT = "distances/s"
HBM_PEAK_FALLBACK = 6800.0
# DRAM read+write bytes per algorithmic byte of the min-plus launch, from ncu
# captures of the same kernel on smaller cases of each workload (scaled by the
# output bytes, which grow with the work); None where no capture was taken.
MP_TRAFFIC_PER_BYTE = {"c2": 1.136, "c4": 1.181, "c1": None}

# Solve workloads: the synthetic graph, its part count, the engine's distance
# type, the committed partition (tests/golden/partitions/make_partitions.py) and, for
# FP32 graphs, the SSSP arithmetic the spec bar needs.
WORKLOADS = {
    "c4": dict(gen="road_like", K=128, dtype="f32", part="road_like_n114599_K128", fp64_sssp=1,
               desc="road-like graph (perturbed planar grid thinned to a near-tree, degree-2 chain "
                    "subdivision), n=114,599, ~239k directed entries, FP32 weights U[0.1,10], K=128 parts, "
                    "full APSP (solve), FP32 dist + int32 pred"),
    "c2": dict(gen="geometric_knn", K=64, dtype="i32", part="geometric_knn_n65536_K64", fp64_sssp=0,
               desc="directed 3-NN geometric graph, n=65,536, int weights U[1,1000], K=64 parts, all parts "
                    "solved (solveSubGraph 1..64 rows), int32 dist + pred"),
    "c1": dict(gen="grid_graph", K=16, dtype="i32", part="grid_n16384_K16", fp64_sssp=0,
               desc="128x128 grid (random spanning tree + each other edge with p=0.6), unweighted, "
                    "K=16 parts, full APSP (solve), int32 hop counts + pred"),
}


def load_graphs_module():
    """The seeded workload generators (pure numpy), loaded from their file
    without importing the engine package, so the reference arm maps no part
    of the engine."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("fap_workload_graphs", ROOT / "fastapsp_gb300" / "graphs.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod  # dataclasses look their module up
    spec.loader.exec_module(mod)
    return mod


def load_workload(name):
    """(graph, K, graph_id, edge cut) of a solve workload; the partition is
    the committed one, checked against the generated graph."""
    import zlib

    wl = WORKLOADS[name]
    g = getattr(load_graphs_module(), wl["gen"])()
    z = np.load(ROOT / "tests" / "golden" / "partitions" / f"partition_{wl['part']}.npz")
    crc = zlib.crc32(np.ascontiguousarray(g.row_offset, np.int32).tobytes())
    crc = zlib.crc32(np.ascontiguousarray(g.col_val, np.int32).tobytes(), crc)
    crc = zlib.crc32(np.ascontiguousarray(g.weight, np.float32).tobytes(), crc)
    if int(z["n"]) != g.n or int(z["m"]) != g.m or int(z["csr_crc"]) != crc:
        raise RuntimeError(f"partition_{wl['part']}.npz does not belong to the generated graph")
    return g, wl["K"], z["graph_id"].astype(np.int32), int(z["edge_cut"])


def boundary_count(g, gid):
    """Vertices with an edge to another part (findBoundry, util_preprocess.h:32-58)."""
    src = np.repeat(np.arange(g.n), np.diff(g.row_offset))
    cut = gid[src] != gid[g.col_val]
    b = np.zeros(g.n, bool)
    b[src[cut]] = True
    b[g.col_val[cut]] = True
    return int(b.sum())


def workload_config(name, g, K, gid, cut):
    """The `config` of both arms' lines: a static description of the work."""
    wl = WORKLOADS[name]
    return {"workload": wl["desc"], "n": g.n, "m": int(g.m), "K": K, "edge_cut": cut,
            "boundary_vertices": boundary_count(g, gid),
            "partition": f"tests/golden/partitions/partition_{wl['part']}.npz (the engine's multilevel partitioner, "
                         "committed; both arms solve the same parts)",
            "l2": "L2 flushed (256 MiB write) before every timed step; outputs "
                  f"{g.n * g.n * 8 / 1e9:.1f} GB"}


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
    return subs, bdys, addmin_mp, addmin_fw


def pinned_host(shape, dtype):
    """Page-locked host rows of exactly `shape` from cudaHostAlloc (the CUDA
    runtime torch loaded; the caching pinned allocator would round each
    buffer up to a power of two, and registered pageable memory measured
    slower for kernel stores); returns (numpy array, free function, source)."""
    import ctypes

    import torch

    nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
    try:
        rt = ctypes.CDLL("libcudart.so.13")
        p = ctypes.c_void_p()
        if rt.cudaHostAlloc(ctypes.byref(p), ctypes.c_size_t(nbytes), 0) == 0 and p.value:
            buf = (ctypes.c_char * nbytes).from_address(p.value)
            arr = np.frombuffer(buf, dtype=dtype).reshape(shape)
            return arr, lambda: rt.cudaFreeHost(p), "cudaHostAlloc"
    except OSError:
        pass
    t = torch.empty(shape, dtype=torch.from_numpy(np.empty(0, dtype)).dtype, pin_memory=True)
    return t.numpy(), lambda: None, "torch pinned allocator"


def run_solve(args, name, rank, world, local_rank):
    """Device-resident solve of a whole workload graph (value), the same
    through the C ABI with host buffers (e2e), rooflines, the plain form."""
    import torch

    import fastapsp_gb300 as fap

    torch.cuda.set_device(local_rank)
    dev = local_rank
    wl = WORKLOADS[name]
    g, K, gid, cut = load_workload(name)
    n = g.n
    dtype = fap.DTYPE_F32 if wl["dtype"] == "f32" else fap.DTYPE_I32
    tdt = torch.float32 if dtype == fap.DTYPE_F32 else torch.int32
    options = {fap._lib.OPT_SSSP_FP64: wl["fp64_sssp"]} if dtype == fap.DTYPE_F32 else {}
    eng = fap.Engine(n, g.row_offset, g.col_val, g.weight, K, graph_id=gid, dtype=dtype, device=dev)
    for o, v in options.items():
        eng.set_option(o, v)
    subs, bdys, addmin_mp, addmin_fw = part_stats(eng, K, n)
    # Under torchrun the parts of the one graph are split over the ranks by
    # the cost-balanced assignment (no collective touches the rows); with
    # --shard replicas every rank solves the whole graph instead.
    share = None
    if world > 1 and args.shard == "parts":
        from fastapsp_gb300.sharding import assign_parts

        share = assign_parts(np.r_[0, subs], np.r_[0, bdys], n, g.m, world)[rank]
    rows = n if share is None else int(sum(subs[q - 1] for q in share))
    dist = torch.empty((max(rows, 1), n), dtype=tdt, device="cuda")
    pred = torch.empty((max(rows, 1), n), dtype=torch.int32, device="cuda")
    flush = torch.empty(64 << 20, dtype=torch.int32, device="cuda")  # 256 MiB > L2
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step():
        if share is None:
            eng.solve(dist, pred, fap.MODE_BATCHED, stream=sptr)
        elif share:
            eng.solve_parts(share, dist, pred, fap.MODE_BATCHED, stream=sptr)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # the first solve tuned the SSSP; later engines on the same graph (the
    # e2e loop) take the tuned values instead of tuning again
    tuned = {o: eng.get_option(o) for o in (fap._lib.OPT_SSSP_METHOD, fap._lib.OPT_SSSP_DELTA,
                                             fap._lib.OPT_SSSP_LANES)}
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
    # whole-job distances per second: every rank's rows (n x n in all when the
    # parts are shared out, n x n per rank for replicas) over the slowest rank
    value = (world if share is None else 1) * float(n) * n / (ms_per_step / 1e3)

    ph = {k: statistics.mean(p[k] for p in phase) for k in phase[0]}
    sssp_stats = eng.sssp_stats()
    launches_per_step = eng.last_launches()  # kernels of one solve (counted by the engine)
    f32 = dtype == fap.DTYPE_F32
    # add-min peaks from registers, measured in this run: int32 DPX add-min,
    # and the form the min-plus runs (int32 with argmin, or FP32 with argmin)
    # (FP32: the kernels' own form, add-mins in groups of four steps keeping
    # the group of the last strict improvement, mode 12; int32: packed keys,
    # one DPX add-min each, mode 0; mode 3 is the one-step FP32 form)
    peak_dpx = eng_ctx_peak(fap, dev, 0)
    peak_mp = eng_ctx_peak(fap, dev, 12 if f32 else 0)
    peak_fw = peak_mp
    peak_f32_step = eng_ctx_peak(fap, dev, 3) if f32 else None

    def rate(x, ms):
        return x / (ms / 1e3) if ms and ms > 0 else float("nan")

    peaks, peak_src = read_peaks()
    hbm = float(peaks.get("hbm_gbs", HBM_PEAK_FALLBACK))
    srcs = int(bdys.sum())
    sssp_bytes = srcs * (4 * (n + 1) + 8 * g.m + 8 * n)
    mp_bytes = int(((subs - bdys) * n * 8).sum() + (bdys * n * 8).sum())  # C written + B read once
    mp_gbs = rate(mp_bytes, ph["min_plus"]) / 1e9
    # add-min steps the strip kernels actually ran (they skip the k-steps whose
    # B row or A column is unreached over a tile): one more solve with counters
    eng.minplus_counters(reset=True)
    eng.fw_counters(reset=True)
    step()
    torch.cuda.synchronize()
    mpc = eng.minplus_counters(reset=True)
    fwc = eng.fw_counters(reset=True)
    executed = int(mpc["executed_addmins"])
    fw_executed = int(fwc["strip_addmins"] + fwc["other_addmins"])

    # plain form (one launch sequence per part, the reference's loop) on the
    # same graph, for batched-vs-plain
    plain_ms = float("nan")
    if args.plain and world == 1:
        eng.solve(dist, pred, fap.MODE_PLAIN, stream=sptr)
        flush.fill_(1)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.solve(dist, pred, fap.MODE_PLAIN, stream=sptr)
        b.record(stream)
        b.synchronize()
        plain_ms = a.elapsed_time(b)
    eng.close()
    del dist, pred
    torch.cuda.empty_cache()

    # end to end through the public C ABI with host buffers: per step the CSR
    # goes host->device (fap_create from page-locked arrays) and the full
    # result rows come back device->host into page-locked rows.
    ro_h = torch.from_numpy(g.row_offset).pin_memory()
    col_h = torch.from_numpy(g.col_val).pin_memory()
    w_h = torch.from_numpy(g.weight).pin_memory()
    gid_h = torch.from_numpy(gid).pin_memory()
    e2e_ms, e2e_parts = [], []
    host_alloc = None
    link_gbs = None
    if args.e2e_steps > 0:
        npdt = np.float32 if f32 else np.int32
        dist_h, free_d, host_alloc = pinned_host((max(rows, 1), n), npdt)
        pred_h, free_p, _ = pinned_host((max(rows, 1), n), np.int32)
        # The host link's own rate into the same rows: a plain device-to-host
        # copy of the distance rows (each e2e step moves twice these bytes).
        try:
            dev_rows = torch.empty((max(rows, 1), n), dtype=tdt, device="cuda")
            dev_rows.zero_()
            host_view = torch.from_numpy(dist_h)
            best = float("inf")
            for _ in range(2):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                host_view.copy_(dev_rows, non_blocking=True)
                torch.cuda.synchronize()
                best = min(best, time.perf_counter() - t0)
            link_gbs = dev_rows.numel() * 4 / best / 1e9
            del dev_rows, host_view
            torch.cuda.empty_cache()
        except RuntimeError:
            link_gbs = None
        for i in range(1 + args.e2e_steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e = fap.Engine(n, ro_h.numpy(), col_h.numpy(), w_h.numpy(), K, graph_id=gid_h.numpy(),
                           dtype=dtype, device=dev)
            for o, v in {**options, **tuned}.items():
                e.set_option(o, v)
            tc = time.perf_counter()
            if share is None:
                e.solve(dist_h, pred_h, fap.MODE_BATCHED)
            elif share:
                e.solve_parts(share, dist_h, pred_h, fap.MODE_BATCHED)
            ts = time.perf_counter()
            e.close()
            t1 = time.perf_counter()
            if i > 0:
                e2e_ms.append((t1 - t0) * 1e3)
                e2e_parts.append(((tc - t0) * 1e3, (ts - tc) * 1e3, (t1 - ts) * 1e3))
        free_d()
        free_p()
        del dist_h, pred_h
    e2e_ms_step = statistics.mean(e2e_ms) if e2e_ms else float("nan")
    h2d = int(g.row_offset.nbytes + g.col_val.nbytes + g.weight.nbytes + gid.nbytes)
    d2h = int(rows) * n * 8

    traffic_scale = MP_TRAFFIC_PER_BYTE.get(name)
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak" if share is None else "strong", "vs_baseline": None,
        "dtype": "f32" if f32 else "int32", "data": "synthetic",
        "parallelism": (f"parts of the one graph shared out over {world} GPUs (cost-balanced, no collective on "
                        f"the rows)" if share is not None else f"replicas x{world}"),
        "config": workload_config(name, g, K, gid, cut),
        "mode": "batched (one launch per phase, CUDA graph)",
        "arithmetic": ("SSSP exact (FP64 option), rounded once to FP32; FW and min-plus in FP32" if f32 and
                       wl["fp64_sssp"] else "f32 (the reference's)" if f32 else "int32 (exact)"),
        "tuning": {"sssp_method": {1: "whole-graph search", 2: "boundary graph"}.get(
                       int(tuned[fap._lib.OPT_SSSP_METHOD]), "not tuned"),
                   "sssp_delta": tuned[fap._lib.OPT_SSSP_DELTA],
                   "sssp_lanes": int(tuned[fap._lib.OPT_SSSP_LANES])},
        "e2e": {"value": (world if share is None else 1) * float(n) * n / (e2e_ms_step / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms_step,
                "create_solve_destroy_ms": [statistics.mean(x) for x in zip(*e2e_parts)] if e2e_parts else None,
                "solve_ms_each": [round(x[1], 1) for x in e2e_parts], "host_rows": host_alloc,
                "host_link_d2h_gbs": link_gbs,
                "host_link_floor_ms": d2h / (link_gbs * 1e9) * 1e3 if link_gbs else None,
                "what": "fap_create (CSR from page-locked host arrays) + fap_solve into page-locked host rows "
                        "(n x n distances + predecessors) + fap_destroy, SSSP settings as tuned on this graph"},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": {
            # What the min-plus must always do is write the n x n rows (its
            # add-min work is data-dependent: steps that cannot change a tile
            # are skipped), so its roofline is HBM; alu_view gives the same
            # launch against the add-min issue rate of its arithmetic.
            "kernel": "mp_strip_kernel (min-plus of the inner rows and decode of their own-part columns)",
            "bound": "hbm",
            "achieved": mp_gbs, "peak": hbm, "unit": "GB/s", "frac": mp_gbs / hbm,
            "peak_source": peak_src,
            "algorithmic_bytes_per_launch": mp_bytes,
            "traffic": traffic_scale * mp_bytes if traffic_scale else None,
            "traffic_source": (f"ncu capture of the same kernel on a smaller case of this workload "
                               f"({traffic_scale} DRAM bytes per algorithmic byte), scaled")
                              if traffic_scale else "no capture of this workload",
            "alu_view": {
                "executed_addmins_per_launch": executed,
                "achieved": rate(executed, ph["min_plus"]) / 1e9, "peak": peak_mp / 1e9,
                "unit": "Gaddmin/s", "frac": rate(executed, ph["min_plus"]) / peak_mp,
                "dense_addmins_per_launch": addmin_mp,
                "strip_tiles": mpc["tiles"], "tiles_without_active_step": mpc["empty_tiles"],
                "peak_source": ("fap_addmin_peak mode 12 (FP32 add-mins in groups of four steps keeping the "
                                "group of the last strict improvement, the kernel's form)" if f32 else
                                "fap_addmin_peak mode 0 (int32 DPX add-min on packed keys, the kernel's form)")
                               + " from registers, measured in this run",
                "peak_dpx_int32": peak_dpx / 1e9,
                "peak_f32_one_step_argmin": peak_f32_step / 1e9 if peak_f32_step else None,
            },
        },
        "roofline_fw": {"achieved": rate(fw_executed, ph["floyd"]) / 1e9, "peak": peak_fw / 1e9,
                        "unit": "Gaddmin/s", "frac": rate(fw_executed, ph["floyd"]) / peak_fw,
                        "executed_addmins": fw_executed, "executed_split": fwc,
                        "dense_addmins": addmin_fw,
                        "dense_equivalent_rate": rate(addmin_fw, ph["floyd"]) / 1e9,
                        "note": "executed add-mins (fap_fw_counters: the remaining-tile strips' device counter "
                                "plus the pivot or tile launches' block products) per FW phase time, against "
                                + ("fap_addmin_peak mode 12 (FP32 add-mins in groups of four keeping the "
                                   "group of the last strict improvement)" if f32 else
                                   "fap_addmin_peak mode 0 (int32 DPX add-min)")},
        "roofline_sssp": {"bound": "hbm", "achieved": rate(sssp_bytes, ph["sssp"]) / 1e9, "peak": hbm,
                          "unit": "GB/s", "frac": rate(sssp_bytes, ph["sssp"]) / 1e9 / hbm,
                          "algorithmic_bytes": sssp_bytes, "peak_source": peak_src},
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


def cpu_sample(oracle, part, g, gid, pre, rows):
    """The reference's CPU algorithm on one part with the min-plus limited to
    `rows` inner rows; returns (extrapolated part seconds, measured seconds,
    part rows)."""
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


def load_oracle(threads):
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle  # test infrastructure: the CPU baseline, never the measured product

    oracle.build()
    oracle.set_threads(threads)
    return oracle


def cpu_baseline(name, seconds, ref_rows):
    """The oracle restatement of the reference's CPU path on whole parts, in
    order, until about `seconds` of host work; distances/s extrapolated."""
    cores = os.cpu_count() or 1
    oracle = load_oracle(cores)
    g, K, gid, _ = load_workload(name)
    pre = oracle.preprocess(K, gid, g.row_offset, g.col_val)
    rows = est = meas = 0.0
    parts = 0
    for part in range(1, K + 1):
        e_p, m_p, sub = cpu_sample(oracle, part, g, gid, pre, ref_rows)
        rows, est, meas, parts = rows + sub, est + e_p, meas + m_p, parts + 1
        if meas >= seconds:
            break
    return {"value": rows * g.n / est, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"parts 1..{parts} of {K}: SSSP (all boundary sources, OpenMP), full FW, min-plus on "
                      f"{ref_rows} inner rows per part extrapolated per add-min; {meas:.1f} s measured"}


def run_reference(args):
    """The reference's CPU algorithm (the oracle restatement of fapGraph::run's
    CPU branch, pinned bit for bit to the reference's own fap.cpp) on the same
    workload and parts as the engine's line, on all host cores: per step one
    part (SSSP from all its boundary vertices, its FW, and the min-plus on its
    first rows, extrapolated per add-min to all of its inner rows)."""
    name = args.config
    cores = os.cpu_count() or 1
    oracle = load_oracle(cores)
    g, K, gid, cut = load_workload(name)
    pre = oracle.preprocess(K, gid, g.row_offset, g.col_val)
    rates, meas = [], []
    for i in range(args.warmup + args.steps):
        part = 1 + (i % K)
        est, m, sub = cpu_sample(oracle, part, g, gid, pre, args.ref_rows)
        if i >= args.warmup:
            rates.append(sub * g.n / est)
            meas.append(m)
    value = statistics.mean(rates)
    sample = (f"per step one part of the {K} (parts in order): SSSP from all its boundary vertices (OpenMP), "
              f"its full Floyd-Warshall, and the min-plus on its first {args.ref_rows} inner rows; the part's "
              f"time is extrapolated per add-min to all its inner rows; distances/s = part rows x n / part time")
    res = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(meas) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": WORKLOADS[name]["dtype"].replace("i32", "int32"),
        "data": "synthetic",
        "config": workload_config(name, g, K, gid, cut),
        "arithmetic": "f32 (the reference's; integer weights are exact)",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    return res


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


def run_profile(args):
    """Device-resident solves only, for ncu: the workload graph (or, with
    --profile-n, a road-like graph of that size in parts of about 900
    vertices, partitioned by the engine) solved --profile-solves times; prints
    the launches of the first solve (tuning included) and of each later one,
    so that a capture can skip to one whole solve."""
    import torch

    import fastapsp_gb300 as fap

    wl = WORKLOADS[args.config]
    if args.profile_n:
        g = load_graphs_module().road_like(args.profile_n)
        K = max(2, round(args.profile_n / 895))
        gid, _ = fap.partition(g.row_offset, g.col_val, K)
    else:
        g, K, gid, _ = load_workload(args.config)
    f32 = wl["dtype"] == "f32" or bool(args.profile_n)
    eng = fap.Engine(g.n, g.row_offset, g.col_val, g.weight, K, graph_id=gid,
                     dtype=fap.DTYPE_F32 if f32 else fap.DTYPE_I32)
    if f32:
        eng.set_option(fap._lib.OPT_SSSP_FP64, 1)
    d = torch.empty((g.n, g.n), dtype=torch.float32 if f32 else torch.int32, device="cuda")
    p = torch.empty((g.n, g.n), dtype=torch.int32, device="cuda")
    counts = []
    for i in range(args.profile_solves):
        if i == args.profile_solves - 1:  # work counters of the last solve
            eng.minplus_counters(reset=True)
            eng.fw_counters(reset=True)
        eng.solve(d, p)
        torch.cuda.synchronize()
        counts.append(eng.last_launches())
    print(json.dumps({"profile": args.config, "n": g.n, "K": K, "launches_per_solve": counts,
                      "phase_ms": eng.last_times(), "minplus_counters": eng.minplus_counters(reset=True),
                      "fw_counters": eng.fw_counters(reset=True)}))


def run_profile_c3(args):
    """The batched Floyd-Warshall of the 512 dense instances only (for ncu),
    --profile-solves times, each on a fresh copy of the inputs."""
    import torch

    import fastapsp_gb300 as fap
    from fastapsp_gb300 import graphs

    mats = graphs.dense_instances()
    ctx = fap.Context(0)
    ms = []
    for _ in range(args.profile_solves):
        dev = [torch.from_numpy(m).cuda() for m in mats]
        preds = [torch.where(d < (1 << 30), torch.arange(d.shape[0], dtype=torch.int32, device="cuda")[:, None],
                             torch.full((1, 1), -1, dtype=torch.int32, device="cuda")).contiguous() for d in dev]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.floyd_batched(1, dev, preds)
        torch.cuda.synchronize()
        ms.append((time.perf_counter() - t0) * 1e3)
    ctx.close()
    print(json.dumps({"profile": "c3", "instances": len(mats), "ms_per_run": ms}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--ref-rows", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="host work of the cpu_baseline sample (whole parts until this is reached)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", dest="plain", action="store_false")
    ap.add_argument("--shard", choices=["parts", "replicas"], default="parts",
                    help="under torchrun: share the graph's parts out over the ranks (default) or solve "
                         "the whole graph on every rank")
    ap.add_argument("--profile", action="store_true",
                    help="only device-resident solves of the workload (for ncu); see run_profile")
    ap.add_argument("--profile-n", type=int, default=0, help="--profile on a road-like graph of this size")
    ap.add_argument("--profile-solves", type=int, default=4)
    ap.add_argument("--no-c3", dest="with_c3", action="store_false",
                    help="leave out the dense batched FW of 512 instances from the solve line")
    ap.add_argument("--config", choices=["c1", "c2", "c3", "c4", "c5"], default="c4",
                    help="c4 (default, the largest single-GPU workload) is the headline; c1/c2 print the same "
                         "line for their graphs, c3/c5 their own lines")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if args.config not in WORKLOADS:
            if rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no batched "
                                  "standalone FW or adjoint path; c3/c5 have no reference arm"}))
            return
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if args.profile and args.config in WORKLOADS:
        import torch

        torch.cuda.set_device(local_rank)
        run_profile(args)
        return
    if args.profile and args.config == "c3":
        import torch

        torch.cuda.set_device(local_rank)
        run_profile_c3(args)
        return
    if args.config not in WORKLOADS:
        import torch

        torch.cuda.set_device(local_rank)
        fn = {"c3": run_c3, "c5": run_c5}[args.config]
        print(json.dumps(fn(args)))
        return

    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    res = run_solve(args, args.config, rank, world, local_rank)
    if rank == 0 and args.with_c3:
        # the dense batched FW (512 int32 instances, no step can be skipped),
        # the FW kernels' own roofline beside the solve's
        c3 = run_c3(argparse.Namespace(steps=3, warmup=2))
        res["fw_dense_512"] = {k: c3[k] for k in ("value", "unit", "ms_per_step", "per_instance_ms",
                                                   "batched_speedup", "frac_of_dpx_peak", "addmins")}
    if rank == 0:
        if not args.no_cpu_baseline:
            res["cpu_baseline"] = cpu_baseline(args.config, args.cpu_seconds, args.ref_rows)
        print(json.dumps(res))
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
