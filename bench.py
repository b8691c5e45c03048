#!/usr/bin/env python3
"""Throughput of the GraphIt edge-traversal path on GB300, in GTEPS.

Workload (default, one GPU): SSSP delta-stepping on a directed R-MAT graph of
scale 22, edge factor 16 (a/b/c = 0.57/0.19/0.19, GAPBS seed 27491095), int32
weights U[1,255]; 32 sources from GAPBS's SourcePicker; one step = SSSP from all
32 sources in the batched mode (one persistent launch).  Delta is 32 (from the
configured sweep {1,8,32,128}; --delta 0 autotunes over it).  The plain path -- the reference's default
schedule, one source at a time -- is measured beside it.  Inputs are synthetic
(the reference's datasets are not available).  TEPS counts each reached
vertex's out-edges once per source (E_r).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
  torchrun ... bench.py --gpus N     (one rank per GPU; sources shard by rank)

Beside the headline the line carries the per-app comparisons on the same graph
(`apps`), the delta sweep on it and on the 4096 x 4096 grid (`sssp_sweep`), and
the other workloads at their own sizes (`other_configs`: BFS on the symmetrized
R-MAT 16, PageRank on R-MAT 24, CC on the symmetrized R-MAT 24).

The default arm runs the engine (libgg.so) through its C ABI; `--impl
reference` times the reference's CPU delta-stepping (GAPBS
OrderedProcessingOperatorNoMerge, as ported in oracle/) on the host cores.
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

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

INT_MAX = 2**31 - 1
SCALE, DEGREE = 22, 16
N_SOURCES = 32
DELTAS = (1, 8, 32, 128)
METRIC = "GTEPS per app at 1 GB300: learned+batched vs plain schedule, exact results"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=40)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--scale", type=int, default=SCALE)
    p.add_argument("--delta", type=int, default=32,
                   help="delta-stepping bucket width (both arms); 0 = autotune over {1,8,32,128}")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--tuning", default="auto",
                   help="launch shape of the batched kernel: 'auto' (autotuned on the graph), 'default' "
                        "(built-in) or 'B,C,E' (CTAs per SM, chunk, edge-parallel threshold)")
    p.add_argument("--no-apps", action="store_true",
                   help="omit the per-app comparison lines (BFS, BC, PageRank)")
    p.add_argument("--no-sweep", action="store_true",
                   help="omit the delta sweep on this graph and the 4096 x 4096 grid")
    p.add_argument("--autotune-table", metavar="PATH", default=None,
                   help="only tabulate the autotuned launch shapes of the batched kernels per graph size "
                        "(R-MAT 12-22, grids 256-2048) as markdown into PATH, then exit")
    p.add_argument("--case", choices=sorted(CASES), default=None,
                   help="only run one small workload of one kernel a few times (for profiler captures), "
                        "print its times, then exit")
    p.add_argument("--no-configs", action="store_true",
                   help="omit the lines at the other configurations' own sizes (BFS on the "
                        "symmetrized R-MAT 16, PageRank on R-MAT 24, CC on the symmetrized R-MAT 24)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_graph(scale):
    from easy_graphit_gb300 import HostGraph
    return HostGraph.rmat(scale, DEGREE)


def bench_config(scale, V, E, delta):
    """The workload, the same in both arms."""
    return {"workload": f"sssp_delta_stepping_rmat{scale}_k16_directed", "V": int(V), "E": int(E),
            "sources": N_SOURCES, "delta": int(delta), "weights": "U[1,255]",
            "graph": "R-MAT a/b/c 0.57/0.19/0.19, GAPBS generator and builder, seed 27491095; "
                     "sources from GAPBS SourcePicker",
            "l2": "inputs larger than L2 (CSR %.2f GB, distances %.2f GB)"
                  % ((4.0 * (V + 1) + 8.0 * E) / 1e9, N_SOURCES * V * 4 / 1e9)}


def reached_stats(off, dist):
    reached = (dist != INT_MAX)
    deg = np.diff(off)
    return int(reached.sum()), int(deg[reached].sum())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# -------------------------------------------------------------- CPU legs
def cpu_sssp(off, dst, w, sources, delta, budget_s):
    """GAPBS ordered-processing SSSP (oracle port) on the host cores over a
    bounded sample of the sources; returns (GTEPS, threads, n_sources, seconds)."""
    import oracle
    threads = os.cpu_count() or 1
    edges = 0
    t0 = time.perf_counter()
    n = 0
    for s in sources:
        d = oracle.sssp_ordered(off, dst, w, int(s), delta, threads)
        edges += reached_stats(off, d)[1]
        n += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return edges / dt / 1e9, threads, n, dt


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    f = ROOT / "profiles" / "sssp_batch_rmat22.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


# ------------------------------------------------------------------- arms
def run_reference(args):
    """The reference's CPU SSSP (GAPBS OrderedProcessingOperatorNoMerge, as
    ported in the oracle) on the host cores, over a graph the oracle builds
    itself (its restatement of GAPBS's generator): no engine code is loaded."""
    rank, world, _ = dist_env()
    if world > 1 and rank != 0:
        return
    import oracle
    off, dst, w = oracle.rmat(args.scale, DEGREE)
    V, E = len(off) - 1, len(dst)
    sources = oracle.pick_sources(off, N_SOURCES)
    delta = args.delta or 32
    per_step = 2  # bounded sample of the 32 sources per step
    vals = []
    for i in range(args.warmup + args.steps):
        srcs = [sources[(2 * i + k) % N_SOURCES] for k in range(per_step)]
        g, threads, n, dt = cpu_sssp(off, dst, w, srcs, delta, 1e9)
        if i >= args.warmup:
            vals.append(g)
    value = float(np.mean(vals))
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GTEPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": bench_config(args.scale, V, E, delta),
        "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": f"{per_step} of the {N_SOURCES} sources per step "
                                   f"(GAPBS OrderedProcessingOperatorNoMerge port, all host threads)"},
        "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_gb300(args):
    import ctypes as C

    import torch
    import torch.distributed as dist

    from easy_graphit_gb300 import (GraphT, LearnedGPUSchedule, Selector, _lib as L, app_schedule,
                                    autotune_batch, default_schedule, get_batch_tuning,
                                    set_batch_tuning)
    from easy_graphit_gb300 import SimpleGPUSchedule as T
    from easy_graphit_gb300.replicas import aggregate_teps, rank_sources

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    hg = make_graph(args.scale)
    off, dst, w = np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)
    V, E = hg.num_vertices, hg.num_edges
    # weak scaling: every rank traverses its own 32 sources on its own replica
    sources = rank_sources(hg, N_SOURCES, rank)
    h_src = np.ascontiguousarray(sources, dtype=np.int32)

    g = GraphT(hg)
    stream = torch.cuda.current_stream(dev)
    g.set_stream(stream.cuda_stream)
    dist_dev = torch.empty((N_SOURCES, V), dtype=torch.int32, device=dev)
    base = dist_dev.data_ptr()
    st = L.gg_stats()

    def batched(delta_, out_ptr, stats=True):
        L.call("gg_sssp_batch", g.handle, C.c_void_p(h_src.ctypes.data), N_SOURCES, delta_,
               C.c_void_p(out_ptr), C.byref(st) if stats else None)
        return st.loop_ms

    # Delta from the configured sweep, picked by a short autotune (all four
    # give identical distances).
    delta = args.delta
    if not delta:
        best = None
        for d in DELTAS:
            batched(d, base)
            t = min(batched(d, base) for _ in range(2))
            if best is None or t < best[0]:
                best = (t, d)
        delta = best[1]

    # Launch shape of the batched kernel (CTAs per SM, edges per queue entry,
    # edge-parallel threshold), autotuned on this graph; untimed.
    tuned, tune_rows = None, []
    if args.tuning == "auto":
        tuned, tune_rows = autotune_batch(g, "sssp", h_src, delta)
    elif args.tuning != "default":
        b_, c_, e_ = (int(x) for x in args.tuning.split(","))
        set_batch_tuning(g, "sssp", b_, c_, e_)
        tuned = {"blocks_per_sm": b_, "chunk": c_, "edge_parallel_max": e_}

    # Algorithmic work per source (untimed): E_r, V_r from the distances.
    batched(delta, base)
    dd = dist_dev.cpu().numpy()
    er, vr = [], []
    for i in range(N_SOURCES):
        v_r, e_r = reached_stats(off, dd[i])
        er.append(e_r)
        vr.append(v_r)
    total_edges = float(sum(er))

    # Plain path for comparison (untimed for `value`): the reference's default
    # SSSP schedule (PUSH, SPARSE, VERTEX_BASED, fused; sssp.cpp:76-79), one
    # source at a time; and the single-source TWCE fused schedule.
    def single(sch_, fuse_):
        a_ = app_schedule(sch_, fuse_)
        t_ = 0.0
        for i, s in enumerate(sources):
            L.call("gg_sssp", g.handle, C.byref(a_), int(s), delta, C.c_void_p(base + i * V * 4),
                   C.byref(st))
            t_ += st.device_ms
        return total_edges / (t_ / 1e3) / 1e9
    plain_sch, plain_fuse = default_schedule("sssp")
    plain_gteps = single(plain_sch, plain_fuse)
    twce = T()
    twce.configLoadBalancing(T.load_balancing_type.TWCE)
    twce_gteps = single(twce, True)
    learned_gteps = single(LearnedGPUSchedule(Selector.pretrained()), False)
    batched(delta, base)
    assert np.array_equal(dist_dev.cpu().numpy(), dd), "batched and single-source distances differ"

    for _ in range(args.warmup):
        batched(delta, base)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    l0 = L.lib().gg_kernel_launches()
    loop_ms = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            loop_ms.append(batched(delta, base))
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = int(L.lib().gg_kernel_launches() - l0)
    ms = ev0.elapsed_time(ev1)
    # whole job: edges of all ranks / the slowest rank's time (no data-path collective)
    value, ms = aggregate_teps(total_edges * args.steps, ms, device=dev)
    ms_per_step = ms / args.steps

    # End to end through the C ABI with host buffers: every step uploads the
    # CSR from pinned host memory into a new graph (which builds its
    # degree-ordered copy), runs the batch with the launch shape chosen above,
    # writes the distances to pinned host memory and releases the graph -- all
    # inside the timed region.  One untimed step first brings the library's
    # device memory pool to its working size; later graphs reuse that memory.
    pin = lambda a_: torch.from_numpy(a_).pin_memory()
    h_off, h_dst, h_w = pin(off), pin(dst), pin(w)
    h_out = torch.empty((N_SOURCES, V), dtype=torch.int32).pin_memory()
    h2d = off.nbytes + dst.nbytes + w.nbytes + h_src.nbytes
    d2h = N_SOURCES * V * 4
    e2e_steps = max(1, min(args.steps, 10))
    shape = get_batch_tuning(g, "sssp")

    def e2e_step():
        ge = GraphT(offsets=h_off, dst=h_dst, weights=h_w)
        ge.set_stream(stream.cuda_stream)
        set_batch_tuning(ge, "sssp", **shape)
        L.call("gg_sssp_batch", ge.handle, C.c_void_p(h_src.ctypes.data), N_SOURCES, delta,
               C.c_void_p(h_out.data_ptr()), None)
        ge.close()

    e2e_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / e2e_steps
    assert np.array_equal(h_out.numpy(), dd)
    e2e_val, e2e_ms = aggregate_teps(total_edges, e2e_ms, device=dev)

    # the comparison lines run on rank 0 only (after the timed region)
    lead = rank == 0
    apps = per_app(g, hg, off, dst, dev, stream, peaks()[0]) if lead and not args.no_apps else None
    sweep = delta_sweep(g, h_src, dist_dev, total_edges, dev) if lead and not args.no_sweep else None
    other = other_configs(peaks()[0]) if lead and not args.no_configs else None
    batched_cfg = config4(g, hg, dev) if lead and not args.no_configs else None

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    peak, peak_kind = peaks()
    alg_bytes = float(sum(12.0 * e + 16.0 * v for e, v in zip(er, vr)))
    achieved = alg_bytes / (float(np.mean(loop_ms)) / 1e3) / 1e9
    traffic = ncu_traffic()
    cpu = None
    if not args.no_cpu_baseline:
        gcpu, threads, n, dt = cpu_sssp(off, dst, w, sources, delta, 15.0)
        cpu = {"value": gcpu, "unit": "GTEPS", "cores": threads, "kind": "port",
               "sample": f"{n} of the {N_SOURCES} sources ({dt:.1f} s), GAPBS "
                         f"OrderedProcessingOperatorNoMerge port, same graph and delta"}
    out = {
        "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": bench_config(args.scale, V, E, delta),
        "comparisons": {"delta_sweep": list(DELTAS),
                        "mode": "batched: 32 sources per persistent launch (gg_sssp_batch)",
                        "plain_gteps": plain_gteps,
                        "plain_schedule": "PUSH SPARSE VERTEX_BASED fused, one source at a time (sssp.cpp default)",
                        "single_twce_gteps": twce_gteps,
                        "single_learned_gteps": learned_gteps,
                        "learned_schedule": "LearnedGPUSchedule(Selector.pretrained()), unfused, one source at a time",
                        "batch_tuning": tuned if tuned else "built-in (blocks_per_sm all that fit, chunk 256, "
                                                             "edge_parallel_max 6)",
                        "autotune_trials": len(tune_rows),
                        "batched_over_plain": value / world / plain_gteps,
                        "parallelism": f"replicas x{world}, sources by rank"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "k_bsssp", "peak_kind": peak_kind,
                     "bytes_model": "sum over sources of 12*E_r + 16*V_r per launch"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": "GTEPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms, "steps": e2e_steps, "warmup": 1,
                "step": "create graph from pinned CSR, gg_sssp_batch into pinned rows, destroy graph"},
        "clocks": clk.summary(),
        "gpu_launches": launches,
        "apps": apps,
        "sssp_sweep": sweep,
        "other_configs": other,
        "batched_config": batched_cfg,
    }
    print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def delta_sweep(g, h_src, dist_dev, total_edges, dev):
    """Batched SSSP (32 sources, one launch) over the delta sweep {1, 8, 32, 128}
    on this graph and on the 4096 x 4096 4-neighbour grid (weights U[1,1000],
    high diameter; there every source runs in a CTA of its own), plus the
    single-source fused loop on the grid (sssp.cpp's schedule, one source) at the
    same deltas.  Loop time by CUDA events; the GAPBS ordered-processing port on
    the host cores runs the same grid source at delta 128, 32 and 8 beside it.
    All deltas give the same distances (checked)."""
    import ctypes as C

    import torch

    import oracle
    from easy_graphit_gb300 import GraphT, HostGraph, default_schedule, sssp, _lib as L
    st = L.gg_stats()
    nsrc = len(h_src)

    def launch(gr, srcs, delta, out):
        L.call("gg_sssp_batch", gr.handle, C.c_void_p(srcs.ctypes.data), len(srcs), delta,
               C.c_void_p(out.data_ptr()), C.byref(st))
        return st.loop_ms

    ref = dist_dev.clone()
    rmat = {}
    for d in DELTAS:
        launch(g, h_src, d, dist_dev)
        ms = min(launch(g, h_src, d, dist_dev) for _ in range(2))
        assert torch.equal(dist_dev, ref), f"delta {d} changed the distances"
        rmat[str(d)] = {"loop_ms": ms, "gteps": total_edges / ms / 1e6}
    del ref
    hg = HostGraph.grid(4096, 4096)
    gg = GraphT(hg)
    srcs = np.ascontiguousarray(hg.pick_sources(nsrc), dtype=np.int32)
    out = torch.empty((nsrc, hg.num_vertices), dtype=torch.int32, device=dev)
    deg = torch.from_numpy(np.diff(np.array(hg.offsets)).astype(np.int64)).to(dev)
    grid = {}
    first = None
    for d in (128, 128, 32, 8, 1):
        ms = launch(gg, srcs, d, out)
        reached = out != INT_MAX
        e_r = float((reached.to(torch.int64) * deg).sum())
        if first is None:
            first = out.clone()
            continue
        assert torch.equal(out, first), f"delta {d} changed the grid distances"
        grid[str(d)] = {"loop_ms": ms, "gteps": e_r / ms / 1e6,
                        "bucket_advances_all_sources": int(st.bucket_advances)}
    del out
    d0 = first[0].cpu().numpy()
    del first
    off, dstg, w = np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)
    e_r0 = reached_stats(off, d0)[1]
    sch, fz = default_schedule("sssp")
    single = {}
    for d in (128, 32, 8, 1):
        dd, sts = sssp(gg, int(srcs[0]), d, sch, fz)
        assert np.array_equal(dd, d0), f"delta {d}: single-source distances differ from the batched ones"
        single[str(d)] = {"device_ms": sts["device_ms"], "gteps": e_r0 / sts["device_ms"] / 1e6,
                          "bucket_advances": sts["bucket_advances"], "fused": sts["fused"]}
    cpu = {}
    for d in (128, 32, 8):
        t0 = time.perf_counter()
        dd = oracle.sssp_ordered(off, dstg, w, int(srcs[0]), d, os.cpu_count() or 1)
        t = time.perf_counter() - t0
        cpu[str(d)] = {"seconds_one_source": t, "gteps": reached_stats(off, dd)[1] / t / 1e9}
    gg.close()
    return {"rmat22_batched": rmat,
            "grid4096_batched": grid,
            "grid4096_single_source_fused": single,
            "grid4096_cpu_port": cpu,
            "grid": "4096 x 4096 4-neighbour, both directions, weights U[1,1000] (V 16,777,216, E 67,092,480)",
            "note": "one timed launch per delta on the grid (after an untimed one at delta 128); "
                    "built-in launch shape (one CTA per source on the grid); single source: sssp.cpp's "
                    "schedule, fused, source 0 of the batch; CPU: GAPBS OrderedProcessingOperatorNoMerge "
                    "port, the same source, all host threads"}


def other_configs(peak):
    """The other workloads at their own sizes, device-timed through the C ABI:
    BFS on the symmetrized R-MAT 16 from its highest-degree vertex (bfs.cpp's
    PUSH TWCE fused schedule and the learned selector; the graph fits in L2, so
    its byte rate is not an HBM figure), PageRank (20 iterations) on the
    directed R-MAT 24, and CC on the symmetrized R-MAT 24, each against the
    reference app's own schedule and the OpenMP port on the host cores (CC);
    and on the same two scale-24 graphs the traversal kernels' lines
    (scale24_directed, scale24_symmetrized) with their roofline fractions."""
    import oracle
    from easy_graphit_gb300 import (GraphT, HostGraph, LearnedGPUSchedule, Selector,
                                    SimpleGPUSchedule as T, bfs, cc, default_schedule, pagerank)
    threads = os.cpu_count() or 1
    res = {}

    def best(run, reps=5):
        out, st = run()
        for _ in range(reps - 1):
            o2, s2 = run()
            if s2["device_ms"] < st["device_ms"]:
                out, st = o2, s2
        return out, st

    hg = HostGraph.rmat(16, 16, symmetrize=True)
    g = GraphT(hg, symmetric=True)
    off, dst = np.array(hg.offsets), np.array(hg.dst)
    src = int(np.argmax(np.diff(off)))
    sch, fz = default_schedule("bfs")
    def bfs2(*a_):  # (depth, stats)
        r_ = bfs(*a_)
        return r_[0], r_[2]

    d, st = best(lambda: bfs2(g, src, sch, fz))
    ok = bool(np.array_equal(d, oracle.bfs(off, dst, src)))
    er = int(np.diff(off)[d >= 0].sum())
    learned = LearnedGPUSchedule(Selector.pretrained())
    d2, st2 = best(lambda: bfs2(g, src, learned))
    t0 = time.perf_counter()
    for _ in range(5):
        oracle.bfs_omp(off, dst, src, threads)
    t = (time.perf_counter() - t0) / 5
    lines = bfs_single_lines(g, off, dst, src)
    vr = int((d >= 0).sum())
    l2 = l2_copy_gbs()
    fastest = min((v for k, v in lines.items() if isinstance(v, dict)), key=lambda v: v["ms"])
    res["bfs_rmat16_symmetrized"] = {
        "V": hg.num_vertices, "E": hg.num_edges, "source": "highest degree",
        "plain_gteps": er / st["device_ms"] / 1e6, "learned_gteps": er / st2["device_ms"] / 1e6,
        "exact": ok and bool(np.array_equal(d2, d)),
        "schedules": lines,
        "roofline_l2": {"achieved": (8.0 * er + 16.0 * vr) / (fastest["ms"] / 1e3) / 1e9, "peak": l2,
                        "unit": "GB/s", "frac": (8.0 * er + 16.0 * vr) / (fastest["ms"] / 1e3) / 1e9 / l2,
                        "bytes_model": "8 E_r + 16 V_r, fastest schedule's trial time",
                        "peak_kind": "L2 copy bandwidth measured here (16 MB working set, torch copy_)"},
        "cpu_port": {"gteps": er / t / 1e9, "cores": threads, "sample": "OpenMP port of bfs.cpp, mean of 5"},
        "note": "PUSH TWCE fused (bfs.cpp default); graph L2-resident"}
    g.close()

    hg = HostGraph.rmat(24, 16)
    g = GraphT(hg)
    E, V = hg.num_edges, hg.num_vertices
    sch, _ = default_schedule("pr")
    r_plain, st_p = best(lambda: pagerank(g, 20, 0.85, sch), 2)
    tw = T().configDirection(T.direction_type.PULL).configLoadBalancing(T.load_balancing_type.TWC)
    r_tw, st_t = best(lambda: pagerank(g, 20, 0.85, tw), 3)
    gbs = 20 * (8.0 * E + 24.0 * V) / (st_t["device_ms"] / 1e3) / 1e9
    res["pagerank_rmat24"] = {
        "V": V, "E": E, "iterations": 20,
        "plain_gteps": 20 * E / st_p["device_ms"] / 1e6, "static_pull_gteps": 20 * E / st_t["device_ms"] / 1e6,
        "rel_l1_static_vs_plain": float(np.abs(r_tw.astype(np.float64) - r_plain).sum()
                                        / np.abs(r_plain.astype(np.float64)).sum()),
        "roofline": {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "bytes_model": "20 x (8 E + 24 V)"},
        "plain_schedule": "PULL EDGE_ONLY blocked 0x42000 (pr.cpp default)"}
    res["rmat24_directed"] = scale24_directed(g, hg, peak)
    g.close()
    del hg

    hg = HostGraph.rmat(24, 16, symmetrize=True)
    g = GraphT(hg, symmetric=True)
    off, dst = np.array(hg.offsets), np.array(hg.dst)
    E = hg.num_edges
    sch, _ = default_schedule("cc")
    lab_r, st_r = best(lambda: cc(g, sch), 2)
    lab_f, st_f = best(lambda: cc(g, sch, True), 5)
    t0 = time.perf_counter()
    lab_c = oracle.cc_omp(off, dst, threads)
    t = time.perf_counter() - t0
    res["cc_rmat24_symmetrized"] = {
        "V": hg.num_vertices, "E": E,
        "plain_gteps": E / st_r["device_ms"] / 1e6, "fused_gteps": E / st_f["device_ms"] / 1e6,
        "plain_ms": st_r["device_ms"], "fused_ms": st_f["device_ms"],
        "exact": bool(np.array_equal(lab_r, lab_f) and np.array_equal(lab_f, lab_c)),
        "cpu_port": {"gteps": E / t / 1e9, "cores": threads, "sample": "whole run, OpenMP port of cc.cpp"},
        "plain_schedule": "PUSH EDGE_ONLY rounds (cc.cpp default)",
        "fused": "union-find in Afforest's sampling order",
        "roofline_fused": roof_line(16.0 * E + 8.0 * hg.num_vertices, st_f["device_ms"], peak,
                                    "one hook round 16 E + 8 V")}
    res["rmat24_symmetrized"] = scale24_symmetrized(g, hg, peak)
    g.close()
    return res


def bfs_single_lines(g, off, dst, src, reps=5):
    """One-source BFS under each schedule, best of `reps` device times: bfs.cpp's
    PUSH TWCE fused and its hybrid "power" schedule unfused (as the reference
    runs them), the same hybrid rule fused (one persistent kernel, direction
    per level on the device), and the fused loop with the selector's direction
    head (selector_fused_bfs.bin).  GTEPS = reached out-edges / time; depths
    compared across schedules."""
    from pathlib import Path

    import easy_graphit_gb300 as G
    plain, pf = G.default_schedule("bfs")
    power, _ = G.default_schedule("bfs", power=True)
    runs = [("plain_push_twce_fused", plain, pf), ("power_hybrid_unfused", power, False),
            ("power_hybrid_fused", power, True)]
    if (Path(G.__file__).resolve().parent / "selector_fused_bfs.bin").exists():
        runs.append(("learned_fused", G.LearnedGPUSchedule(G.Selector.pretrained_fused_bfs()), True))
    out, first = {}, None
    for name, sch, fz in runs:
        best = None
        for _ in range(reps):
            d, _, st = G.bfs(g, src, sch, fz)
            if best is None or st["device_ms"] < best[1]["device_ms"]:
                best = (d, st)
        d, st = best
        if first is None:
            first = d
        er = int(np.diff(off)[d >= 0].sum())
        out[name] = {"gteps": er / st["device_ms"] / 1e6, "ms": st["device_ms"],
                     "pull_levels": st["pull_iterations"], "levels": st["iterations"],
                     "exact": bool(np.array_equal(d, first))}
    fixed = max(v["gteps"] for k, v in out.items() if not k.startswith("learned"))
    if "learned_fused" in out:
        out["learned_fused_over_best_fixed"] = out["learned_fused"]["gteps"] / fixed
    return out


def l2_copy_gbs(mb=8, reps=200):
    """Copy bandwidth with a working set that stays in L2 (two buffers of `mb`
    MB, far under the 129 MB L2, which is split between the two dies): read +
    write bytes over CUDA-event time, best of three bursts."""
    import torch
    a = torch.empty(mb << 18, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    for _ in range(5):
        b.copy_(a)
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            b.copy_(a)
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * a.numel() * 4 * reps / (e0.elapsed_time(e1) / 1e3) / 1e9)
    return best


def roof_line(alg_bytes, ms, peak, model):
    gbs = alg_bytes / (ms / 1e3) / 1e9
    return {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak, "bytes_model": model}


def reach_of(deg, rows):
    """Sum over rows of (reached out-edges, reached vertices)."""
    er = vr = 0
    for r in rows:
        m = (r >= 0) & (r != INT_MAX)
        er += int(deg[m].sum())
        vr += int(m.sum())
    return er, vr


def scale24_directed(g, hg, peak):
    """R-MAT 24 directed (the 50 %-of-HBM target's scale): batched BFS (64
    sources, learned directions), batched SSSP (32 sources, delta 32), and
    single-source BFS (bfs.cpp's schedule) and SSSP (sssp.cpp's and TWCE,
    fused), each with GTEPS and its roofline fraction by the per-app byte
    model; single and batched outputs compared."""
    from easy_graphit_gb300 import (Selector, SimpleGPUSchedule as T, bfs, bfs_batch, default_schedule,
                                    set_batch_selector, sssp, sssp_batch)
    res = {}
    deg = np.diff(np.array(hg.offsets))
    srcs = np.ascontiguousarray(hg.pick_sources(64), dtype=np.int32)
    set_batch_selector(g, "bfs", Selector.pretrained_batched_bfs())
    bfs_batch(g, srcs)
    depth, st = min((bfs_batch(g, srcs) for _ in range(2)), key=lambda r_: r_[1]["loop_ms"])
    set_batch_selector(g, "bfs", None)
    er, vr = reach_of(deg, depth)
    sch, fz = default_schedule("bfs")
    bfs(g, int(srcs[0]), sch, fz)
    one, _, st1 = bfs(g, int(srcs[0]), sch, fz)
    er1, vr1 = reach_of(deg, [one])
    res["bfs"] = {"batched_learned_gteps": er / st["loop_ms"] / 1e6, "sources": 64,
                  "roofline_batched": roof_line(8.0 * er + 16.0 * vr, st["loop_ms"], peak,
                                                "8 E_r + 16 V_r per source"),
                  "single_plain_gteps": er1 / st1["device_ms"] / 1e6,
                  "roofline_single": roof_line(8.0 * er1 + 16.0 * vr1, st1["device_ms"], peak, "8 E_r + 16 V_r"),
                  "exact": bool(np.array_equal(depth[0], one))}
    del depth
    s32 = srcs[:32]
    sssp_batch(g, s32, 32)
    dist, st = min((sssp_batch(g, s32, 32) for _ in range(2)), key=lambda r_: r_[1]["loop_ms"])
    er, vr = reach_of(deg, dist)
    psch, pfz = default_schedule("sssp")
    twce = T().configLoadBalancing(T.load_balancing_type.TWCE)
    d1, stp = sssp(g, int(s32[0]), 32, psch, pfz)
    sssp(g, int(s32[0]), 32, twce, True)
    _, stt = sssp(g, int(s32[0]), 32, twce, True)
    er1, vr1 = reach_of(deg, [d1])
    res["sssp"] = {"batched_gteps": er / st["loop_ms"] / 1e6, "sources": 32, "delta": 32,
                   "roofline_batched": roof_line(12.0 * er + 16.0 * vr, st["loop_ms"], peak,
                                                 "12 E_r + 16 V_r per source"),
                   "single_plain_gteps": er1 / stp["device_ms"] / 1e6,
                   "single_twce_fused_gteps": er1 / stt["device_ms"] / 1e6,
                   "roofline_single_twce": roof_line(12.0 * er1 + 16.0 * vr1, stt["device_ms"], peak,
                                                     "12 E_r + 16 V_r"),
                   "exact": bool(np.array_equal(dist[0], d1))}
    return res


def scale24_symmetrized(g, hg, peak):
    """R-MAT 24 symmetrized: batched BC (64 sources) with its roofline."""
    from easy_graphit_gb300 import bc_batch
    deg = np.diff(np.array(hg.offsets))
    srcs = np.ascontiguousarray(hg.pick_sources(64), dtype=np.int32)
    bc_batch(g, srcs)
    dep, st = bc_batch(g, srcs)
    er2 = st["edges_traversed"]  # 2 x the reached out-edges, summed over sources
    vr = int(hg.num_vertices) * 64  # a connected graph: every vertex reached from every source
    return {"bc": {"batched_gteps": er2 / st["loop_ms"] / 1e6, "sources": 64,
                   "roofline_batched": roof_line(12.0 * er2 + 32.0 * vr, st["loop_ms"], peak,
                                                 "2 x (8 E_r + 16 V_r) + 8 E_r per source")}}


def config4(g, hg, dev):
    """The batched configuration as written: 256 BFS and 256 SSSP sources on
    R-MAT 22 replayed from CUDA-graph plans (every persistent launch of every
    group captured once), and 64 graphs of uneven size (R-MAT scales 12-20,
    edge factors 4-32, grids 256^2-2048^2) in one traversal per app."""
    import torch
    from easy_graphit_gb300 import BatchPlan, GraphT, HostGraph, Selector, bfs_batch, multigraph_batch, \
        set_batch_selector, sssp_batch
    res = {}
    off = np.array(hg.offsets)
    deg = np.diff(off)
    V = hg.num_vertices
    srcs = np.ascontiguousarray(hg.pick_sources(256, seed=7), dtype=np.int32)
    set_batch_selector(g, "bfs", Selector.pretrained_batched_bfs())
    out = torch.empty((256, V), dtype=torch.int32, device=dev)
    for app in ("bfs", "sssp"):
        plan = BatchPlan(g, app, srcs, out, delta=32)
        plan.run()
        st = min((plan.run() for _ in range(3)), key=lambda r_: r_["device_ms"])
        rows = out.cpu().numpy()
        want, _ = (bfs_batch(g, srcs) if app == "bfs" else sssp_batch(g, srcs, 32))
        reached = (rows >= 0) & (rows != INT_MAX)
        er = int((reached * deg[None, :]).sum())
        res[f"{app}256_plan"] = {"gteps": er / st["device_ms"] / 1e6, "ms": st["device_ms"],
                                 "launches_per_replay": st["launches"],
                                 "exact_vs_calls": bool(np.array_equal(rows, want))}
        plan.close()
        del rows, want
    set_batch_selector(g, "bfs", None)
    del out
    parts = HostGraph.mix(64)
    local = [int(p.pick_sources(1, seed=i)[0]) for i, p in enumerate(parts)]
    for app in ("bfs", "sssp"):
        multigraph_batch(parts, app, local, delta=32)
        r, st = multigraph_batch(parts, app, local, delta=32)
        er = sum(int(np.diff(np.array(p.offsets))[(x >= 0) & (x != INT_MAX)].sum()) for p, x in zip(parts, r))
        res[f"mix64_{app}"] = {"gteps": er / st["loop_ms"] / 1e6, "ms": st["loop_ms"],
                               "graphs": 64, "vertices": int(sum(p.num_vertices for p in parts)),
                               "edges": int(sum(p.num_edges for p in parts)), "classes": st["classes"]}
    return res


def per_app(g, hg, off, dst, dev, stream, peak):
    """Plain (the app's own schedule, one source at a time) against the batched
    or static-gather path on the same graph, device-timed; outputs compared.
    `roofline` gives the fast path's algorithmic bytes (per-app model, summed
    over sources) over its loop time, as a fraction of the measured copy
    bandwidth."""
    import torch

    def roof(alg_bytes, ms, model):
        gbs = alg_bytes / (ms / 1e3) / 1e9
        return {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak, "bytes_model": model}

    from easy_graphit_gb300 import (SimpleGPUSchedule as T, bc, bc_batch, bfs, bfs_batch, cc,
                                    default_schedule, pagerank)
    import oracle
    E = hg.num_edges
    V = hg.num_vertices
    threads = os.cpu_count() or 1
    srcs = np.ascontiguousarray(hg.pick_sources(64, seed=27491095), dtype=np.int32)
    res = {}

    def cpu_leg(fn):  # one bounded CPU run of an oracle port: (result, seconds)
        t0 = time.perf_counter()
        r_ = fn()
        return r_, time.perf_counter() - t0
    # BFS: bfs.cpp's PUSH TWCE fused per source vs 64 sources per launch
    sch, fz = default_schedule("bfs")
    t_plain, er, vr, rows = 0.0, 0, 0, []
    for s in srcs:
        d, _, st = bfs(g, int(s), sch, fz)
        t_plain += st["device_ms"]
        er += int(np.diff(off)[d >= 0].sum())
        vr += int((d >= 0).sum())
        rows.append(d)
    bfs_batch(g, srcs)
    depth, st = min((bfs_batch(g, srcs) for _ in range(3)), key=lambda r_: r_[1]["loop_ms"])
    # learned + batched: the direction of every level chosen on the device by
    # the shipped selector network (trained on engine-made per-level timings)
    from easy_graphit_gb300 import Selector, set_batch_selector, set_batch_tuning
    model = Selector.pretrained_batched_bfs()
    set_batch_selector(g, "bfs", model)
    bfs_batch(g, srcs)
    depth_l, st_l = min((bfs_batch(g, srcs) for _ in range(3)), key=lambda r_: r_[1]["loop_ms"])
    set_batch_selector(g, "bfs", None)
    set_batch_tuning(g, "bfs", bottom_up_div=-1)
    _, st_td = min((bfs_batch(g, srcs) for _ in range(3)), key=lambda r_: r_[1]["loop_ms"])
    set_batch_tuning(g, "bfs")
    res["bfs"] = {"sources": len(srcs), "plain_gteps": er / t_plain / 1e6,
                  "batched_gteps": er / st["loop_ms"] / 1e6,
                  "learned_batched_gteps": er / st_l["loop_ms"] / 1e6,
                  "batched_top_down_only_gteps": er / st_td["loop_ms"] / 1e6,
                  "learned_batched_over_plain": t_plain / st_l["loop_ms"],
                  "exact": bool(np.array_equal(depth, np.stack(rows)) and np.array_equal(depth_l, depth)),
                  "plain_schedule": "PUSH TWCE fused (bfs.cpp default)",
                  "batched_rule": "bottom-up when the frontier holds more than V/bottom_up_div vertices",
                  "learned": "per-level direction by the selector network on the device (selector_batched_bfs.bin)",
                  "roofline": roof(8.0 * er + 16.0 * vr, st_l["loop_ms"], "sum over sources of 8 E_r + 16 V_r")}
    rows_c, t = cpu_leg(lambda: [oracle.bfs_omp(off, dst, int(x), threads) for x in srcs[:4]])
    er_c = sum(int(np.diff(off)[d_ >= 0].sum()) for d_ in rows_c)
    res["bfs"]["cpu_port"] = {"gteps": er_c / t / 1e9, "cores": threads,
                              "sample": "4 of the 64 sources, OpenMP port of bfs.cpp (oracle)"}
    res["bfs"]["single_source_schedules"] = bfs_single_lines(g, off, dst, int(srcs[0]))
    # BC: bc.cpp's PUSH TWCE fused per source vs 64 sources per launch
    sch, fz = default_schedule("bc")
    t_plain, er2, rows = 0.0, 0, []
    for s in srcs:
        dep, st = bc(g, int(s), sch, fz)
        t_plain += st["device_ms"]
        er2 += st["edges_traversed"]
        rows.append(dep)
    bc_batch(g, srcs)
    dep_b, st = bc_batch(g, srcs)
    ref = np.stack(rows).astype(np.float64)
    rel = float(np.abs(dep_b - ref).sum() / max(np.abs(ref).sum(), 1e-300))
    res["bc"] = {"sources": len(srcs), "plain_gteps": er2 / t_plain / 1e6,
                 "batched_gteps": st["edges_traversed"] / st["loop_ms"] / 1e6,
                 "rel_l1_batched_vs_plain": rel,
                 "plain_schedule": "PUSH TWCE fused (bc.cpp default); TEPS = 2 E_r / t",
                 "roofline": roof(24.0 * er + 32.0 * vr, st["loop_ms"],
                                  "sum over sources of 2 x (8 E_r + 16 V_r) + 8 E_r")}
    _, t = cpu_leg(lambda: oracle.bc(off, dst, int(srcs[0])))
    er0 = int(np.diff(off)[rows_c[0] >= 0].sum())
    res["bc"]["cpu_port"] = {"gteps": 2 * er0 / t / 1e9, "cores": 1,
                             "sample": "1 source, FP64 restatement of bc.cpp (oracle), one thread"}
    # CC: cc.cpp's EDGE_ONLY hook / pointer-jump rounds vs the fused union-find pass
    sch, _ = default_schedule("cc")
    cc(g, sch)
    lab_r, st_r = cc(g, sch)
    cc(g, sch, True)
    lab_f, st_f = min((cc(g, sch, True) for _ in range(3)), key=lambda r_: r_[1]["device_ms"])
    res["cc"] = {"plain_gteps": E / st_r["device_ms"] / 1e6, "fused_gteps": E / st_f["device_ms"] / 1e6,
                 "exact": bool(np.array_equal(lab_r, lab_f)), "plain_rounds": st_r["iterations"],
                 "plain_schedule": "PUSH EDGE_ONLY rounds (cc.cpp default); TEPS = E / t (weak components)",
                 "fused": "union-find in Afforest's sampling order (csrc/cc_uf.cu)"}
    _, t = cpu_leg(lambda: oracle.cc_omp(off, dst, threads))
    res["cc"]["cpu_port"] = {"gteps": E / t / 1e9, "cores": threads,
                             "sample": "whole run, OpenMP port of cc.cpp's hook / jump rounds (oracle)"}
    # PageRank: pr.cpp's PULL EDGE_ONLY blocked vs PULL TWC (static in-degree bins)
    sch, _ = default_schedule("pr")
    pagerank(g, 20, 0.85, sch)
    r_plain, st_p = pagerank(g, 20, 0.85, sch)
    tw = T().configDirection(T.direction_type.PULL).configLoadBalancing(T.load_balancing_type.TWC)
    pagerank(g, 20, 0.85, tw)
    r_tw, st_t = pagerank(g, 20, 0.85, tw)
    res["pr"] = {"iterations": 20, "plain_gteps": 20 * E / st_p["device_ms"] / 1e6,
                 "static_pull_gteps": 20 * E / st_t["device_ms"] / 1e6,
                 "rel_l1_static_vs_plain": float(np.abs(r_tw.astype(np.float64) - r_plain).sum()
                                                 / np.abs(r_plain.astype(np.float64)).sum()),
                 "plain_schedule": "PULL EDGE_ONLY blocked 0x42000 (pr.cpp default)",
                 "roofline": roof(20 * (8.0 * E + 24.0 * hg.num_vertices), st_t["device_ms"],
                                  "20 x (8 E + 24 V)")}
    order = np.argsort(dst, kind="stable")
    tsrc = np.repeat(np.arange(V, dtype=np.int32), np.diff(off))[order]
    toff = np.concatenate([[0], np.cumsum(np.bincount(dst, minlength=V))]).astype(np.int32)
    del order
    _, t = cpu_leg(lambda: oracle.pagerank_omp(toff, tsrc, np.diff(off).astype(np.int32), 20, 0.85, threads))
    res["pr"]["cpu_port"] = {"gteps": 20 * E / t / 1e9, "cores": threads,
                             "sample": "20 iterations, OpenMP pull port of pr.cpp (oracle)"}
    return res


def autotune_table(path, delta=32):
    """gg_batch_autotune for batched BFS (64 sources), SSSP (32 sources) and BC
    (64 sources) on R-MAT graphs of scale 12 to 22 (edge factor 16; BC and grids
    symmetric) and grids of side 256 to 2048: the chosen CTAs per SM, chunk,
    edge-parallel threshold and bottom-up divisor, with the tuned and built-in
    launch shapes' times (CUDA events around one persistent launch)."""
    from easy_graphit_gb300 import GraphT, HostGraph, autotune_batch, set_batch_tuning
    sizes = [("rmat", 12), ("rmat", 14), ("rmat", 16), ("rmat", 18), ("rmat", 20), ("rmat", 22),
             ("grid", 256), ("grid", 1024), ("grid", 2048)]
    apps = [("bfs", 64), ("sssp", 32), ("bc", 64)]
    lines = ["| graph | V | E | app | sources | CTAs/SM | chunk | edge-parallel max | bottom-up div | "
             "tuned ms | built-in ms | trials |", "|---|---|---|---|---|---|---|---|---|---|---|---|"]
    t0 = time.time()
    for kind, size in sizes:
        for app, nsrc in apps:
            sym = app == "bc" or (kind == "grid" and app == "bfs")  # grid weights differ per direction
            hg = HostGraph.rmat(size, 16, symmetrize=sym) if kind == "rmat" else HostGraph.grid(size, size)
            g = GraphT(hg, symmetric=sym)
            name = (f"R-MAT {size}{' sym' if sym else ''}" if kind == "rmat" else f"grid {size}x{size}")
            if kind == "grid" and app == "sssp":  # meshes: one CTA per source, no launch shape to tune
                from easy_graphit_gb300 import sssp_batch
                srcs = hg.pick_sources(nsrc)
                sssp_batch(g, srcs, delta)
                ms = min(sssp_batch(g, srcs, delta)[1]["loop_ms"] for _ in range(2))
                lines.append(f"| {name} | {hg.num_vertices} | {hg.num_edges} | {app} | {nsrc} | "
                             f"one CTA per source | - | - | - | {ms:.3f} | - | 0 |")
                print(lines[-1], flush=True)
                g.close()
                continue
            best, rows = autotune_batch(g, app, hg.pick_sources(nsrc), delta)
            fit = max(t["blocks_per_sm"] for t, _ in rows)
            ms = min(m for t, m in rows if t == best)
            base = next((m for t, m in rows if t["blocks_per_sm"] == fit and t["chunk"] in (0, 256)
                         and t["edge_parallel_max"] in (0, 6) and t["bottom_up_div"] in (0, 16)), None)
            lines.append(f"| {name} | {hg.num_vertices} | {hg.num_edges} | {app} | {nsrc} | "
                         f"{best['blocks_per_sm']} | {best['chunk'] if app != 'bfs' else '-'} | "
                         f"{best['edge_parallel_max'] if app == 'sssp' else '-'} | "
                         f"{best['bottom_up_div'] if app == 'bfs' else '-'} | {ms:.3f} | "
                         f"{'-' if base is None else f'{base:.3f}'} | {len(rows)} |")
            print(lines[-1], flush=True)
            set_batch_tuning(g, app)
            g.close()
    text = "\n".join(lines) + f"\n\n({time.time() - t0:.0f} s; delta {delta} for SSSP)\n"
    Path(path).write_text(text)


def run_case(name, reps=3):
    """One small workload per kernel, sized for profiler captures (inputs larger
    than L2, a few GB on the device at most): prints the device times."""
    from easy_graphit_gb300 import (GraphT, HostGraph, LearnedGPUSchedule, Selector, SimpleGPUSchedule as T,
                                    bc_batch, bfs, bfs_batch, cc, default_schedule, pagerank,
                                    set_batch_selector, sssp, sssp_batch)
    kind, what = CASES[name]
    if kind == "grid":
        hg, sym = HostGraph.grid(2048, 2048), False
    else:
        hg, sym = HostGraph.rmat(20, 16, symmetrize=kind == "rmat20s"), kind == "rmat20s"
    g = GraphT(hg, symmetric=sym)
    off = np.array(hg.offsets)
    hub = int(np.argmax(np.diff(off)))
    srcs = np.ascontiguousarray(hg.pick_sources(64), dtype=np.int32)
    times = []
    for _ in range(reps):
        if what == "sssp_single":
            sch, fz = default_schedule("sssp")
            st = sssp(g, int(srcs[0]), 32, sch, fz)[1]
        elif what == "sssp_batch":
            st = sssp_batch(g, srcs[:32], 32)[1]
        elif what == "bfs_learned_fused":
            st = bfs(g, hub, LearnedGPUSchedule(Selector.pretrained_fused_bfs()), True)[2]
        elif what == "bfs_batch_learned":
            set_batch_selector(g, "bfs", Selector.pretrained_batched_bfs())
            st = bfs_batch(g, srcs)[1]
        elif what == "bc_batch":
            st = bc_batch(g, srcs)[1]
        elif what == "pr_static_pull":
            st = pagerank(g, 20, 0.85, T().configDirection(T.direction_type.PULL)
                          .configLoadBalancing(T.load_balancing_type.TWC))[1]
        elif what == "cc_fused":
            st = cc(g, None, True)[1]
        times.append(round(st["loop_ms"] or st["device_ms"], 3))
    print(json.dumps({"case": name, "V": hg.num_vertices, "E": hg.num_edges, "loop_ms": times}))
    g.close()


# name -> (graph, workload) of run_case
CASES = {
    "sssp_grid2048_single": ("grid", "sssp_single"),
    "sssp_grid2048_batched": ("grid", "sssp_batch"),
    "sssp_rmat20_batched": ("rmat20", "sssp_batch"),
    "bfs_rmat20s_learned_fused": ("rmat20s", "bfs_learned_fused"),
    "bfs_rmat20_batched_learned": ("rmat20", "bfs_batch_learned"),
    "bc_rmat20s_batched": ("rmat20s", "bc_batch"),
    "pr_rmat20_static_pull": ("rmat20", "pr_static_pull"),
    "cc_rmat20s_fused": ("rmat20s", "cc_fused"),
}


def main():
    args = parse()
    if args.case:
        run_case(args.case)
        return
    if args.autotune_table:
        autotune_table(args.autotune_table)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
