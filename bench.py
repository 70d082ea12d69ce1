#!/usr/bin/env python3
"""Benchmark of the GB300 Delaunay build on the 1M-point 3D workload.

One step = one complete triangulation of N = 1,000,000 points i.i.d. uniform in
[0,1)^3 (seeded splitmix64) into the exact Delaunay graph: super-simplex
sizing, round-parallel insertion of every point, sorted edge list.

  value   Mpts/s with the points resident in HBM and the edge list written to
          HBM (vd_delaunay_device on a reused tree), CUDA-event timed per step.
  e2e     the same through the reference-facing one-shot call with host
          buffers (vd_delaunay_tree: pinned host points in, pinned host uint32
          edge pairs out), copies inside the timed region.
  roofline  dominant kernel of the build, achieved algorithmic bytes per launch
          over its CUDA-event launch time (events recorded by the library on the
          build's stream during a second timed region of K steps).

Between timed steps the L2 (129 MB) is flushed by writing a 256 MB buffer.
`--impl reference` times the reference's parallel CPU path, restated in C++
(oracle/: 1e5 sequential inserts, then 2-ring queue, greedy rounds and
per-round parallel updates on all host threads), on the same 1M points.
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpts/s 3D 1M exact graph"
N_POINTS = 1_000_000
SEED = 0x5EED

# Algorithmic bytes per unit: k_cavity moves one 32-byte simplex record and
# four 32-byte split-coordinate records per conflict test; the decide half of
# the check reads a candidate's claims and lists (~1264 B) and the commit half
# writes a winner's star (~1240 B).
BYTES_PER_TEST_3D = 160
BYTES_PER_CHECK = 1264
BYTES_PER_WIN = 1240


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=N_POINTS)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-subs", action="store_true", help="skip the C1 / C3 / C4-sample records of the c2 line")
    p.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "c5"],
                   help="c2: 1M-point 3D build (the headline line); c3: near-degenerate 262,144 points with "
                        "predicate fallback rates; c4: 4,096 sets batched vs one set per launch; c5: Poisson "
                        "request stream through the serving loop")
    p.add_argument("--requests", type=int, default=20_000, help="c5: requests in the stream")
    p.add_argument("--slots", type=int, default=3, help="c5: server slots")
    p.add_argument("--max-batch-points", type=int, default=2_000_000, help="c5: largest batch a slot forms")
    return p.parse_args()


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel):
    """dram bytes per launch of `kernel` from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_c2_1m.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=5)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) < 9:
                continue
            for k, name in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


CPU_PREFIX = 100_000  # points the reference inserts one at a time first (src/lib.rs:108)


def cpu_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


def cpu_sample_desc(threads, n):
    return (f"{n} points, the full workload (1M i.i.d. uniform in [0,1)^3, splitmix64 seed 0xD1A00002), per step: "
            f"the reference's parallel path restated in C++ (oracle/, not the crate: no Rust toolchain here) on "
            f"{threads} host threads -- the first {CPU_PREFIX} points inserted one at a time as src/lib.rs:108-114 "
            f"does, the rest through 2-ring queue, greedy round placement and per-round parallel updates "
            f"(src/scheduler.rs, src/delaunay_tree.rs:336-386), exact predicates, sorted edge list")


def cpu_build(p, threads):
    from oracle import oracle as O
    t0 = time.perf_counter()
    tri = O.Triangulation(p, seed=SEED, threads=threads, prefix=CPU_PREFIX)
    _ = tri.edges()
    return time.perf_counter() - t0


def cpu_baseline(pts):
    """The reference's parallel CPU path (C++ restatement, all host threads),
    one build of the full workload."""
    threads = cpu_threads()
    dt = cpu_build(pts, threads)
    return {"value": round(len(pts) / dt / 1e6, 4), "unit": "Mpts/s", "cores": threads, "kind": "port",
            "seconds": round(dt, 2), "sample": cpu_sample_desc(threads, len(pts))}


def run_reference(args, rank):
    """The reference arm: the CPU restatement of the reference's parallel path
    on the same 1M-point workload as the GPU arm (warm-up on a 20k sample)."""
    if rank != 0:
        return
    from voronoids_gb300 import workloads as W
    threads = cpu_threads()
    p = W.c2_points() if args.n == N_POINTS else W.uniform_points(args.n, 3, W.config_seed(2))
    for _ in range(args.warmup):
        cpu_build(p[:20_000], threads)
    times = [cpu_build(p, threads) for _ in range(args.steps)]
    ms = 1e3 * float(np.mean(times))
    v = len(p) / (ms / 1e3) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "Mpts/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "1M points i.i.d. uniform in [0,1)^3 (splitmix64 seed 0xD1A00002), exact 3D "
                               "Delaunay tetrahedralization, sorted input-index edge list (the GPU arm's workload); "
                               "warm-up steps on its first 20,000 points", "points": len(p)},
        "cpu_baseline": {"value": round(v, 4), "unit": "Mpts/s", "cores": threads, "kind": "port",
                         "sample": cpu_sample_desc(threads, len(p))},
        "e2e": {"value": round(v, 4), "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def golden_digest(name):
    """(rows, sha256) of the oracle's edge list of a workload (tests/golden/big_edges.json)."""
    with open(os.path.join(ROOT, "tests", "golden", "big_edges.json")) as f:
        g = json.load(f)[name]
    return g["edges"], g["sha256"]


def edge_digest(uv_dev, m):
    """(rows, sha256) of the first m device uint32 edge pairs as little-endian int64."""
    import hashlib
    e = uv_dev[:m].cpu().numpy().astype("<i8")
    return int(e.shape[0]), hashlib.sha256(np.ascontiguousarray(e).tobytes()).hexdigest()


def timed_builds(L, tree, pts_d, n, uv_d, cap, steps, warmup, flush, stream):
    """CUDA-event milliseconds of `steps` builds (vd_delaunay_device), L2 flushed before each."""
    import torch
    m = ctypes.c_int64(0)

    def step():
        rc = L.vd_delaunay_device(tree, ctypes.c_void_p(pts_d.data_ptr()), n, SEED, ctypes.c_void_p(uv_d.data_ptr()),
                                  cap, ctypes.byref(m))
        if rc not in (0, 4):
            raise SystemExit(f"vd_delaunay_device failed: {rc}")

    for _ in range(warmup):
        step()
    times = []
    for _ in range(steps):
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return times, int(m.value)


def measure_c1(L, steps, flush):
    """C1: 10,000 uniform 2D points.  GPU build (device-resident, events),
    parity with the oracle's digest, and the reference's own path for this
    size -- sequential insert_point calls (src/lib.rs:117-121), restated with
    its float conflict test on one host thread."""
    import torch
    from voronoids_gb300 import workloads as W
    pts_h = W.c1_points()
    n = len(pts_h)
    pts_d = torch.from_numpy(pts_h).cuda()
    cap = 4 * n + 1024
    uv_d = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    st = ctypes.c_int(0)
    tree = ctypes.c_void_p(L.vd_tree_new_device(2, ctypes.c_void_p(pts_d.data_ptr()), n,
                                                ctypes.c_void_p(stream.cuda_stream), ctypes.byref(st)))
    times, m = timed_builds(L, tree, pts_d, n, uv_d, cap, steps, 3, flush, stream)
    L.vd_tree_free(tree)
    rows, sha = edge_digest(uv_d, m)
    ms = float(np.mean(times))
    from oracle import oracle as O
    cpu = []
    for _ in range(5):
        t0 = time.perf_counter()
        f = O.FloatTriangulation(pts_h)
        _ = f.edges()
        cpu.append(time.perf_counter() - t0)
    cpu_s = float(np.median(cpu))
    return {"points": n, "value": round(n / (ms / 1e3) / 1e6, 4), "unit": "Mpts/s", "ms_per_step": round(ms, 3),
            "edges": m, "parity_oracle_digest": (rows, sha) == golden_digest("c1"),
            "cpu_baseline": {"value": round(n / cpu_s / 1e6, 4), "unit": "Mpts/s", "cores": 1, "kind": "port",
                             "sample": "the full 10,000 points per run, median of 5: the reference's sequential "
                                       "path (new + insert_point per point, src/lib.rs:117-121 and "
                                       "src/delaunay_tree.rs:33-211) restated in C++ with its f64 circumsphere "
                                       "and strict in_sphere test (oracle/ FloatTriangulation)"}}


def measure_c3(L, steps, warmup, flush):
    """C3: 262,144 near-degenerate 3D points: time, per-stage fallback rates of
    the predicate tiers, the validator and the oracle's digest."""
    import torch
    from voronoids_gb300 import _native
    from voronoids_gb300 import workloads as W
    pts_h = W.c3_points()
    n = len(pts_h)
    pts_d = torch.from_numpy(pts_h).cuda()
    cap = 10 * n + 1024
    uv_d = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    st = ctypes.c_int(0)
    tree = ctypes.c_void_p(L.vd_tree_new_device(3, ctypes.c_void_p(pts_d.data_ptr()), n,
                                                ctypes.c_void_p(stream.cuda_stream), ctypes.byref(st)))
    times, m = timed_builds(L, tree, pts_d, n, uv_d, cap, steps, warmup, flush, stream)
    s1 = _native.VdStats()
    L.vd_get_stats(tree, ctypes.byref(s1))
    stats = {k: getattr(s1, k) for k, _ in s1._fields_}
    ok = ctypes.c_int(0)
    viol = np.zeros(6, dtype=np.int64)
    L.vd_check_delaunay(tree, ctypes.byref(ok), viol.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    L.vd_tree_free(tree)
    rows, sha = edge_digest(uv_d, m)
    tot = stats["pred_f32"] + stats["pred_f64"] + stats["pred_exact"]
    ms = float(np.mean(times))
    return {
        "points": n, "value": round(n / (ms / 1e3) / 1e6, 4), "unit": "Mpts/s", "ms_per_step": round(ms, 3),
        "steps": steps,
        "predicates": {"decided_f32_filter": stats["pred_f32"], "decided_f64_filter": stats["pred_f64"],
                       "decided_exact": stats["pred_exact"], "of_exact_by_perturbation": stats["pred_sos"],
                       "fallback_rate_f32_to_f64": round((stats["pred_f64"] + stats["pred_exact"]) / max(tot, 1), 6),
                       "fallback_rate_f64_to_exact": round(stats["pred_exact"] /
                                                           max(stats["pred_f64"] + stats["pred_exact"], 1), 6)},
        "validator_ok": bool(ok.value), "violations": viol.tolist(), "edges": m,
        "parity_oracle_digest": (rows, sha) == golden_digest("c3"),
        "build_stats": {k: stats[k] for k in ("rounds", "max_cavity", "max_facets", "spilled", "cavity_tests")},
    }


def run_c3(args):
    """Near-degenerate 3D build (jittered lattice + tight Gaussian clusters):
    time, exactness and the share of predicates each precision tier decided."""
    import torch
    from voronoids_gb300 import _native
    L = _native.load()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    clk = Clocks(0)
    clk.start()
    r = measure_c3(L, args.steps, max(args.warmup, 3), flush)
    clocks = clk.stop()
    line = {
        "metric": "Mpts/s 3D near-degenerate build; predicate tier shares", "value": r["value"],
        "unit": "Mpts/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": C3_DESC, "points": r["points"], "l2": "flushed between steps (256 MB write)"},
        "predicates": r["predicates"], "validator_ok": r["validator_ok"], "violations": r["violations"],
        "edges": r["edges"], "parity_oracle_digest": r["parity_oracle_digest"], "build_stats": r["build_stats"],
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


C3_DESC = ("262,144 3D points: 131,072 distinct sites of the 64^3 lattice (i/64) with uniform jitter +-1e-12 per "
           "coordinate, 131,072 from 64 Gaussians (centres uniform in the cube, sigma 0.01, not clipped); "
           "splitmix64 seed 0xD1A00003")


def measure_c4(L, nsets, steps, warmup, flush, autotune):
    """`nsets` independent 3D sets (log-uniform 32..65,536 points): one batched
    build per step against one build per set on the same GPU, set by set equal."""
    import torch
    from voronoids_gb300 import workloads as W
    pts_h, off = W.c4_sets(nsets)
    n = int(off[-1])
    pts_d = torch.from_numpy(pts_h).cuda()
    cap = 9 * n
    uv_d = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    st = ctypes.c_int(0)
    tree = ctypes.c_void_p(L.vd_tree_create(3, ctypes.c_void_p(stream.cuda_stream), ctypes.byref(st)))
    eoff = np.zeros(nsets + 1, dtype=np.int64)
    i64p = ctypes.POINTER(ctypes.c_int64)
    offp = off.astype(np.int64)
    tuned = None
    if autotune:
        # launch shape and round settings tuned on a 2M-point sample of the sets
        tv = np.zeros(9, dtype=np.int64)
        rc = L.vd_autotune_batch(tree, ctypes.c_void_p(pts_d.data_ptr()), offp.ctypes.data_as(i64p), nsets,
                                 2_000_000, tv.ctypes.data_as(i64p))
        if rc not in (0, 4):
            raise SystemExit(f"vd_autotune_batch failed: {rc}")
        tuned = dict(zip(("warps_per_sm", "blocks_per_sm", "passes", "thin", "ratio_x1000", "sample_us",
                          "sample_points", "sample_sets", "adjacent"), tv.tolist()))

    def batched():
        rc = L.vd_batch_delaunay_device(tree, ctypes.c_void_p(pts_d.data_ptr()), offp.ctypes.data_as(i64p), nsets,
                                        SEED, ctypes.c_void_p(uv_d.data_ptr()), cap, eoff.ctypes.data_as(i64p))
        if rc not in (0, 4):
            raise SystemExit(f"vd_batch_delaunay_device failed: {rc}")

    for _ in range(warmup):
        batched()
    times = []
    launches0 = L.vd_kernel_launches()
    for _ in range(steps):
        flush.fill_(1)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batched()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    launches = (L.vd_kernel_launches() - launches0) // max(steps, 1)
    ok = ctypes.c_int(0)
    L.vd_check_delaunay(tree, ctypes.byref(ok), None)
    ms = float(np.mean(times))
    ref_edges = uv_d[: int(eoff[-1])].clone()
    ref_eoff = eoff.copy()
    # one set per launch on a second tree, compared set by set
    t2 = ctypes.c_void_p(L.vd_tree_create(3, ctypes.c_void_p(stream.cuda_stream), ctypes.byref(st)))
    out2 = torch.empty((9 * 65536 + 1024, 2), dtype=torch.int32, device="cuda")
    m = ctypes.c_int64(0)
    L.vd_delaunay_device(t2, ctypes.c_void_p(pts_d.data_ptr()), int(off[1]), SEED, ctypes.c_void_p(out2.data_ptr()),
                         out2.shape[0], ctypes.byref(m))
    mismatch = 0
    one_ms = 0.0
    for k in range(nsets):
        a, b = int(off[k]), int(off[k + 1])
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rc = L.vd_delaunay_device(t2, ctypes.c_void_p(pts_d.data_ptr() + 24 * a), b - a, SEED,
                                  ctypes.c_void_p(out2.data_ptr()), out2.shape[0], ctypes.byref(m))
        e1.record(stream)
        e1.synchronize()
        one_ms += e0.elapsed_time(e1)
        if rc not in (0, 4) or m.value != ref_eoff[k + 1] - ref_eoff[k] or \
                not torch.equal(out2[: m.value], ref_edges[ref_eoff[k]:ref_eoff[k + 1]]):
            mismatch += 1
    L.vd_tree_free(t2)
    return {"tree": tree, "points": n, "sets": nsets, "offsets": offp, "pts_h": pts_h, "cap": cap,
            "value": round(n / (ms / 1e3) / 1e6, 4), "unit": "Mpts/s", "ms_per_step": round(ms, 3),
            "one_set_per_launch": {"value": round(n / (one_ms / 1e3) / 1e6, 4), "unit": "Mpts/s",
                                   "ms_total": round(one_ms, 1), "mismatching_sets": mismatch},
            "batched_over_one_set_per_launch": round(one_ms / ms, 2), "autotuned": tuned,
            "validator_ok": bool(ok.value), "edges": int(ref_eoff[-1]), "gpu_launches": int(launches)}


def measure_reference_pattern(L, n_seq=CPU_PREFIX):
    """voronoids.delaunay's own call pattern on the 1M-point workload
    (src/lib.rs:104-125): new, then the first 1e5 points one insert_point
    call each (vd_insert_point: one single-warp launch per point), then
    add_points_to_tree for the rest (vd_insert_points), then the edge list.
    Wall clock from host points to host edges; the edges must equal the
    oracle's digest."""
    from voronoids_gb300 import workloads as W
    import torch
    pts = W.c2_points()
    n = len(pts)
    st = ctypes.c_int(0)
    dp = ctypes.POINTER(ctypes.c_double)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tree = ctypes.c_void_p(L.vd_tree_new(3, pts.ctypes.data_as(dp), n, ctypes.byref(st)))
    base = pts.ctypes.data
    for i in range(n_seq):
        rc = L.vd_insert_point(tree, ctypes.cast(ctypes.c_void_p(base + 24 * i), dp))
        if rc != 0:
            raise SystemExit(f"vd_insert_point failed: {rc}")
    t1 = time.perf_counter()
    rest = np.ascontiguousarray(pts[n_seq:])
    rc = L.vd_insert_points(tree, rest.ctypes.data_as(dp), n - n_seq, SEED)
    if rc != 0:
        raise SystemExit(f"vd_insert_points failed: {rc}")
    m = ctypes.c_int64(0)
    L.vd_num_edges(tree, ctypes.byref(m))
    uv = np.zeros((m.value, 2), dtype=np.int64)
    L.vd_edges(tree, uv.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), m.value, ctypes.byref(m))
    t2 = time.perf_counter()
    L.vd_tree_free(tree)
    import hashlib
    digest = (int(uv.shape[0]), hashlib.sha256(np.ascontiguousarray(uv, dtype="<i8").tobytes()).hexdigest())
    return {"points": n, "sequential_points": n_seq, "sequential_s": round(t1 - t0, 3),
            "us_per_insert_point": round(1e6 * (t1 - t0) / n_seq, 2), "rest_s": round(t2 - t1, 3),
            "total_s": round(t2 - t0, 3), "value": round(n / (t2 - t0) / 1e6, 4), "unit": "Mpts/s",
            "parity_oracle_digest": digest == golden_digest("c2")}


def run_c4_ranks(args, world, rank, local):
    """C4 across ranks (torchrun, one process per GPU): each rank builds its
    share of the 4,096 sets (longest-processing-time assignment by size,
    voronoids_gb300.shard.lpt_assign) as one batched build per step, with no
    collective on the data path; the step time is the maximum over ranks and
    `value` is all ranks' points over it.  VD_DIST_BACKEND=gloo runs the
    barriers and the reduction on the host (several ranks on one GPU, for
    testing); the default is NCCL."""
    import torch
    import torch.distributed as dist
    from voronoids_gb300 import _native, shard
    from voronoids_gb300 import workloads as W
    dev = local % max(torch.cuda.device_count(), 1)  # several ranks may share one GPU (gloo test runs)
    torch.cuda.set_device(dev)
    backend = os.environ.get("VD_DIST_BACKEND", "nccl")
    dist.init_process_group(backend, init_method="env://")
    red_dev = torch.device("cuda", dev) if backend == "nccl" else torch.device("cpu")
    L = _native.load()
    pts_h, off = W.c4_sets()
    sizes = np.diff(off)
    share = shard.lpt_assign(sizes, world)[rank]
    loc = np.ascontiguousarray(np.concatenate([pts_h[off[i]:off[i + 1]] for i in share]))
    loff = np.concatenate([[0], np.cumsum(sizes[share])]).astype(np.int64)
    n, nsets = int(loff[-1]), len(share)
    pts_d = torch.from_numpy(loc).cuda()
    cap = 9 * n + 1024
    uv_d = torch.empty((cap, 2), dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    st = ctypes.c_int(0)
    tree = ctypes.c_void_p(L.vd_tree_create(3, ctypes.c_void_p(stream.cuda_stream), ctypes.byref(st)))
    eoff = np.zeros(nsets + 1, dtype=np.int64)
    i64p = ctypes.POINTER(ctypes.c_int64)
    tv = np.zeros(9, dtype=np.int64)
    L.vd_autotune_batch(tree, ctypes.c_void_p(pts_d.data_ptr()), loff.ctypes.data_as(i64p), nsets,
                        min(2_000_000, n), tv.ctypes.data_as(i64p))

    def step():
        rc = L.vd_batch_delaunay_device(tree, ctypes.c_void_p(pts_d.data_ptr()), loff.ctypes.data_as(i64p), nsets,
                                        SEED, ctypes.c_void_p(uv_d.data_ptr()), cap, eoff.ctypes.data_as(i64p))
        if rc not in (0, 4):
            raise SystemExit(f"vd_batch_delaunay_device failed: {rc}")

    for _ in range(max(args.warmup, 3)):
        step()
    times = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        dist.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ok = ctypes.c_int(0)
    L.vd_check_delaunay(tree, ctypes.byref(ok), None)
    L.vd_tree_free(tree)
    t = torch.tensor([float(np.mean(times)), float(n), float(ok.value == 0)], dtype=torch.float64, device=red_dev)
    mx = t[:1].clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    tot = t[1:].clone()
    dist.all_reduce(tot, op=dist.ReduceOp.SUM)
    ms, total, bad = float(mx.item()), int(tot[0].item()), int(tot[1].item())
    if rank == 0:
        line = {
            "metric": "Mpts/s batched build, 4,096 3D sets", "value": round(total / (ms / 1e3) / 1e6, 4),
            "unit": "Mpts/s", "n_gpus": world, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "4,096 independent 3D sets, sizes floor(exp(U(ln 32, ln 65536))), uniform [0,1)^3 "
                                   "(splitmix64 seed 0xD1A00004), the sets split across ranks by size (LPT), one "
                                   "batched build per rank per step", "points": total, "sets": len(sizes),
                       "parallelism": f"sets across {world} ranks", "l2": "flushed between steps (256 MB write)"},
            "ranks_failing_validator": bad,
        }
        print(json.dumps(line), flush=True)
    dist.destroy_process_group()


def run_c4(args):
    """4,096 independent 3D sets (log-uniform 32..65,536 points): one batched
    build per step against one build per set, same GPU, same outputs."""
    import torch
    from voronoids_gb300 import _native
    L = _native.load()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    clk = Clocks(0)
    clk.start()
    r = measure_c4(L, 4096, args.steps, max(args.warmup, 3), flush, autotune=True)
    clocks = clk.stop()
    tree, n, nsets, offp, cap = r["tree"], r["points"], r["sets"], r["offsets"], r["cap"]
    # end to end: host points in, host edges out (vd_batch_delaunay)
    pts_pin = torch.from_numpy(r["pts_h"]).pin_memory()
    uv_pin = torch.empty((cap, 2), dtype=torch.int32).pin_memory()
    hp = ctypes.cast(ctypes.c_void_p(pts_pin.data_ptr()), ctypes.POINTER(ctypes.c_double))
    i64p = ctypes.POINTER(ctypes.c_int64)
    eoff = np.zeros(nsets + 1, dtype=np.int64)
    etimes = []
    for _ in range(max(1, args.steps // 2)):
        t0 = time.perf_counter()
        L.vd_batch_delaunay(tree, hp, offp.ctypes.data_as(i64p), nsets, SEED, ctypes.c_void_p(uv_pin.data_ptr()),
                            cap, eoff.ctypes.data_as(i64p))
        etimes.append(time.perf_counter() - t0)
    ems = 1e3 * float(np.mean(etimes))
    L.vd_tree_free(tree)
    line = {
        "metric": "Mpts/s batched build, 4,096 3D sets", "value": r["value"], "unit": "Mpts/s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "4,096 independent 3D sets, sizes floor(exp(U(ln 32, ln 65536))), uniform [0,1)^3 "
                               "(splitmix64 seed 0xD1A00004), one batched build per step", "points": n,
                   "sets": nsets, "l2": "flushed between steps (256 MB write)"},
        "one_set_per_launch": r["one_set_per_launch"],
        "batched_over_one_set_per_launch": r["batched_over_one_set_per_launch"], "autotuned": r["autotuned"],
        "validator_ok": r["validator_ok"], "edges": r["edges"], "clocks": clocks, "gpu_launches": r["gpu_launches"],
        "e2e": {"value": round(n / (ems / 1e3) / 1e6, 4), "unit": "Mpts/s", "h2d_bytes_per_step": int(n * 24),
                "d2h_bytes_per_step": int(eoff[-1] * 8), "ms_per_step": round(ems, 3)},
    }
    print(json.dumps(line), flush=True)


def run_c5(args):
    """Poisson stream of triangulation requests (2D/3D 50/50, log-uniform
    100..200,000 points) through the serving loop at 80% of its measured
    capacity; latency from submission to completion."""
    from voronoids_gb300 import _native
    from voronoids_gb300 import workloads as W
    L = _native.load()
    reqs = W.c5_requests(args.requests)
    mean_pts = float(np.mean([r[1] for r in reqs]))
    budget = 64 << 30
    i64p = ctypes.POINTER(ctypes.c_int64)

    def serve(stream_reqs, arrivals):
        st = ctypes.c_int(0)
        srv = ctypes.c_void_p(L.vd_server_new(budget, args.slots, args.max_batch_points, SEED, ctypes.byref(st)))
        if st.value != 0:
            raise SystemExit(f"vd_server_new failed: {st.value}")
        nreq = len(stream_reqs)
        sub_t = np.zeros(nreq)
        done_t = np.zeros(nreq)
        lag = np.zeros(nreq)
        statuses = np.zeros(nreq, dtype=np.int64)
        id_of = {}
        uv = np.empty(2 * (10 * 200_000 + 64), dtype=np.uint32)
        finished = [0]
        t_start = time.perf_counter()

        def poller():
            ids = np.zeros(4096, dtype=np.int64)
            m = ctypes.c_int64(0)
            ne = ctypes.c_int64(0)
            rs = ctypes.c_int(0)
            while finished[0] < nreq:
                L.vd_server_poll(srv, ids.ctypes.data_as(i64p), 4096, ctypes.byref(m), 5)
                now = time.perf_counter() - t_start
                for rid in ids[: m.value].tolist():
                    k = id_of.get(rid)
                    while k is None:  # submit() has not recorded it yet
                        time.sleep(0.0001)
                        k = id_of.get(rid)
                    done_t[k] = now
                    L.vd_server_result(srv, rid, ctypes.c_void_p(uv.ctypes.data), len(uv) // 2, ctypes.byref(ne),
                                       ctypes.byref(rs))
                    statuses[k] = rs.value
                    finished[0] += 1

        th = threading.Thread(target=poller, daemon=True)
        th.start()
        rid = ctypes.c_int64(0)
        for k, r in enumerate(stream_reqs):
            p = W.c5_points(r)
            if arrivals is not None:
                wait = arrivals[k] - (time.perf_counter() - t_start)
                if wait > 0:
                    time.sleep(wait)
            now = time.perf_counter() - t_start
            lag[k] = now - (arrivals[k] if arrivals is not None else 0.0)
            sub_t[k] = now
            rc = L.vd_server_submit(srv, r[0], p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), r[1],
                                    ctypes.byref(rid))
            if rc != 0:
                raise SystemExit(f"vd_server_submit failed: {rc}")
            id_of[rid.value] = k
        th.join()
        stats = np.zeros(8, dtype=np.int64)
        L.vd_server_stats(srv, stats.ctypes.data_as(i64p))
        L.vd_server_free(srv)
        return sub_t, done_t, lag, statuses, stats

    # capacity: a closed burst of the first requests
    ncap = min(2000, len(reqs))
    sub_t, done_t, _, _, _ = serve(reqs[:ncap], None)
    cap_pts = sum(r[1] for r in reqs[:ncap]) / (done_t.max() - sub_t.min())
    rate = 0.8 * cap_pts / mean_pts  # requests per second
    gaps = np.random.default_rng(SEED).exponential(1.0 / rate, len(reqs))
    arrivals = np.cumsum(gaps) - gaps[0]
    clk = Clocks(0)
    clk.start()
    sub_t, done_t, lag, statuses, stats = serve(reqs, arrivals)
    clocks = clk.stop()
    lat = 1e3 * (done_t - sub_t)
    total = sum(r[1] for r in reqs)
    span = done_t.max() - sub_t.min()
    line = {
        "metric": "served Mpts/s with p50/p99 latency, Poisson request stream", "value": round(total / span / 1e6, 4),
        "unit": "Mpts/s", "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": round(1e3 * span, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{len(reqs)} requests, 2D/3D 50/50, sizes log-uniform 100..200,000 points uniform "
                               f"in the unit square/cube (splitmix64 seed 0xD1A00005), Poisson arrivals at 80% of "
                               f"the measured capacity", "points": int(total), "slots": args.slots,
                   "max_batch_points": args.max_batch_points, "pool_budget_bytes": budget},
        "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 2), "p99": round(float(np.percentile(lat, 99)), 2),
                       "mean": round(float(lat.mean()), 2), "max": round(float(lat.max()), 2)},
        "capacity_mpts_s": round(cap_pts / 1e6, 4), "arrival_rate_req_s": round(rate, 2),
        "submission_lag_ms_p99": round(1e3 * float(np.percentile(lag, 99)), 2),
        "failed_requests": int(np.count_nonzero(statuses)),
        "server": {"batches": int(stats[2]), "peak_bytes_in_flight": int(stats[4]), "isolated": int(stats[6])},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "c3":
        run_c3(args)
        return
    if args.workload == "c4":
        if world > 1:
            run_c4_ranks(args, world, rank, local)
        else:
            run_c4(args)
        return
    if args.workload == "c5":
        run_c5(args)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")

    from voronoids_gb300 import _native
    from voronoids_gb300 import workloads as W
    L = _native.load()
    n = args.n
    pts_h = W.uniform_points(n, 3, W.config_seed(2)) if n != N_POINTS else W.c2_points()
    dev = torch.device("cuda", local)
    pts_d = torch.from_numpy(pts_h).to(dev).contiguous()
    cap = 8 * n + 1024
    uv_d = torch.empty(2 * cap, dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    st = ctypes.c_int(0)
    tree = L.vd_tree_new_device(3, ctypes.c_void_p(pts_d.data_ptr()), n, ctypes.c_void_p(stream.cuda_stream),
                                ctypes.byref(st))
    if not tree or st.value != 0:
        raise SystemExit(f"vd_tree_new_device failed: {st.value}")
    tree = ctypes.c_void_p(tree)
    m = ctypes.c_int64(0)

    def step():
        rc = L.vd_delaunay_device(tree, ctypes.c_void_p(pts_d.data_ptr()), n, SEED,
                                  ctypes.c_void_p(uv_d.data_ptr()), cap, ctypes.byref(m))
        if rc != 0:
            raise SystemExit(f"vd_delaunay_device failed: {rc}")

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    def timed_region(profiling):
        L.vd_set_profiling(tree, 1 if profiling else 0)
        times = []
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        launches0 = L.vd_kernel_launches()
        for _ in range(args.steps):
            flush.fill_(1)  # L2 flush between steps, outside the events
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return times, L.vd_kernel_launches() - launches0

    clk = Clocks(local)
    clk.start()
    times, launches = timed_region(False)
    clocks = clk.stop()
    ms = float(np.mean(times))
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n / (ms / 1e3) / 1e6

    # second timed region with per-kernel events (roofline)
    s0 = _native.VdStats()
    L.vd_get_stats(tree, ctypes.byref(s0))
    ptimes, _ = timed_region(True)
    nk = ctypes.c_int(0)
    L.vd_profile(tree, None, None, 0, ctypes.byref(nk))
    kms = np.zeros(nk.value)
    kcnt = np.zeros(nk.value, dtype=np.int64)
    L.vd_profile(tree, kms.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                 kcnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), nk.value, ctypes.byref(nk))
    names = [L.vd_profile_name(i).decode() for i in range(nk.value)]
    s1 = _native.VdStats()
    L.vd_get_stats(tree, ctypes.byref(s1))
    stats = {k: getattr(s1, k) for k, _ in s1._fields_}
    L.vd_set_profiling(tree, 0)
    round_k = [i for i, nm in enumerate(names) if nm.startswith("k_")]
    dom = max(round_k, key=lambda i: kms[i])
    dname = names[dom]
    # units processed in the profiled region (the stats counters are per build)
    tests = stats["cavity_tests"]
    if dname == "k_cavity":
        algo_bytes = BYTES_PER_TEST_3D * tests * args.steps
    elif dname == "k_check":  # adjacent mode: the commit half (stars of the winners)
        algo_bytes = BYTES_PER_WIN * stats["inserted"] * args.steps
    elif dname == "k_decide":  # adjacent mode: claims and lists of every searched candidate
        algo_bytes = BYTES_PER_CHECK * stats["searched"] * args.steps
    else:
        algo_bytes = None
    peak, peak_kind = measured_peaks()
    roof = None
    if algo_bytes is not None and kcnt[dom] > 0:
        per_launch = algo_bytes / kcnt[dom]
        avg_ms = kms[dom] / kcnt[dom]
        achieved = per_launch / (avg_ms / 1e3) / 1e9
        traffic = profile_traffic(dname)
        roof = {"bound": "hbm", "kernel": dname, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 5), "peak_source": peak_kind,
                "traffic": traffic, "algorithmic_bytes_per_launch": round(per_launch, 1),
                "avg_launch_ms": round(avg_ms, 4), "launches": int(kcnt[dom])}
    kernel_share = {names[i]: round(float(kms[i] / max(kms.sum(), 1e-9)), 4) for i in range(len(names))}

    # end to end through the host-buffer one-shot call
    e2e = None
    if not args.no_e2e:
        pts_pin = torch.from_numpy(pts_h).pin_memory()
        uv_pin = torch.empty(2 * cap, dtype=torch.int32).pin_memory()
        hp = ctypes.cast(ctypes.c_void_p(pts_pin.data_ptr()), ctypes.POINTER(ctypes.c_double))
        for _ in range(2):
            L.vd_delaunay_tree(tree, hp, n, SEED, ctypes.c_void_p(uv_pin.data_ptr()), cap, ctypes.byref(m))
        etimes = []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = L.vd_delaunay_tree(tree, hp, n, SEED, ctypes.c_void_p(uv_pin.data_ptr()), cap, ctypes.byref(m))
            etimes.append(time.perf_counter() - t0)
            if rc != 0:
                raise SystemExit(f"vd_delaunay_tree failed: {rc}")
        ems = 1e3 * float(np.mean(etimes))
        if dist:
            t = torch.tensor([ems], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ems = float(t.item())
        e2e = {"value": round(world * n / (ems / 1e3) / 1e6, 4), "unit": "Mpts/s",
               "h2d_bytes_per_step": int(n * 3 * 8), "d2h_bytes_per_step": int(m.value * 8),
               "ms_per_step": round(ems, 3)}

    # whole build against HBM: algorithmic bytes per inserted 3D point
    # 1820 + 128 ln N (point, killed and created simplex records, outer
    # neighbour rewrites, edge output, relocations)
    bpp = 1820.0 + 128.0 * math.log(n)
    peak_b, _ = measured_peaks()
    build_roof = {"bytes_per_point": round(bpp, 1), "achieved": round(bpp * n / (ms / 1e3) / 1e9, 2),
                  "peak": peak_b, "unit": "GB/s", "frac": round(bpp * n / (ms / 1e3) / 1e9 / peak_b, 5)}
    edges = int(m.value)
    L.vd_tree_free(tree)
    # the other configurations, measured beside the headline on rank 0:
    # C1 (2D 10k), C3 (near-degenerate 262k), a 256-set sample of C4
    subs = {}
    if rank == 0 and world == 1 and not args.no_subs:
        subs["c1"] = measure_c1(L, args.steps, flush)
        subs["c3"] = measure_c3(L, min(args.steps, 5), 2, flush)
        c4 = measure_c4(L, 256, min(args.steps, 5), 2, flush, autotune=False)
        L.vd_tree_free(c4["tree"])
        for k in ("tree", "offsets", "pts_h", "cap"):
            c4.pop(k)
        c4["workload"] = ("256 independent 3D sets, sizes floor(exp(U(ln 32, ln 65536))), uniform [0,1)^3 "
                          "(splitmix64 seed 0xD1A00004, the C4 distribution), default tuning")
        subs["c4_sample"] = c4
        subs["reference_call_pattern"] = measure_reference_pattern(L)
    cpu = cpu_baseline(pts_h) if rank == 0 and world == 1 else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": "Mpts/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "1M points i.i.d. uniform in [0,1)^3 (splitmix64 seed 0xD1A00002), exact 3D "
                                   "Delaunay tetrahedralization with the reference's super simplex, sorted "
                                   "input-index edge list", "points": n,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "flushed between steps (256 MB write)", "edges": edges,
                       "tuning": "3D defaults: adjacent round mode, 2 resolution passes, thinning radius 2, "
                                 "priority levels 64 x1.25 fed at 0.12 x inserted, rounds replayed as CUDA graphs"},
            "clocks": clocks, "gpu_launches": int(launches), "e2e": e2e, "roofline": roof,
            "cpu_baseline": cpu,
            "build_stats": {k: stats[k] for k in ("rounds", "inserted", "max_cavity", "pred_f32", "pred_f64",
                                                  "pred_exact", "walk_steps", "cavity_tests", "searched")},
            "kernel_share": kernel_share,
            "build_roofline": build_roof,
            "ms_per_step_profiled": round(float(np.mean(ptimes)), 3),
        }
        line.update(subs)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
