"""Where the time of a build goes, round by round (diagnostic, needs a GPU).

The reference prints the time of each stage of ``add_points_to_tree`` with
``println!`` (src/delaunay_tree.rs:337-368).  This module gives the GPU
build's counterpart:

* ``prefixes``: builds of the first n points of a workload for growing n,
  each timed on its stream with CUDA events (points already on the device,
  L2 flushed before every timed build, rounds replayed as CUDA graphs), with
  the round count and, from a second build with per-kernel events, the
  average time of one launch of every kernel.  The difference between two
  prefixes is what the later points cost.
* ``rounds``: one traced build (kernel by kernel, one synchronisation per
  round), summed by the number of active points at the start of a round.

    python -m voronoids_gb300.round_profile [--dim 3] [--n 1000000] [--first-block N]

``--first-block`` sets how many first points one block inserts before the
rounds (``vd_set_first_block``; 0: none, default: the library's).
"""
import argparse
import ctypes
import json

import numpy as np

from . import _native
from . import workloads as W


def _tree_on_device(L, torch, pts, first_block=None):
    n, dim = pts.shape
    dev = torch.from_numpy(np.ascontiguousarray(pts)).cuda().contiguous()
    stream = torch.cuda.current_stream()
    st = ctypes.c_int(0)
    h = L.vd_tree_new_device(dim, ctypes.c_void_p(dev.data_ptr()), n, ctypes.c_void_p(stream.cuda_stream),
                             ctypes.byref(st))
    if not h or st.value != 0:
        raise RuntimeError(f"vd_tree_new_device failed: {st.value}")
    h = ctypes.c_void_p(h)
    if first_block is not None and L.vd_set_first_block(h, int(first_block)) != 0:
        raise RuntimeError("vd_set_first_block failed")
    return h, dev, stream


def _profile(L, tree):
    nk = ctypes.c_int(0)
    L.vd_profile(tree, None, None, 0, ctypes.byref(nk))
    ms = np.zeros(nk.value)
    cnt = np.zeros(nk.value, dtype=np.int64)
    L.vd_profile(tree, ms.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                 cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), nk.value, ctypes.byref(nk))
    return {L.vd_profile_name(i).decode(): (float(ms[i]), int(cnt[i])) for i in range(nk.value) if cnt[i]}


def prefixes(pts, sizes, seed=0x5EED, reps=5, first_block=None):
    """One record per prefix size: build time (ms), rounds, microseconds per
    round and per kernel launch."""
    import torch
    L = _native.load()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out = []
    for n in sizes:
        tree, dev, stream = _tree_on_device(L, torch, pts[:n], first_block)
        cap = 8 * n + 1024
        uv = torch.empty(2 * cap, dtype=torch.int32, device="cuda")
        m = ctypes.c_int64(0)

        def build():
            rc = L.vd_delaunay_device(tree, ctypes.c_void_p(dev.data_ptr()), n, seed, ctypes.c_void_p(uv.data_ptr()),
                                      cap, ctypes.byref(m))
            if rc != 0:
                raise RuntimeError(f"vd_delaunay_device failed: {rc}")

        for _ in range(3):
            build()
        times = []
        for _ in range(reps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            build()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        s = _native.VdStats()
        L.vd_get_stats(tree, ctypes.byref(s))
        L.vd_set_profiling(tree, 1)
        build()
        torch.cuda.synchronize()
        prof = _profile(L, tree)
        L.vd_set_profiling(tree, 0)
        L.vd_tree_free(tree)
        ms = float(np.median(times))
        out.append({"n": n, "ms": round(ms, 3), "rounds": s.rounds, "us_per_round": round(1e3 * ms / max(s.rounds, 1), 1),
                    "us_per_launch": {k: round(1e3 * v[0] / v[1], 1) for k, v in prof.items()}})
    return out


def rounds(pts, seed=0x5EED, buckets=(0, 1000, 10000, 50000), first_block=None):
    """A traced build summed by active points at the start of a round:
    rounds, GPU milliseconds (per-kernel events, no graphs), points inserted."""
    from .tree import DelaunayTree
    warm = DelaunayTree(pts)
    warm.add_points_to_tree(pts, seed=seed)
    warm.close()
    t = DelaunayTree(pts)
    if first_block is not None:
        t.set_first_block(first_block)
    t.set_profiling(True)
    t.set_trace(True)
    t.add_points_to_tree(pts, seed=seed)
    tr = t.trace()
    t.close()
    act, ins, us = tr[:, 1], tr[:, 4], tr[:, 6]
    dins = np.diff(np.r_[0, ins])
    edges = list(buckets) + [np.iinfo(np.int64).max]
    out = []
    for lo, hi in zip(edges[:-1], edges[1:]):
        sel = (act >= lo) & (act < hi)
        out.append({"active_from": int(lo), "rounds": int(sel.sum()), "ms": round(float(us[sel].sum()) / 1e3, 2),
                    "inserted": int(dins[sel].sum())})
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--dim", type=int, default=3, choices=(2, 3))
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--first-block", type=int, default=None)
    a = ap.parse_args()
    pts = W.uniform_points(a.n, a.dim, W.config_seed(2 if a.dim == 3 else 1))
    sizes = [s for s in (300, 3000, 30000, 300000) if s < a.n] + [a.n]
    for rec in prefixes(pts, sizes, first_block=a.first_block):
        print(json.dumps({"prefix": rec}), flush=True)
    for rec in rounds(pts, first_block=a.first_block):
        print(json.dumps({"rounds_by_active": rec}), flush=True)


if __name__ == "__main__":
    main()
