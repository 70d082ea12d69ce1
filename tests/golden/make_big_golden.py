"""Edge-list digests of the full-size workloads, made by the CPU oracle.

Test infrastructure only.  The sequential exact oracle (``oracle/``) builds
the Delaunay triangulation of each workload below; the sorted (u, v) edge
list, an (m, 2) little-endian int64 array, is reduced to its row count and a
SHA-256 of its bytes.  ``big_edges.json`` keeps those two numbers per
workload, so the GPU tests can compare a full-size build bit for bit without
the oracle's minutes of CPU time on the test machine.

    python tests/golden/make_big_golden.py            # all workloads
    python tests/golden/make_big_golden.py c3         # one of them

Workloads (inputs from ``voronoids_gb300/workloads.py``):
  c1   10,000 uniform 2D points, seed 0xD1A00001
  c2   1,000,000 uniform 3D points, seed 0xD1A00002
  c3   262,144 near-degenerate 3D points (jittered lattice + tight clusters)
  u2   1,000,000 uniform 2D points, seed 0xD1A00006
  l3   the exact 64^3 lattice scaled by 1/64 (262,144 points; the scaling is exact in
       binary, so every cell stays cospherical) in a seeded random order: every tie
       goes through the symbolic perturbation
  l2   the exact 512^2 lattice scaled by 1/512 (262,144 points, every cell cocircular),
       likewise
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from voronoids_gb300 import workloads as W  # noqa: E402

OUT = os.path.join(HERE, "big_edges.json")


def workloads():
    return {
        "c1": lambda: W.c1_points(),
        "c2": lambda: W.c2_points(),
        "c3": lambda: W.c3_points(),
        "u2": lambda: W.uniform_points(1_000_000, 2, W.config_seed(6)),
        "l3": lambda: lattice(64, 3),
        "l2": lambda: lattice(512, 2),
    }


def lattice(side, dim):
    """All sites of the side^dim integer lattice scaled by 1/side (side a power of two,
    so the scaling is exact), in a seeded random order."""
    assert side & (side - 1) == 0
    g = W.lattice_points(side, dim) / side
    order = np.argsort(W.splitmix64(W.config_seed(7) + dim, len(g)), kind="stable")
    return np.ascontiguousarray(g[order])


def digest(edges):
    """(rows, sha256 hex) of a sorted (m, 2) edge array as little-endian int64."""
    e = np.ascontiguousarray(edges, dtype="<i8")
    return int(e.shape[0]), hashlib.sha256(e.tobytes()).hexdigest()


def main(names):
    table = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            table = json.load(f)
    for name in names:
        p = workloads()[name]()
        t0 = time.time()
        tri = O.Triangulation(p, seed=1)
        if tri.status != 0:
            raise SystemExit(f"{name}: oracle status {tri.status}")
        rows, sha = digest(tri.edges())
        table[name] = {"points": int(p.shape[0]), "dim": int(p.shape[1]), "edges": rows, "sha256": sha,
                       "duplicates": tri.num_duplicates()}
        print(f"{name}: {p.shape[0]} points, {rows} edges, {time.time() - t0:.1f} s", flush=True)
    with open(OUT, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main(sys.argv[1:] or list(workloads()))
