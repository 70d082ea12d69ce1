"""How the reference's floating-point conflict test departs from the exact one.

Test infrastructure only (a diagnostic; it reads nothing outside this
repository).  For each workload the reference's own sequential insertion
path is run with its inexact predicate (``FloatTriangulation``: circumsphere
centre and radius in f64, then the strict ``dist^2 < r^2`` of
src/geometry.rs:91-97, the super simplex's sphere and the radius-0 ghosts of
src/delaunay_tree.rs:389-510) and compared with the exact oracle:

  float-only / exact-only  edges present in one edge list and not the other
  empty                    points whose located set was empty (the reference
                           panics there, src/delaunay_tree.rs:53)
  bad links                neighbour links that do not close onto a facet
  validator                the exact validator on the float result:
                           asymmetric links and non-Delaunay facets

    python oracle/float_diagnostic.py [c1] [c2_100k] [c3]
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from voronoids_gb300 import workloads as W  # noqa: E402

CASES = {
    "c1": lambda: W.c1_points(),
    "c2_100k": lambda: W.c2_points()[:100_000],
    "c3": lambda: W.c3_points(),
}


def compare(points):
    """Diagnostic record of one point set."""
    t0 = time.time()
    f = O.FloatTriangulation(points)
    seconds = time.time() - t0
    fe, ee = f.edges(), O.Triangulation(points).edges()
    key = lambda e: e[:, 0] * (1 << 32) + e[:, 1]  # noqa: E731
    verts, simp, nbr, bad = f.export()
    val = O.validate(points.shape[1], verts, simp, nbr, expect_vertices=len(verts))
    return {
        "points": int(points.shape[0]),
        "float_seconds": round(seconds, 2),
        "edges_exact": int(len(ee)),
        "float_only": int(np.setdiff1d(key(fe), key(ee)).size),
        "exact_only": int(np.setdiff1d(key(ee), key(fe)).size),
        "empty": f.stats["empty_located"],
        "malformed_new": f.stats["malformed_new"],
        "max_killed": f.stats["max_killed"],
        "bad_links": bad,
        "asymmetric": val["asymmetric"],
        "non_positive": val["non_positive"],
        "not_delaunay": val["not_delaunay"],
        "missing_vertices": val["missing_vertices"],
    }


if __name__ == "__main__":
    for name in sys.argv[1:] or list(CASES):
        print(name, compare(CASES[name]()), flush=True)
