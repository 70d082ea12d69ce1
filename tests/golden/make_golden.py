"""Generates the committed golden fixtures (run in a container with scipy).

The reference crate cannot be built here (no Rust toolchain, crates not
vendored), so its own test vectors are restated from its test sources and
the Delaunay graph is pinned by an independent implementation: Qhull
(scipy.spatial.Delaunay) run on the input points together with the
reference's super-simplex vertices.  For points in general position the
Delaunay triangulation of that set is unique, so its edges among input
points are exactly what the reference computes.

Outputs (npz): points, super vertices, and the sorted edge list.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from voronoids_gb300 import workloads as W  # noqa: E402


def qhull_edges(points):
    from scipy.spatial import Delaunay
    dim = points.shape[1]
    sv, _ = O.super_vertices(points)
    allp = np.vstack([sv[:, :dim], points])
    tri = Delaunay(allp)
    assert len(tri.coplanar) == 0
    ns = dim + 1
    e = set()
    for s in tri.simplices:
        for i in range(ns):
            for j in range(i + 1, ns):
                a, b = int(s[i]), int(s[j])
                if a >= ns and b >= ns:
                    a, b = a - ns, b - ns
                    e.add((min(a, b), max(a, b)))
    return np.array(sorted(e), dtype=np.int64), sv


CASES = {
    "uniform2d_2000": lambda: W.uniform_points(2000, 2, W.config_seed(1) + 100),
    "uniform3d_2000": lambda: W.uniform_points(2000, 3, W.config_seed(2) + 100),
    "clusters3d_3000": lambda: W.c3_points(n=3000, seed=W.config_seed(3) + 100)[1500:],
}


def main():
    for name, gen in CASES.items():
        p = gen()
        e, sv = qhull_edges(p)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), points=p, super_vertices=sv, edges=e)
        print(name, p.shape, len(e))


if __name__ == "__main__":
    main()
