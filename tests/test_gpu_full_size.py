"""GPU: the full-size workloads, pinned bit for bit to the oracle.

``tests/golden/big_edges.json`` holds, per workload, the row count and the
SHA-256 of the sorted (u, v) int64 edge list that the sequential exact oracle
builds (``tests/golden/make_big_golden.py``; minutes of CPU time, so the
digests are committed instead of recomputed here).  The GPU build of the same
points must give the same rows and digest, i.e. the identical edge list, and
the oracle's independent CPU validator (big-integer predicates) must accept
the simplices the GPU exports.

Reference semantics: ``voronoids.delaunay`` (src/lib.rs:104-125) and
``add_points_to_tree`` (src/delaunay_tree.rs:336-386); ``check_delaunay``
(:512-541) for the validator.
"""
import importlib.util
import json
import os
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _maker():
    spec = importlib.util.spec_from_file_location("make_big_golden", os.path.join(GOLDEN, "make_big_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


MAKER = _maker()
with open(os.path.join(GOLDEN, "big_edges.json")) as _f:
    DIGESTS = json.load(_f)


def build(vd, name, seed):
    p = MAKER.workloads()[name]()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t = vd.delaunay(p, seed=seed)
    return p, t


@pytest.mark.parametrize("name", ["c1", "c2", "c3", "u2", "l3", "l2"])
def test_edge_list_digest_matches_oracle(vd, name):
    g = DIGESTS[name]
    p, t = build(vd, name, W.config_seed(2))
    assert p.shape == (g["points"], g["dim"])
    rows, sha = MAKER.digest(t.edges())
    assert rows == g["edges"]
    assert sha == g["sha256"]
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    assert len(t.duplicates()) == g["duplicates"]
    t.close()


@pytest.mark.parametrize("name", ["c2", "c3"])
def test_cpu_validator_accepts_gpu_simplices(vd, oracle, name):
    p, t = build(vd, name, 12345)
    v, nb = t.simplices()
    t.close()
    sv, _ = oracle.super_vertices(p)
    verts = np.vstack([sv, p])
    ids = np.where(v < 0, -v - 1, v + 4).astype(np.int32)
    res = oracle.validate(3, verts, ids, nb, expect_vertices=len(verts))
    assert res["non_positive"] == 0 and res["asymmetric"] == 0, res
    assert res["not_delaunay"] == 0 and res["not_perturbed_delaunay"] == 0, res
    assert res["hull_facets"] == 4 and res["missing_vertices"] == 0, res
    # every interior facet is shared by two simplices, the hull's 4 by one
    assert 2 * res["facets"] + res["hull_facets"] == 4 * len(ids)
