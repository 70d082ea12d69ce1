"""GPU: point location queries (``locate``) on a finished tree.

Each returned list must be exactly the conflict region: every listed
simplex strictly contains the query in its circumsphere (exact, the query
being the newest vertex) and no face neighbour of the list does (the
conflict region is connected, so this pins the whole set).
"""
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def check_region(oracle, dim, p, sv, verts, nbrs, q, ids):
    def coords(v):
        return sv[-1 - v][:dim] if v < 0 else p[v]

    ns = dim + 1

    def key(v):
        return -1 - v if v < 0 else ns + v

    def conflict(s):
        vs = verts[s][:ns]
        c = np.array([coords(v) for v in vs])
        k = np.array([key(v) for v in vs] + [2 ** 31 - 1], dtype=np.int32)
        return oracle.insphere_sos(c, q, k) > 0

    region = set(int(x) for x in ids)
    assert len(region) == len(ids)
    assert list(ids) == sorted(ids)
    for s in region:
        assert conflict(s)
        for nb in nbrs[s][:ns]:
            if nb >= 0 and nb not in region:
                assert not conflict(nb)


@pytest.mark.parametrize("dim", [2, 3])
def test_locate_is_exact_conflict_region(vd, oracle, dim):
    p = W.uniform_points(3000, dim, 70 + dim)
    t = vd.delaunay(p)
    verts, nbrs = t.simplices()
    sv, _ = oracle.super_vertices(p)
    q = W.uniform_points(60, dim, 80 + dim) * 1.2 - 0.1  # some queries outside the points' hull
    lists = t.locate(q)
    assert len(lists) == len(q)
    for qi, ids in zip(q, lists):
        assert len(ids) >= 1
        check_region(oracle, dim, p, sv, verts, nbrs, qi, ids)
    # one query through the single-point entry gives the same list
    assert np.array_equal(t.locate(q[7]), lists[7])


def test_locate_on_a_vertex_and_lattice(vd, oracle):
    lat = W.lattice_points(5, 3)  # cospherical ties everywhere
    t = vd.delaunay(lat)
    verts, nbrs = t.simplices()
    sv, _ = oracle.super_vertices(lat)
    q = np.vstack([lat[17], (lat[3] + lat[4]) / 2, [0.37, 0.41, 0.29]])
    lists = t.locate(q)
    for qi, ids in zip(q, lists):
        check_region(oracle, 3, lat, sv, verts, nbrs, qi, ids)
    assert len(lists[0]) == 0  # an existing vertex conflicts with nothing (strict test)
