"""GPU: rounds run in one cooperative launch (small-round kernel) build the
same triangulation as rounds launched kernel by kernel."""
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def build(vd, p, small, seed=0, adjacent=True):
    t = vd.DelaunayTree(p)
    t.set_small_rounds(small)
    t.set_adjacent(adjacent)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t.add_points_to_tree(p, seed=seed)
    return t


@pytest.mark.parametrize("dim,n", [(3, 30000), (2, 20000)])
@pytest.mark.parametrize("small", [0, 2000, 1 << 30])
@pytest.mark.parametrize("adjacent", [True, False])
def test_small_rounds_same_triangulation(vd, oracle, dim, n, small, adjacent):
    p = W.uniform_points(n, dim, 8800 + n)
    t = build(vd, p, small, seed=3, adjacent=adjacent)
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    assert np.array_equal(t.edges(), oracle.Triangulation(p, seed=3).edges())


def test_small_rounds_degenerate_and_batch(vd, oracle):
    lat = W.lattice_points(8, 3)
    t = build(vd, lat, 1 << 30, seed=1)
    assert t.check_delaunay()
    assert np.array_equal(t.edges(), oracle.Triangulation(lat, seed=1).edges())
    sets = [W.uniform_points(int(k), 3, 40 + i) for i, k in enumerate([50, 3000, 700, 9000])]
    bt = vd.DelaunayTree.create(3)
    bt.set_small_rounds(1 << 30)
    got = vd.delaunay_batch(sets, seed=2, tree=bt)
    assert bt.check_delaunay()
    for s, e in zip(sets, got):
        assert np.array_equal(e, oracle.Triangulation(s, seed=2).edges())
