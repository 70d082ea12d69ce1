"""GPU: the adjacent round mode (touching cavities win together after an
exact shared-facet test, stars stitched after the pass) builds the same
triangulation: bit-identical edges against the oracle and the validator."""
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def build(vd, p, seed=0, passes=None, thin=None):
    t = vd.DelaunayTree(p)
    t.set_adjacent(True)
    if passes:
        t.set_tuning(passes, thin)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t.add_points_to_tree(p, seed=seed)
    return t


@pytest.mark.parametrize("dim,n", [(3, 200), (3, 5000), (3, 60000), (2, 3000), (2, 40000)])
def test_adjacent_matches_oracle(vd, oracle, dim, n):
    p = W.uniform_points(n, dim, 3100 + n)
    t = build(vd, p, seed=n)
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    assert np.array_equal(t.edges(), oracle.Triangulation(p, seed=n).edges())


@pytest.mark.parametrize("passes,thin", [(1, 1), (3, 1), (2, 2)])
def test_adjacent_tunings(vd, oracle, passes, thin):
    p = W.uniform_points(20000, 3, 77)
    t = build(vd, p, seed=5, passes=passes, thin=thin)
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    assert np.array_equal(t.edges(), oracle.Triangulation(p, seed=5).edges())


def test_adjacent_degenerate_inputs(vd, oracle):
    lat = W.lattice_points(9, 3)
    t = build(vd, lat, seed=2)
    assert t.check_delaunay()
    assert np.array_equal(t.edges(), oracle.Triangulation(lat, seed=2).edges())
    c3 = W.c3_points(n=20000)
    t = build(vd, c3, seed=3)
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    assert np.array_equal(t.edges(), oracle.Triangulation(c3, seed=3).edges())
    d = np.random.default_rng(4).random((3000, 3))
    d[100:200] = d[:100]  # duplicates
    t = build(vd, d, seed=4)
    assert t.check_delaunay()
    assert np.array_equal(t.edges(), oracle.Triangulation(d, seed=4).edges())


def test_adjacent_incremental_and_batch(vd, oracle):
    p = W.uniform_points(30000, 3, 91)
    t = vd.DelaunayTree(p)
    t.set_adjacent(True)
    for a, b in ((0, 1000), (1000, 11000), (11000, 30000)):
        t.add_points_to_tree(p[a:b], seed=a)
    assert t.check_delaunay()
    sizes = W.c4_sizes(30, seed=W.config_seed(4) + 3)
    sets = [W.uniform_points(int(n), 3, 700 + i) for i, n in enumerate(sizes)]
    bt = vd.DelaunayTree.create(3)
    bt.set_adjacent(True)
    got = vd.delaunay_batch(sets, seed=6, tree=bt)
    ok, det = bt.check_delaunay(details=True)
    assert ok, det
    for s, e in zip(sets, got):
        assert np.array_equal(e, oracle.Triangulation(s, seed=6).edges())
