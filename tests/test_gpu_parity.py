"""GPU: the CUDA build against the oracle and the golden vectors.

Parity bar: the sorted input-index edge list is bit-identical to the oracle's
(exact integer comparison), and the exact validator passes.  At full sizes,
size-independent properties replace the oracle (validator, Euler counts).
"""
import os
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def gpu_edges(vd, pts, seed=0):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t = vd.delaunay(pts, seed=seed)
    return t, t.edges()


def test_max_simplex_id_after_new(vd):
    # tests/test_delaunay_tree.rs:20 and :44 of the reference
    t3 = vd.DelaunayTree(np.random.default_rng(0).random((1000, 3)))
    assert t3.max_simplex_id == 4
    t2 = vd.DelaunayTree([[0.3, 0.1], [1.0, 0.2], [0.1, 1.0], [0.5, 0.5]])
    assert t2.max_simplex_id == 3


@pytest.mark.parametrize("name", ["uniform2d_2000", "uniform3d_2000", "clusters3d_3000"])
def test_golden(vd, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    t, e = gpu_edges(vd, g["points"])
    assert np.array_equal(e, g["edges"])
    assert t.check_delaunay()


def test_c1_2d_10k_bit_identical(vd, oracle):
    p = W.c1_points()
    t, e = gpu_edges(vd, p, seed=W.config_seed(1))
    o = oracle.Triangulation(p, seed=W.config_seed(1))
    assert o.status == 0
    assert np.array_equal(e, o.edges())
    ok, det = t.check_delaunay(details=True)
    assert ok, det


@pytest.mark.parametrize("n", [2, 3, 5, 17, 200, 5000, 50000])
def test_3d_uniform_vs_oracle(vd, oracle, n):
    p = W.uniform_points(n, 3, 1000 + n)
    t, e = gpu_edges(vd, p, seed=n)
    o = oracle.Triangulation(p, seed=n)
    assert np.array_equal(e, o.edges())
    assert t.check_delaunay()
    assert t.num_vertices == n


@pytest.mark.parametrize("n", [2, 3, 10, 1000, 30000])
def test_2d_uniform_vs_oracle(vd, oracle, n):
    p = W.uniform_points(n, 2, 2000 + n)
    t, e = gpu_edges(vd, p, seed=n)
    o = oracle.Triangulation(p, seed=n)
    assert np.array_equal(e, o.edges())
    assert t.check_delaunay()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_insertion_order_does_not_change_result(vd, seed):
    p = W.uniform_points(20000, 3, 77)
    _, e0 = gpu_edges(vd, p, seed=0)
    _, e1 = gpu_edges(vd, p, seed=seed + 100)
    assert np.array_equal(e0, e1)


@pytest.mark.parametrize("dim,side", [(2, 16), (2, 33), (3, 6), (3, 11)])
def test_exact_lattice_vs_oracle(vd, oracle, dim, side):
    """Cospherical / cocircular everywhere: ties go through the perturbation."""
    p = W.lattice_points(side, dim) / side
    p = p[np.random.default_rng(side).permutation(len(p))]
    t, e = gpu_edges(vd, p, seed=side)
    o = oracle.Triangulation(p, seed=side)
    assert np.array_equal(e, o.edges())
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    st = t.stats()
    assert st["pred_exact"] > 0 and st["pred_sos"] >= 0


def test_c3_near_degenerate_small(vd, oracle):
    p = W.c3_points(n=20000, seed=W.config_seed(3) + 1)
    t, e = gpu_edges(vd, p, seed=3)
    o = oracle.Triangulation(p, seed=3)
    assert np.array_equal(e, o.edges())
    st = t.stats()
    assert st["pred_f64"] > 0  # the lattice half defeats the f32 filter
    assert t.check_delaunay()


def test_duplicates_match_oracle(vd, oracle):
    rng = np.random.default_rng(21)
    p = rng.random((3000, 3))
    p = np.vstack([p, p[rng.integers(0, 3000, 200)], p[:5]])
    with pytest.warns(RuntimeWarning):
        t = vd.delaunay(p, seed=5)
    o = oracle.Triangulation(p, seed=5)
    assert np.array_equal(t.edges(), o.edges())
    assert len(t.duplicates()) == o.num_duplicates()
    assert t.check_delaunay()


def test_incremental_calls_equal_one_shot(vd):
    p = W.uniform_points(30000, 3, 5)
    t = vd.DelaunayTree(p)
    t.add_points_to_tree(p[:1000], seed=1)
    t.add_points_to_tree(p[1000:9000], seed=2)
    t.add_points_to_tree(p[9000:], seed=3)
    _, e = gpu_edges(vd, p)
    assert np.array_equal(t.edges(), e)
    assert t.check_delaunay()


def test_insert_point_one_by_one(vd, oracle):
    p = W.uniform_points(60, 2, 9)
    t = vd.DelaunayTree(p)
    for q in p:
        t.insert_point(q)
    assert np.array_equal(t.edges(), oracle.Triangulation(p).edges())


def test_insert_point_one_by_one_3d(vd, oracle):
    """TreeUpdate::new + insert_point (src/delaunay_tree.rs:709-740, :125-211),
    the reference's sequential path (src/lib.rs:108-114), in 3D."""
    p = W.uniform_points(300, 3, 19)
    t = vd.DelaunayTree(p)
    for q in p:
        t.insert_point(q)
    assert t.num_vertices == len(p)
    assert np.array_equal(t.edges(), oracle.Triangulation(p).edges())
    assert t.check_delaunay()
    # a repeated point is skipped and recorded; points outside the super simplex are errors
    with pytest.warns(RuntimeWarning):
        t.insert_point(p[5])
    assert np.array_equal(t.duplicates(), [[300, 5]])
    assert np.array_equal(t.edges(), oracle.Triangulation(p).edges())
    with pytest.raises(vd.VDError) as ei:
        t.insert_point(np.array([50.0, 50.0, 50.0]))
    assert ei.value.status == 6
    # then the rest of a larger set through add_points_to_tree, as the reference does past 1e5 points
    q = W.uniform_points(5000, 3, 20)
    t2 = vd.DelaunayTree(q)
    for x in q[:200]:
        t2.insert_point(x)
    t2.add_points_to_tree(q[200:], seed=4)
    assert np.array_equal(t2.edges(), oracle.Triangulation(q).edges())


def test_validator_on_gpu_simplices(vd, oracle):
    p = W.uniform_points(4000, 3, 31)
    t, _ = gpu_edges(vd, p)
    v, nb = t.simplices()
    sv, _ = oracle.super_vertices(p)
    verts = np.vstack([sv, p])
    ids = np.where(v < 0, -v - 1, v + 4)
    ids[:, 3] = np.where(v[:, 3] == -1, ids[:, 3], ids[:, 3])
    res = oracle.validate(3, verts, ids.astype(np.int32), nb, expect_vertices=len(verts))
    assert res["non_positive"] == 0 and res["asymmetric"] == 0
    assert res["not_delaunay"] == 0 and res["not_perturbed_delaunay"] == 0
    assert res["hull_facets"] == 4 and res["missing_vertices"] == 0


def test_errors_are_statuses(vd):
    with pytest.raises(vd.VDError) as ei:
        vd.DelaunayTree(np.ones((5, 3)))
    assert ei.value.status == 12  # degenerate super simplex
    t = vd.DelaunayTree(np.random.default_rng(0).random((100, 3)))
    with pytest.raises(vd.VDError) as ei:
        t.add_points_to_tree(np.array([[100.0, 100.0, 100.0]]))
    assert ei.value.status == 6  # outside the super simplex
    t2 = vd.DelaunayTree(np.random.default_rng(0).random((100, 2)))
    with pytest.raises(vd.VDError) as ei:
        t2.add_points_to_tree(np.array([[0.5, np.nan]]))
    assert ei.value.status == 5


@pytest.mark.slow
def test_c2_full_size_properties(vd):
    """1M uniform 3D points: exact validator + counting identities."""
    p = W.c2_points()
    t, e = gpu_edges(vd, p, seed=W.config_seed(2))
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    st = t.stats()
    n = len(p)
    assert st["inserted"] == n and st["duplicates"] == 0
    # every vertex has an edge; sorted, unique, u < v
    assert len(np.unique(e)) == n
    assert np.all(e[:, 0] < e[:, 1])
    k = e[:, 0] * n + e[:, 1]
    assert np.all(np.diff(k) > 0)
    assert 7.4 < len(e) / n < 7.9
    # Euler: for a triangulated ball V - E + F - T = 1 over all simplices
    assert st["live_simplices"] == 1 + st["created"] - st["killed"]


@pytest.mark.parametrize("dim", [2, 3])
def test_reused_tree_matches_fresh(vd, oracle, dim):
    # a tree reset for new points must show nothing of its earlier build
    a = W.uniform_points(30000, dim, 61)
    b = W.uniform_points(12000, dim, 62)
    t = vd.DelaunayTree(a)
    t.add_points_to_tree(a, seed=1)
    for pts, seed in ((b, 2), (a, 3), (b, 4)):
        t.reset(pts)
        t.add_points_to_tree(pts, seed=seed)
        ok, det = t.check_delaunay(details=True)
        assert ok, det
        assert np.array_equal(t.edges(), oracle.Triangulation(pts, seed=seed).edges())
    t.close()
