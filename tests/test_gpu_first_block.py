"""GPU: the first points of a fresh call inserted by one block (vd_set_first_block).

The block inserts the first whole priority levels one point at a time, the
triangulation in shared memory, and the rounds go on from there.  The
triangulation is unique, so the edge list must equal the oracle's whether the
block runs or not, for every share of the input it takes: all of it (small
inputs), a part, or none.  Equal points must be resolved as the rounds do: of
equal points the one with the lowest insertion priority stays, whichever
comes first in the input (reference behaviour on duplicates: a panic,
src/delaunay_tree.rs:53; here they are skipped and reported).
"""
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def build(vd, pts, seed, first_block=None):
    t = vd.DelaunayTree(pts)
    if first_block is not None:
        t.set_first_block(first_block)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t.add_points_to_tree(pts, seed=seed)
    return t


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("n", [5, 60, 300, 5000])
def test_first_block_gives_the_oracle_edges(vd, oracle, dim, n):
    p = W.uniform_points(n, dim, 900 + n + dim)
    want = oracle.Triangulation(p, seed=7).edges()
    rounds = {}
    for fb in (0, None, 1 << 20):
        t = build(vd, p, 7, fb)
        assert np.array_equal(t.edges(), want), fb
        ok, det = t.check_delaunay(details=True)
        assert ok, (fb, det)
        st = t.stats()
        # the block's created / removed counts agree with the slots it left
        assert st["inserted"] == n and st["live_simplices"] == len(t.simplices()[0])
        rounds[fb] = st["rounds"]
        t.close()
    if n >= 300:
        assert rounds[None] < rounds[0]  # the block took the rounds of the first points


@pytest.mark.parametrize("dim", [2, 3])
def test_first_block_duplicates_keep_the_lowest_priority(vd, oracle, dim):
    rng = np.random.default_rng(40 + dim)
    p = rng.random((300, dim))
    # equal points on both sides of every order: later copies of earlier
    # points and earlier copies of later ones
    p = np.vstack([p[150:], p, p[:150]])
    for seed in (1, 2):
        t = build(vd, p, seed)
        o = oracle.Triangulation(p, seed=seed)
        assert np.array_equal(t.edges(), o.edges()), seed
        assert len(t.duplicates()) == o.num_duplicates() == 300
        assert t.check_delaunay()
        t.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_first_block_on_exact_lattices(vd, oracle, dim):
    side = 6 if dim == 3 else 15
    p = W.lattice_points(side, dim)
    for seed in (3, 4):
        t = build(vd, p, seed)
        assert np.array_equal(t.edges(), oracle.Triangulation(p, seed=seed).edges()), seed
        assert t.check_delaunay()
        t.close()


def test_first_block_argument(vd):
    t = vd.DelaunayTree(W.uniform_points(100, 3, 1))
    with pytest.raises(vd.VDError):
        t.set_first_block(-1)
    t.close()
