"""GPU: inputs that stress the predicate tiers, checked against the oracle.

* Rescaling every coordinate by a power of two is exact in floating point,
  and so is the reference's super simplex of the rescaled points (its
  bounding sphere and vertex formulas, src/geometry.rs:99-142 and
  src/delaunay_tree.rs:392-406, :547-558, scale with it).  The triangulation
  is therefore the same, and the edge list must not change.  Factors 2^+-100
  push the squared terms of the in-sphere test out of FP32 range, so the
  filters must hand those tests on instead of deciding them.
* A cloud of width 1e-3 translated to 1000: the FP32 filter sees coordinates
  whose high halves are nearly equal, and the low halves carry the geometry.
* Concentric integer spheres (3D) and circles (2D): every point of a shell is
  exactly cospherical (cocircular) with the others of its shell, so nearly
  every in-sphere test is a tie, and the symbolic perturbation by vertex id
  (the reference's strict test for the newest point, src/geometry.rs:91-97)
  decides.
"""
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def gpu_build(vd, pts, seed):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        return vd.delaunay(pts, seed=seed)


def shells3(radii):
    """The origin and the integer points on spheres of the given radii."""
    out = [np.zeros((1, 3))]
    for R in radii:
        r = np.arange(-R, R + 1)
        a, b, c = np.meshgrid(r, r, r, indexing="ij")
        m = a * a + b * b + c * c == R * R
        out.append(np.stack([a[m], b[m], c[m]], 1))
    return np.concatenate(out).astype(np.float64)


def shells2(squares):
    """The origin and the integer points on circles of the given squared radii."""
    out = [np.zeros((1, 2))]
    for R2 in squares:
        R = int(np.sqrt(R2)) + 1
        r = np.arange(-R, R + 1)
        a, b = np.meshgrid(r, r, indexing="ij")
        m = a * a + b * b == R2
        out.append(np.stack([a[m], b[m]], 1))
    return np.concatenate(out).astype(np.float64)


@pytest.mark.parametrize("dim", [2, 3])
def test_power_of_two_scaling_keeps_the_edges(vd, oracle, dim):
    p = W.uniform_points(4000, dim, 770 + dim)
    want = oracle.Triangulation(p, seed=1).edges()
    for k in (0, -100, -30, 30, 100):
        t = gpu_build(vd, p * 2.0 ** k, seed=1)
        assert np.array_equal(t.edges(), want), k
        assert t.check_delaunay(), k
        t.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_far_translated_cloud_matches_oracle(vd, oracle, dim):
    p = W.uniform_points(4000, dim, 780 + dim) * 1e-3 + 1000.0
    t = gpu_build(vd, p, seed=2)
    assert np.array_equal(t.edges(), oracle.Triangulation(p, seed=2).edges())
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    t.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_concentric_shells_match_oracle(vd, oracle, dim):
    p = shells3((21, 45, 65)) if dim == 3 else shells2((5525, 27625, 71825, 1221025))
    for seed in (3, 4):
        t = gpu_build(vd, p, seed=seed)
        assert np.array_equal(t.edges(), oracle.Triangulation(p, seed=seed).edges()), seed
        ok, det = t.check_delaunay(details=True)
        assert ok, det
        st = t.stats()
        assert st["pred_exact"] > 0  # exact ties: no filter can decide them
        assert st["pred_sos"] > 0  # and the perturbation decided them
        t.close()
