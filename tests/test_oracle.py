"""CPU: the oracle against the reference's own known answers and against
independent golden vectors (Qhull on the same point set plus the
reference's super vertices, tests/golden/make_golden.py)."""
import math
import os

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_circumsphere_known_answer(oracle):
    # tests/test_geometry.rs:4-15 of the reference (bit-exact assertion)
    c, r = oracle.circumsphere_float([[1.0, 0.0, 0.0], [0.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    assert list(c) == [0.5, 0.5, 0.5]
    assert r == 0.8660254037844386


def _py_bounding_sphere(pts):
    """Line-by-line Python restatement of src/geometry.rs:99-142 (Python floats
    round like Rust's f64; no fused operations)."""
    dim = len(pts[0])
    lo = [min(p[i] for p in pts) for i in range(dim)]
    hi = [max(p[i] for p in pts) for i in range(dim)]
    c = [(hi[i] + lo[i]) / 2.0 for i in range(dim)]
    ud = math.sqrt(sum((hi[i] - c[i]) * (hi[i] - c[i]) for i in range(dim)))
    ld = math.sqrt(sum((lo[i] - c[i]) * (lo[i] - c[i]) for i in range(dim)))
    r = ud if ud > ld else ld
    for p in pts:
        d = 0.0
        for i in range(dim):
            d += (c[i] - p[i]) * (c[i] - p[i])
        if not d < r * r:
            r = r * 1.5
    return c, r


def test_super_triangle_of_reference_literal(oracle):
    # tests/test_delaunay_tree.rs:42 sizes the 2D tree from these four points
    pts = [[0.3, 0.1], [1.0, 0.2], [0.1, 1.0], [0.5, 0.5]]
    c, r = _py_bounding_sphere(pts)
    R = r * 10.0
    want = [[c[0] + R, c[1]],
            [c[0] + R * math.cos(2.0 * math.pi / 3.0), c[1] + R * math.sin(2.0 * math.pi / 3.0)],
            [c[0] + R * math.cos(4.0 * math.pi / 3.0), c[1] + R * math.sin(4.0 * math.pi / 3.0)]]
    sv, R2 = oracle.super_vertices(np.array(pts))
    assert R2 == R
    assert sv[:, :2].tolist() == want


def test_super_tetrahedron_matches_python_restatement(oracle):
    rng = np.random.default_rng(3)
    pts = rng.random((500, 3)) * 2 - 1
    c, r = _py_bounding_sphere(pts.tolist())
    R = r * 10.0
    a1, a2 = 2.0 * math.pi / 3.0, 4.0 * math.pi / 3.0
    want = [[c[0], c[1], c[2] + R], [c[0] + R, c[1], c[2] - R],
            [c[0] + R * math.cos(a1), c[1] + R * math.sin(a1), c[2] - R],
            [c[0] + R * math.cos(a2), c[1] + R * math.sin(a2), c[2] - R]]
    sv, R2 = oracle.super_vertices(pts)
    assert R2 == R and sv.tolist() == want


def test_bounding_sphere_grows_on_corner_point(oracle):
    # a point exactly on the bounding-box corner is not strictly inside: x1.5
    pts = np.array([[0.0, 0.0], [1.0, 1.0]])
    c, r = oracle.bounding_sphere(pts)
    pc, pr = _py_bounding_sphere(pts.tolist())
    assert list(c) == pc and r == pr and r >= math.sqrt(0.5)


@pytest.mark.parametrize("name", ["uniform2d_2000", "uniform3d_2000", "clusters3d_3000"])
def test_oracle_matches_golden(oracle, name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    t = oracle.Triangulation(g["points"], seed=1)
    assert t.status == 0
    sv, _ = oracle.super_vertices(g["points"])
    assert np.array_equal(sv, g["super_vertices"])
    assert np.array_equal(t.edges(), g["edges"])


@pytest.mark.parametrize("dim,n", [(2, 3000), (3, 3000)])
def test_oracle_output_is_delaunay(oracle, dim, n):
    p = np.random.default_rng(dim).random((n, dim))
    t = oracle.Triangulation(p)
    v, nb = t.simplices()
    res = oracle.validate(dim, t.vertices(), v, nb, expect_vertices=n + dim + 1)
    assert res["non_positive"] == 0 and res["asymmetric"] == 0
    assert res["not_delaunay"] == 0 and res["not_perturbed_delaunay"] == 0
    assert res["hull_facets"] == dim + 1 and res["missing_vertices"] == 0


def test_validator_catches_planted_flip(oracle):
    """A mistake planted in the oracle's own output (on the CPU) is caught."""
    p = np.random.default_rng(11).random((200, 2))
    t = oracle.Triangulation(p)
    v, nb = t.simplices()
    verts = t.vertices()
    # flip one interior edge shared by two triangles made of input points
    for s in range(len(v)):
        for f in range(3):
            o = nb[s, f]
            if o < 0 or min(v[s, :3].min(), v[o, :3].min()) < 3:
                continue
            g = int(np.where(nb[o] == s)[0][0])
            a = v[s, f]
            b = v[o, g]
            shared = [x for x in v[s, :3] if x != a]
            v2 = v.copy()
            v2[s, :3] = [a, shared[0], b]
            v2[o, :3] = [b, shared[1], a]
            res = oracle.validate(2, verts, v2, nb, expect_vertices=0)
            assert res["not_delaunay"] + res["asymmetric"] + res["non_positive"] > 0
            return
    pytest.fail("no interior edge found")


def test_exact_degenerate_lattice(oracle):
    from voronoids_gb300 import workloads as W
    for dim, side in [(2, 12), (3, 5)]:
        p = W.lattice_points(side, dim) / side
        t = oracle.Triangulation(p)
        assert t.status == 0
        st = t.stats()
        assert st["sos"] > 0  # ties were resolved by the perturbation
        v, nb = t.simplices()
        res = oracle.validate(dim, t.vertices(), v, nb, expect_vertices=len(p) + dim + 1)
        assert res["not_delaunay"] == 0 and res["not_perturbed_delaunay"] == 0
        assert res["non_positive"] == 0 and res["missing_vertices"] == 0


def test_duplicates_keep_lowest_priority(oracle):
    p = np.random.default_rng(5).random((100, 3))
    p = np.vstack([p, p[[3, 7, 7]]])  # 100 == 3, 101 == 7, 102 == 7
    t = oracle.Triangulation(p, seed=9)
    assert t.num_duplicates() == 3
    e = t.edges()
    used = np.unique(e)
    pr = {i: oracle.priority(4 + i, 9) for i in (3, 7, 100, 101, 102)}
    keep3 = min((3, 100), key=lambda i: pr[i])
    keep7 = min((7, 101, 102), key=lambda i: pr[i])
    assert keep3 in used and keep7 in used
    for i in {3, 100} - {keep3}:
        assert i not in used
    for i in {7, 101, 102} - {keep7}:
        assert i not in used


def test_priority_is_a_bijective_mix(oracle):
    # the GPU uses the same mix; spot-check distinctness over a window
    vals = {oracle.priority(v, 12345) for v in range(20000)}
    assert len(vals) == 20000


@pytest.mark.parametrize("dim,n,prefix", [(3, 6000, 1000), (2, 8000, 500), (3, 3000, 10_000)])
def test_parallel_reference_path_same_triangulation(oracle, dim, n, prefix):
    # the reference's parallel path (queue, greedy rounds, per-round updates)
    # restated on threads: the same unique triangulation as the sequential one
    p = W.uniform_points(n, dim, 404 + n)
    a = oracle.Triangulation(p, seed=3)
    b = oracle.Triangulation(p, seed=3, threads=4, prefix=prefix)
    assert a.status == 0 and b.status == 0
    assert np.array_equal(a.edges(), b.edges())


def test_big_golden_digest_of_c1_reproduces(oracle):
    """The committed full-size digests come from tests/golden/make_big_golden.py;
    its 10k-point 2D entry is recomputed here from the oracle."""
    import importlib.util
    import json
    import os
    gdir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    spec = importlib.util.spec_from_file_location("make_big_golden", os.path.join(gdir, "make_big_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    with open(os.path.join(gdir, "big_edges.json")) as f:
        table = json.load(f)
    p = m.workloads()["c1"]()
    rows, sha = m.digest(oracle.Triangulation(p, seed=1).edges())
    assert (rows, sha) == (table["c1"]["edges"], table["c1"]["sha256"])
    assert set(table) >= {"c1", "c2", "c3", "u2"}


def test_float_semantics_agree_with_exact_on_uniform_points(oracle):
    """The reference's inexact path (sequential, input order) gives the exact
    triangulation on well-spread inputs; oracle/float_diagnostic.py reports
    where it does not."""
    from voronoids_gb300 import workloads as W
    for p in (W.c1_points()[:4000], W.uniform_points(3000, 3, 17)):
        f = oracle.FloatTriangulation(p)
        assert f.stats["inserted"] == len(p) and f.stats["empty_located"] == 0
        assert np.array_equal(f.edges(), oracle.Triangulation(p).edges())
        verts, simp, nbr, bad = f.export()
        res = oracle.validate(p.shape[1], verts, simp, nbr, expect_vertices=len(verts))
        assert bad == 0 and res["asymmetric"] == 0 and res["not_delaunay"] == 0



def _shells(dim):
    """The origin and the integer points on concentric spheres (3D) or
    circles (2D): each shell is exactly cospherical (cocircular)."""
    out = [np.zeros((1, dim))]
    for R2 in ((441, 2025) if dim == 3 else (5525, 27625, 71825)):
        R = int(math.isqrt(R2)) + 1
        r = np.arange(-R, R + 1)
        g = np.meshgrid(*([r] * dim), indexing="ij")
        m = sum(x * x for x in g) == R2
        out.append(np.stack([x[m] for x in g], 1))
    return np.concatenate(out).astype(np.float64)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_power_of_two_scaling_keeps_edges(oracle, dim):
    # rescaling by 2^k is exact, and so is the reference's super simplex of the
    # rescaled points: the same triangulation, the same edges
    p = W.uniform_points(600, dim, 870 + dim)
    want = oracle.Triangulation(p, seed=1).edges()
    for k in (-100, -30, 30, 100):
        assert np.array_equal(oracle.Triangulation(p * 2.0 ** k, seed=1).edges(), want), k


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_insertion_order_free_on_exact_ties(oracle, dim):
    # every in-sphere test between points of one shell is an exact tie, decided
    # by the perturbation by vertex id; the triangulation is still unique, so
    # the reference's parallel path (another insertion order, same ids) and the
    # sequential one agree, and the result passes the oracle's validator
    p = _shells(dim)
    a = oracle.Triangulation(p, seed=3)
    b = oracle.Triangulation(p, seed=3, threads=4, prefix=len(p) // 5)
    assert a.status == 0 and b.status == 0
    assert np.array_equal(a.edges(), b.edges())
    v, nb = a.simplices()
    res = oracle.validate(dim, a.vertices(), v, nb, expect_vertices=len(p) + dim + 1)
    assert res["non_positive"] == 0 and res["asymmetric"] == 0
    assert res["not_perturbed_delaunay"] == 0 and res["missing_vertices"] == 0
