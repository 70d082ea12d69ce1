"""GPU: the reference's dictionary view (PyDelauanyTree / PyVertex /
PySimplex, src/lib.rs:12-102) over a GPU tree."""
import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim", [2, 3])
def test_dictionary_view(vd, oracle, dim):
    from voronoids_gb300 import compat
    p = W.uniform_points(1500, dim, 600 + dim)
    t = compat.delaunay(p)
    simp = t.simplices
    vert = t.vertices
    off = 2 * (dim + 1)
    assert t.max_simplex_id == t.tree.max_simplex_id
    # every input point is a vertex with its coordinates, ids from 2 * (dim + 1)
    for i in (0, 1, 777, 1499):
        assert vert[off + i].point == [float(x) for x in p[i]]
    sv, _ = oracle.super_vertices(p)
    for k in range(dim + 1):
        assert np.allclose(vert[k].point, sv[k][:dim], rtol=0, atol=0)
    # incidence lists agree with the simplices
    for vid, v in list(vert.items())[:200]:
        for s in v.simplex:
            assert vid in simp[s].vertices
    # circumspheres: equidistant to the vertices (relative 1e-9 of the radius)
    coords = {vid: np.array(v.point) for vid, v in vert.items()}
    for sid, s in simp.items():
        c = np.array(s.center)
        d = [np.linalg.norm(coords[v] - c) for v in s.vertices]
        assert np.allclose(d, s.radius, rtol=1e-9, atol=0), (sid, d, s.radius)
        for nb in s.neighbors:
            assert sid in simp[nb].neighbors
    # and they agree with the reference's own formula (src/geometry.rs:2-56,
    # restated by the oracle) within 1e-8 of the radius
    for sid, s in list(simp.items())[::5]:
        cr, rr = oracle.circumsphere_float(np.array([coords[v] for v in s.vertices]))
        assert np.all(np.abs(np.array(s.center)[:dim] - cr[:dim]) <= 1e-8 * rr), sid
        assert abs(s.radius - rr) <= 1e-8 * rr, sid
    # the edge graph of the view is the oracle's
    e = set()
    for s in simp.values():
        vs = [v - off for v in s.vertices if v >= off]
        e.update((min(a, b), max(a, b)) for a in vs for b in vs if a != b)
    assert np.array_equal(np.array(sorted(e)), oracle.Triangulation(p).edges())
