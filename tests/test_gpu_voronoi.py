"""GPU: the Voronoi dual of a build against a dual derived from the oracle.

The reference's purpose is the Voronoi tessellation (README.md:2-4); it keeps
only the Voronoi vertices, the circumcentre and radius of every simplex
(src/delaunay_tree.rs:10-17, computed by src/geometry.rs:2-56).  The GPU
gives the vertices (vd_circumspheres), the edges (vd_voronoi_edges: simplex
pairs sharing a facet) and the cells (vd_voronoi_cells: simplices incident to
each input vertex).  Simplices are matched with the oracle's by their vertex
sets, so the two numberings need not agree.  Circumcentres are compared with
the oracle's restatement of the reference's own formula (nalgebra LU in 3D,
slope formula in 2D) within 1e-8 of the radius; the two FP64 evaluations
differ by about 1e-11 of the radius on these inputs.
"""
import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def keys_gpu(v, dim):
    return [tuple(sorted(r[: dim + 1].tolist())) for r in v]


def keys_oracle(ov, dim):
    ns = dim + 1
    out = []
    for r in ov:
        ids = [(-(1 + x) if x < ns else x - ns) for x in r[: dim + 1].tolist()]
        out.append(tuple(sorted(ids)))
    return out


@pytest.mark.parametrize("dim,n", [(2, 3000), (3, 3000)])
def test_voronoi_dual_matches_oracle(vd, oracle, dim, n):
    p = W.uniform_points(n, dim, 900 + dim)
    t = vd.delaunay(p, seed=2)
    v, _ = t.simplices()
    kg = keys_gpu(v, dim)
    ov, on = oracle.Triangulation(p).simplices()
    ko = keys_oracle(ov, dim)
    assert set(kg) == set(ko) and len(kg) == len(ko)

    # edges: one per interior facet, sorted, i < j
    E = t.voronoi_edges()
    assert np.all(E[:, 0] < E[:, 1])
    k = E[:, 0] * len(kg) + E[:, 1]
    assert np.all(np.diff(k) > 0)
    got = {frozenset((kg[i], kg[j])) for i, j in E.tolist()}
    want = set()
    for s in range(len(ov)):
        for f in range(dim + 1):
            o = int(on[s, f])
            if o > s:
                want.add(frozenset((ko[s], ko[o])))
    assert got == want
    assert 2 * len(E) + (dim + 1) == (dim + 1) * len(kg)  # facets: interior twice, hull once

    # cells: the simplices incident to each input vertex, sorted
    off, ids = t.voronoi_cells()
    assert off.shape == (n + 1,) and off[-1] == len(ids)
    inc = [set() for _ in range(n)]
    for key in ko:
        for x in key:
            if x >= 0:
                inc[x].add(key)
    for u in range(n):
        cell = ids[off[u]:off[u + 1]]
        assert np.all(np.diff(cell) > 0)
        assert {kg[i] for i in cell.tolist()} == inc[u]

    # vertices: circumcentres against the reference's formula
    c, r = t.circumspheres()
    sv, _ = oracle.super_vertices(p)
    pts = np.vstack([sv[:, :dim], p])
    for i in range(0, len(v), 7):
        ids_i = [(-x - 1) if x < 0 else x + dim + 1 for x in v[i, : dim + 1].tolist()]
        cr, rr = oracle.circumsphere_float(pts[ids_i])
        assert np.all(np.abs(c[i, :dim] - cr[:dim]) <= 1e-8 * rr), i
        assert abs(r[i] - rr) <= 1e-8 * rr, i


def test_voronoi_dual_of_a_batched_tree(vd):
    """A batched tree holds several sets; its dual covers all of them, in the
    global numbering of vd_simplices, and each set's cells are its own."""
    sets = [W.uniform_points(n, 3, 300 + n) for n in (400, 1500, 60)]
    off = np.concatenate([[0], np.cumsum([len(p) for p in sets])])
    t = vd.DelaunayTree.create(3)
    t.batch(np.concatenate(sets), off, seed=3)
    v, nb = t.simplices()
    E = t.voronoi_edges()
    assert 2 * len(E) + 4 * len(sets) == 4 * len(v)  # every super simplex keeps its 4 hull faces
    cells_off, ids = t.voronoi_cells()
    assert len(cells_off) == off[-1] + 1
    for s in range(len(sets)):
        for u in range(off[s], off[s + 1]):
            cell = ids[cells_off[u]:cells_off[u + 1]]
            assert len(cell) > 0
            # a cell's simplices belong to the point's own set: their input vertices share its range
            verts = v[cell]
            inner = verts[verts >= 0]
            assert np.all((inner >= off[s]) & (inner < off[s + 1]))
    t.close()


def test_voronoi_cells_skip_duplicates(vd):
    p = W.uniform_points(500, 3, 77)
    p = np.vstack([p, p[:3]])
    with pytest.warns(RuntimeWarning):
        t = vd.delaunay(p, seed=1)
    off, ids = t.voronoi_cells()
    sizes = np.diff(off)
    skipped = t.duplicates()[:, 0]  # of equal points, the one with the lowest priority is kept
    assert len(skipped) == 3
    assert np.all(sizes[skipped] == 0)
    assert np.all(np.delete(sizes, skipped) > 0)
    # every live simplex with no super vertex appears in exactly dim + 1 cells
    v, _ = t.simplices()
    inner = np.all(v >= 0, axis=1)
    counts = np.bincount(ids, minlength=len(v))
    assert np.all(counts[inner] == 4)
