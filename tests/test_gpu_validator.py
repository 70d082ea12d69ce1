"""GPU: the exact validator rejects triangulations that are not Delaunay.

The device validator (``vd_check.cu``) replaces the reference's
``check_delaunay`` (src/delaunay_tree.rs:512-541 3D, :642-671 2D).  A valid GPU
build is exported, edited on the host into a wrong triangulation and checked
again through ``vd_check_triangulation``:

  * an edge flip (2D) / a 2-3 flip (3D) of an interior facet: still a
    triangulation with symmetric links and positive simplices, but the new
    facets are not locally Delaunay;
  * a one-sided neighbour link;
  * a simplex with two vertices swapped (negative orientation).

Each verdict must be "not ok" with the violation counts of the oracle's
independent CPU validator (big-integer predicates) on the same arrays.
"""
import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu

KEYS = ["non_positive", "asymmetric", "not_delaunay", "not_perturbed_delaunay", "hull_facets", "facets"]


def exported(vd, oracle, dim, n, seed):
    """A GPU build as (points incl. super vertices, vertex ids, neighbour ids)."""
    p = W.uniform_points(n, dim, seed)
    t = vd.delaunay(p, seed=1)
    v, nb = t.simplices()
    t.close()
    sv, _ = oracle.super_vertices(p)
    pts = np.vstack([sv[:, :dim], p])
    ids = np.where(v < 0, -v - 1, v + dim + 1).astype(np.int32)
    if dim == 2:
        ids[:, 3] = -1
    return pts, ids, nb.astype(np.int32).copy()


def both(vd, oracle, dim, pts, ids, nb):
    ok, viol = vd.check_triangulation(pts, ids, nb)
    ref = oracle.validate(dim, pts, ids, nb)
    return ok, viol, {k: ref[k] for k in KEYS}


def orient(oracle, pts, tet):
    return oracle.orient(pts[list(tet)])


def flip_2d(oracle, pts, ids, nb, nsuper):
    """Flip the first interior edge whose quadrilateral is convex."""
    for s in range(len(ids)):
        for f in range(3):
            o = int(nb[s, f])
            if o <= s or (ids[s, :3] < nsuper).any() or (ids[o, :3] < nsuper).any():
                continue
            a, b = ids[s, :3].tolist(), ids[o, :3].tolist()
            g = nb[o, :3].tolist().index(s)
            p, q, r, x = a[f], a[(f + 1) % 3], a[(f + 2) % 3], b[g]
            if orient(oracle, pts, (p, q, x)) <= 0 or orient(oracle, pts, (p, x, r)) <= 0:
                continue
            n_rp, n_pq = int(nb[s, (f + 1) % 3]), int(nb[s, (f + 2) % 3])
            n_xr, n_xq = int(nb[o, b.index(q)]), int(nb[o, b.index(r)])
            ids[s, :3] = (p, q, x)
            nb[s, :3] = (n_xq, o, n_pq)
            ids[o, :3] = (p, x, r)
            nb[o, :3] = (n_xr, n_rp, s)
            for m, old, new in ((n_xq, o, s), (n_rp, s, o)):
                if m >= 0:
                    nb[m, :3] = np.where(nb[m, :3] == old, new, nb[m, :3])
            return ids, nb
    raise AssertionError("no convex interior quadrilateral found")


def flip_23(oracle, pts, ids, nb, nsuper):
    """2-3 flip of the first interior facet whose opposite vertices see it
    from both sides: three tetrahedra around the new edge replace two."""
    for s in range(len(ids)):
        for f in range(4):
            o = int(nb[s, f])
            if o <= s or (ids[s] < nsuper).any() or (ids[o] < nsuper).any():
                continue
            a, b = ids[s].tolist(), ids[o].tolist()
            g = nb[o].tolist().index(s)
            p, x = a[f], b[g]
            u = [a[i] for i in range(4) if i != f]
            edges = [(u[0], u[1], u[2]), (u[1], u[2], u[0]), (u[2], u[0], u[1])]
            sg = [orient(oracle, pts, (p, x, i, j)) for i, j, _ in edges]
            if 0 in sg or len(set(sg)) != 1:
                continue
            slots = [s, o, len(ids)]
            ids = np.vstack([ids, np.full((1, 4), -1, np.int32)])
            nb = np.vstack([nb, np.full((1, 4), -1, np.int32)])
            slot_of = {}
            outer = []
            for k, (i, j, w) in enumerate(edges):
                if sg[0] < 0:
                    i, j = j, i
                slot_of[w] = slots[k]  # the tetrahedron without w
                outer.append((int(nb[o, b.index(w)]), o, int(nb[s, a.index(w)]), s))
            new_rows = []
            for k, (i, j, w) in enumerate(edges):
                if sg[0] < 0:
                    i, j = j, i
                n_opp_p = outer[k][0]   # across (x, i, j): o's face opposite w
                n_opp_x = outer[k][2]   # across (p, i, j): s's face opposite w
                new_rows.append(((p, x, i, j), (n_opp_p, n_opp_x, slot_of[i], slot_of[j])))
            for k, (tv, tn) in enumerate(new_rows):
                ids[slots[k]] = tv
                nb[slots[k]] = tn
            for k, (n_o, old_o, n_s, old_s) in enumerate(outer):
                for m, old in ((n_o, old_o), (n_s, old_s)):
                    if m >= 0:
                        nb[m] = np.where(nb[m] == old, slots[k], nb[m])
            return ids, nb
    raise AssertionError("no flippable interior facet found")


@pytest.mark.parametrize("dim", [2, 3])
def test_valid_build_passes_both_validators(vd, oracle, dim):
    pts, ids, nb = exported(vd, oracle, dim, 3000, 500 + dim)
    ok, viol, ref = both(vd, oracle, dim, pts, ids, nb)
    assert ok, viol
    assert viol == ref
    assert viol["hull_facets"] == dim + 1 and viol["facets"] > 0


@pytest.mark.parametrize("dim", [2, 3])
def test_flip_is_caught(vd, oracle, dim):
    pts, ids, nb = exported(vd, oracle, dim, 2000, 600 + dim)
    flip = flip_2d if dim == 2 else flip_23
    ids, nb = flip(oracle, pts, ids, nb, dim + 1)
    ok, viol, ref = both(vd, oracle, dim, pts, ids, nb)
    assert not ok
    assert viol["non_positive"] == 0 and viol["asymmetric"] == 0
    assert viol["not_delaunay"] >= 1 and viol["not_perturbed_delaunay"] >= 1
    assert viol == ref


@pytest.mark.parametrize("dim", [2, 3])
def test_one_sided_link_is_caught(vd, oracle, dim):
    pts, ids, nb = exported(vd, oracle, dim, 2000, 700 + dim)
    nv = dim + 1
    s = next(i for i in range(len(ids)) if (nb[i, :nv] >= 0).all() and (ids[i, :nv] >= nv).all())
    other = next(i for i in range(len(ids)) if i != s and i not in nb[s, :nv] and s not in nb[i, :nv])
    nb[s, 0] = other  # s claims a neighbour that does not know it; the old neighbour still points at s
    ok, viol, ref = both(vd, oracle, dim, pts, ids, nb)
    assert not ok
    assert viol["asymmetric"] == 2
    assert viol == ref


@pytest.mark.parametrize("dim", [2, 3])
def test_flipped_orientation_is_caught(vd, oracle, dim):
    pts, ids, nb = exported(vd, oracle, dim, 2000, 800 + dim)
    nv = dim + 1
    s = next(i for i in range(len(ids)) if (ids[i, :nv] >= nv).all())
    ids[s, [0, 1]] = ids[s, [1, 0]]  # swap two vertices and their faces: same simplex, other orientation
    nb[s, [0, 1]] = nb[s, [1, 0]]
    ok, viol, ref = both(vd, oracle, dim, pts, ids, nb)
    assert not ok
    assert viol["non_positive"] == 1 and viol["asymmetric"] == 0
    assert viol == ref


def test_out_of_range_ids_are_structural_faults(vd, oracle):
    pts, ids, nb = exported(vd, oracle, 3, 1000, 901)
    ids[5, 2] = len(pts) + 7      # vertex id past the points
    nb[9, 1] = len(ids) + 3       # neighbour id past the simplices
    ok, viol = vd.check_triangulation(pts, ids, nb)
    assert not ok and viol["asymmetric"] >= 2


def test_bad_arguments_are_rejected(vd):
    import ctypes
    from voronoids_gb300 import _native
    with pytest.raises(ValueError):
        vd.check_triangulation(np.zeros((4, 3)), np.zeros((1, 4), np.int32), np.zeros((1, 3), np.int32))
    pts = np.zeros((4, 3))
    v = np.zeros((1, 4), np.int32)
    ok = ctypes.c_int(7)
    i32p = ctypes.POINTER(ctypes.c_int32)
    rc = _native.load().vd_check_triangulation(4, pts.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 4,
                                               v.ctypes.data_as(i32p), v.ctypes.data_as(i32p), 1,
                                               ctypes.byref(ok), None)
    assert rc == 1  # VD_ERR_ARG: dimension 4
