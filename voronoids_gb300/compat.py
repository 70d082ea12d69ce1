"""The reference's Python view of a triangulation, over a GPU tree.

``voronoids.delaunay(points)`` of the reference (src/lib.rs:104-125) returns a
``PyDelauanyTree`` whose getters build dictionaries (src/lib.rs:65-102):
``vertices`` {id: PyVertex(point, simplex)}, ``simplices`` {id:
PySimplex(vertices, center, radius, neighbors)} and ``max_simplex_id``.
:func:`delaunay` here returns the same shape, filled from the GPU tree:

* vertex ids follow the reference: the super-simplex vertices are 0..dim,
  input point i is 2 * (dim + 1) + i (the reference numbers its ghost
  vertices dim+1 .. 2*dim+1 in between);
* simplex ids are positions in the GPU tree's simplex export (the reference's
  ids count its creation order, which a parallel build does not share);
* ``center``/``radius`` are the circumspheres of the final simplices,
  computed in FP64 on the GPU (``vd_circumspheres``);
* the reference's ghost simplices (radius 0, outside the super simplex) are
  not materialised: a super-simplex hull face has no neighbour entry.
"""
import ctypes

import numpy as np

from . import _native
from .tree import DelaunayTree, _check, _points


class PyVertex:
    __slots__ = ("point", "simplex")

    def __init__(self, point, simplex):
        self.point = point
        self.simplex = simplex


class PySimplex:
    __slots__ = ("vertices", "center", "radius", "neighbors")

    def __init__(self, vertices, center, radius, neighbors):
        self.vertices = vertices
        self.center = center
        self.radius = radius
        self.neighbors = neighbors


class PyDelauanyTree:
    """Dictionary view of a :class:`DelaunayTree` (the reference's class name)."""

    def __init__(self, tree, points, super_vertices):
        self.tree = tree
        self._points = points
        self._super = super_vertices

    @property
    def max_simplex_id(self):
        return self.tree.max_simplex_id

    def _arrays(self):
        verts, nbrs = self.tree.simplices()
        n = ctypes.c_int64(0)
        L = _native.load()
        dp = ctypes.POINTER(ctypes.c_double)
        _check(L.vd_circumspheres(self.tree._h, None, None, 0, ctypes.byref(n)), "circumspheres")
        centers = np.zeros((n.value, 3))
        radii = np.zeros(n.value)
        _check(L.vd_circumspheres(self.tree._h, centers.ctypes.data_as(dp), radii.ctypes.data_as(dp), n.value,
                                  ctypes.byref(n)), "circumspheres")
        return verts, nbrs, centers, radii

    def _ref_ids(self, v):
        """GPU vertex numbers (super -1-k, points i) -> reference vertex ids."""
        dim = self.tree.dim
        v = np.asarray(v, dtype=np.int64)
        return np.where(v < 0, -1 - v, v + 2 * (dim + 1))

    @property
    def simplices(self):
        dim = self.tree.dim
        verts, nbrs, centers, radii = self._arrays()
        ids = self._ref_ids(verts[:, : dim + 1])
        out = {}
        for s in range(len(verts)):
            nb = [int(x) for x in nbrs[s, : dim + 1] if x >= 0]
            out[s] = PySimplex([int(x) for x in ids[s]], [float(x) for x in centers[s, :dim]], float(radii[s]), nb)
        return out

    @property
    def vertices(self):
        dim = self.tree.dim
        verts, _ = self.tree.simplices()
        ids = self._ref_ids(verts[:, : dim + 1]).ravel()
        owner = np.repeat(np.arange(len(verts)), dim + 1)
        order = np.argsort(ids, kind="stable")
        ids, owner = ids[order], owner[order]
        cuts = np.flatnonzero(np.diff(ids)) + 1
        out = {}
        for grp_ids, grp in zip(np.split(ids, cuts), np.split(owner, cuts)):
            vid = int(grp_ids[0])
            if vid <= dim:
                point = self._super[vid][:dim]
            else:
                point = self._points[vid - 2 * (dim + 1)]
            out[vid] = PyVertex([float(x) for x in point], [int(x) for x in grp])
        return out


def delaunay(points, seed=0):
    """``voronoids.delaunay(points)`` with the reference's dictionary view."""
    p = _points(points)
    t = DelaunayTree(p)
    t.add_points_to_tree(p, seed=seed)
    sv = np.zeros(12)
    r = ctypes.c_double(0)
    dp = ctypes.POINTER(ctypes.c_double)
    _check(_native.load().vd_super_simplex(p.shape[1], p.ctypes.data_as(dp), p.shape[0], sv.ctypes.data_as(dp),
                                           ctypes.byref(r)), "super_simplex")
    return PyDelauanyTree(t, p, sv.reshape(4, 3))
