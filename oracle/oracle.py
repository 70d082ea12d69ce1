"""ctypes wrapper of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module.  The product (``voronoids_gb300``) never does.

The oracle restates the reference's sequential Delaunay semantics with exact
predicates (see the header of ``vd_oracle.cpp`` for the file:line map).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        i64p = ctypes.POINTER(ctypes.c_int64)
        i32p = ctypes.POINTER(ctypes.c_int32)
        llp = ctypes.POINTER(ctypes.c_longlong)
        L.vdo_bounding_sphere.argtypes = [ctypes.c_int, dp, ctypes.c_int64, dp, dp]
        L.vdo_super_vertices.argtypes = [ctypes.c_int, dp, ctypes.c_int64, dp, dp]
        L.vdo_circumsphere_float.argtypes = [ctypes.c_int, dp, dp, dp]
        L.vdo_priority.argtypes = [ctypes.c_uint32, ctypes.c_uint64]
        L.vdo_priority.restype = ctypes.c_uint32
        L.vdo_orient.argtypes = [ctypes.c_int, dp]
        L.vdo_insphere_sos.argtypes = [ctypes.c_int, dp, i32p]
        L.vdo_insphere_exact.argtypes = [ctypes.c_int, dp]
        L.vdo_build.argtypes = [ctypes.c_int, dp, ctypes.c_int64, ctypes.c_uint64,
                                ctypes.POINTER(ctypes.c_int)]
        L.vdo_build.restype = ctypes.c_void_p
        L.vdo_build_parallel.argtypes = [ctypes.c_int, dp, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int,
                                         ctypes.c_int64, ctypes.POINTER(ctypes.c_int)]
        L.vdo_build_parallel.restype = ctypes.c_void_p
        L.vdo_parallel_rounds.restype = ctypes.c_int
        L.vdo_free.argtypes = [ctypes.c_void_p]
        L.vdo_num_duplicates.argtypes = [ctypes.c_void_p]
        L.vdo_num_duplicates.restype = ctypes.c_int64
        L.vdo_stats.argtypes = [ctypes.c_void_p, llp]
        L.vdo_edges.argtypes = [ctypes.c_void_p, i64p, ctypes.c_int64]
        L.vdo_edges.restype = ctypes.c_int64
        L.vdo_num_vertices.argtypes = [ctypes.c_void_p]
        L.vdo_num_vertices.restype = ctypes.c_int64
        L.vdo_vertices.argtypes = [ctypes.c_void_p, dp]
        L.vdo_simplices.argtypes = [ctypes.c_void_p, i32p, i32p]
        L.vdo_simplices.restype = ctypes.c_int64
        L.vdo_validate.argtypes = [ctypes.c_int, dp, ctypes.c_int64, i32p, i32p,
                                   ctypes.c_int64, ctypes.c_int64, llp]
        L.vdo_build_float.argtypes = [ctypes.c_int, dp, ctypes.c_int64, llp]
        L.vdo_build_float.restype = ctypes.c_void_p
        L.vdo_float_edges.argtypes = [ctypes.c_void_p, i64p, ctypes.c_int64]
        L.vdo_float_edges.restype = ctypes.c_int64
        L.vdo_float_export.argtypes = [ctypes.c_void_p, dp, i32p, i32p, llp]
        L.vdo_float_export.restype = ctypes.c_int64
        L.vdo_float_free.argtypes = [ctypes.c_void_p]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def bounding_sphere(points):
    p = _c(points, np.float64)
    dim = p.shape[1]
    c = np.zeros(3)
    r = np.zeros(1)
    lib().vdo_bounding_sphere(dim, _dp(p), p.shape[0], _dp(c), _dp(r))
    return c[:dim], float(r[0])


def super_vertices(points):
    """Super-simplex vertices (dim+1, 3) in the reference's order, and R."""
    p = _c(points, np.float64)
    dim = p.shape[1]
    out = np.zeros((dim + 1, 3))
    r = np.zeros(1)
    lib().vdo_super_vertices(dim, _dp(p), p.shape[0], _dp(out), _dp(r))
    return out, float(r[0])


def circumsphere_float(vertices):
    v = _c(vertices, np.float64)
    dim = v.shape[1]
    c = np.zeros(3)
    r = np.zeros(1)
    lib().vdo_circumsphere_float(dim, _dp(v), _dp(c), _dp(r))
    return c[:dim], float(r[0])


def priority(vid, seed):
    return int(lib().vdo_priority(vid, seed))


def _pad3(pts):
    p = _c(pts, np.float64)
    if p.shape[1] == 2:
        p = np.concatenate([p, np.zeros((p.shape[0], 1))], axis=1)
    return np.ascontiguousarray(p)


def orient(pts):
    """Exact orient of dim+1 points (2D: det[a-c; b-c]; 3D: det[a-d; b-d; c-d])."""
    p = _c(pts, np.float64)
    dim = p.shape[1]
    q = _pad3(p)
    return int(lib().vdo_orient(dim, _dp(q)))


def insphere_sos(simplex, query, keys):
    s = _c(simplex, np.float64)
    dim = s.shape[1]
    q = _pad3(np.vstack([s, np.asarray(query, dtype=np.float64)[None, :]]))
    k = _c(keys, np.int32)
    return int(lib().vdo_insphere_sos(dim, _dp(q), k.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))


def insphere_exact(simplex, query):
    s = _c(simplex, np.float64)
    dim = s.shape[1]
    q = _pad3(np.vstack([s, np.asarray(query, dtype=np.float64)[None, :]]))
    return int(lib().vdo_insphere_exact(dim, _dp(q)))


class Triangulation:
    """Sequential exact Bowyer-Watson over `points` (super simplex sized
    from the same points, as ``voronoids.delaunay`` does)."""

    def __init__(self, points, seed=0, threads=0, prefix=100_000):
        """threads > 0: the reference's parallel path (sequential `prefix`
        points, then 2-ring queue, greedy rounds and per-round parallel
        updates on `threads` host threads); same triangulation."""
        p = _c(points, np.float64)
        self.dim = p.shape[1]
        self.n = p.shape[0]
        st = ctypes.c_int(0)
        if threads > 0:
            self._h = lib().vdo_build_parallel(self.dim, _dp(p), self.n, seed, int(threads), int(prefix),
                                               ctypes.byref(st))
        else:
            self._h = lib().vdo_build(self.dim, _dp(p), self.n, seed, ctypes.byref(st))
        self.status = st.value

    def __del__(self):
        if getattr(self, "_h", None):
            lib().vdo_free(self._h)
            self._h = None

    def edges(self):
        L = lib()
        m = L.vdo_edges(self._h, None, 0)
        out = np.zeros((m, 2), dtype=np.int64)
        L.vdo_edges(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), m)
        return out

    def num_duplicates(self):
        return int(lib().vdo_num_duplicates(self._h))

    def stats(self):
        out = (ctypes.c_longlong * 7)()
        lib().vdo_stats(self._h, out)
        return dict(alive=out[0], created=out[1], exact=out[2], sos=out[3], walk=out[4],
                    max_cavity=out[5], max_facets=out[6])

    def vertices(self):
        L = lib()
        nv = L.vdo_num_vertices(self._h)
        out = np.zeros((nv, 3))
        L.vdo_vertices(self._h, _dp(out))
        return out

    def simplices(self):
        L = lib()
        ns = L.vdo_simplices(self._h, None, None)
        v = np.zeros((ns, 4), dtype=np.int32)
        n = np.zeros((ns, 4), dtype=np.int32)
        i32p = ctypes.POINTER(ctypes.c_int32)
        L.vdo_simplices(self._h, v.ctypes.data_as(i32p), n.ctypes.data_as(i32p))
        return v, n


def validate(dim, verts, simp, nbr, expect_vertices=0):
    """Exact structural + local-Delaunay check of a triangulation.

    Returns a dict of violation counts (all zero for a valid Delaunay
    triangulation) plus the number of facets checked."""
    v = _pad3(verts)
    s = _c(simp, np.int32)
    n = _c(nbr, np.int32)
    out = (ctypes.c_longlong * 8)()
    i32p = ctypes.POINTER(ctypes.c_int32)
    lib().vdo_validate(dim, _dp(v), v.shape[0], s.ctypes.data_as(i32p), n.ctypes.data_as(i32p),
                       s.shape[0], expect_vertices, out)
    keys = ["non_positive", "asymmetric", "not_delaunay", "not_perturbed_delaunay",
            "hull_facets", "facets", "missing_vertices", "exact_calls"]
    return dict(zip(keys, list(out)))


class FloatTriangulation:
    """The reference's own insertion path with its floating-point conflict
    test (circumsphere centre and radius, then ``dist^2 < r^2``), sequential
    in input order: a diagnostic of how the reference's inexact decisions
    differ from the exact triangulation.  See ``vdo_build_float``."""

    def __init__(self, points):
        p = _c(points, np.float64)
        self.dim = p.shape[1]
        st = (ctypes.c_longlong * 8)()
        self._h = lib().vdo_build_float(self.dim, _dp(p), p.shape[0], st)
        if not self._h:
            raise ValueError("bad input")
        keys = ["inserted", "empty_located", "malformed_new", "max_killed", "live_simplices", "vertices"]
        self.stats = dict(zip(keys, list(st)[:6]))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().vdo_float_free(self._h)
            self._h = None

    def edges(self):
        L = lib()
        m = L.vdo_float_edges(self._h, None, 0)
        out = np.zeros((m, 2), dtype=np.int64)
        L.vdo_float_edges(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), m)
        return out

    def export(self):
        """(verts (nv, 3), simplices (ns, 4) int32, neighbours (ns, 4) int32,
        links that could not be placed on a face) in ``validate``'s layout."""
        L = lib()
        i32p = ctypes.POINTER(ctypes.c_int32)
        ns = L.vdo_float_export(self._h, None, None, None, None)
        nv = self.stats["vertices"] - (self.dim + 1)
        verts = np.zeros((nv, 3))
        simp = np.zeros((ns, 4), dtype=np.int32)
        nbr = np.zeros((ns, 4), dtype=np.int32)
        bad = ctypes.c_longlong(0)
        L.vdo_float_export(self._h, _dp(verts), simp.ctypes.data_as(i32p), nbr.ctypes.data_as(i32p),
                           ctypes.byref(bad))
        return verts, simp, nbr, int(bad.value)
