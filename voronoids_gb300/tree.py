"""Python mirror of the reference's DelaunayTree API on the GB300 library.

Reference surface (kazewong/Voronoids):
  DelaunayTree::<N, N+1>::new(points)      src/delaunay_tree.rs:389-510, 544-640
  DelaunayTree::insert_point(&update)      src/delaunay_tree.rs:125-211 (+ TreeUpdate::new :709-740)
  DelaunayTree::add_points_to_tree(points) src/delaunay_tree.rs:336-386
  DelaunayTree::check_delaunay()           src/delaunay_tree.rs:512-541, 642-671
  DelaunayTree::max_simplex_id             src/delaunay_tree.rs:29
  voronoids.delaunay(points)               src/lib.rs:104-125

The reference panics on failure; here every failure raises ``VDError`` with
the library's status, except duplicate points, which are skipped and
reported through ``duplicates()`` (the reference panics on them).
"""
import ctypes
import warnings

import numpy as np

from . import _native


class VDError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        name = _native.STATUS.get(status, str(status))
        msg = _native.load().vd_status_str(status).decode()
        super().__init__(f"{what}: {name} ({msg})" if what else f"{name} ({msg})")


def _check(rc, what):
    if rc == _native.VD_OK:
        return
    if rc == _native.VD_ERR_DUPLICATE:
        warnings.warn(f"{what}: duplicate points were skipped", RuntimeWarning, stacklevel=3)
        return
    raise VDError(rc, what)


def _points(points, dim=None):
    p = np.ascontiguousarray(points, dtype=np.float64)
    if p.ndim == 1:
        p = p.reshape(1, -1)
    if p.ndim != 2 or p.shape[1] not in (2, 3) or (dim is not None and p.shape[1] != dim):
        raise ValueError(f"points must have shape (n, {dim or '2|3'}), got {p.shape}")
    return p


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class DelaunayTree:
    """A Delaunay triangulation held on the GPU.

    ``DelaunayTree(points)`` sizes the super simplex from ``points`` exactly as
    the reference's ``new`` does; the points are not inserted."""

    def __init__(self, points, stream=None):
        L = _native.load()
        p = _points(points)
        self.dim = p.shape[1]
        st = ctypes.c_int(0)
        if stream is None:
            h = L.vd_tree_new(self.dim, _dp(p), p.shape[0], ctypes.byref(st))
        else:
            h = L.vd_tree_new_on_stream(self.dim, _dp(p), p.shape[0], ctypes.c_void_p(stream),
                                        ctypes.byref(st))
        if not h:
            raise VDError(3, "vd_tree_new")
        self._h = ctypes.c_void_p(h)
        if st.value != _native.VD_OK:
            L.vd_tree_free(self._h)
            self._h = None
            raise VDError(st.value, "vd_tree_new")

    # -- lifetime ---------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            _native.load().vd_tree_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- insertion --------------------------------------------------------------
    def add_points_to_tree(self, points, seed=0):
        """Round-parallel insertion of all ``points`` (host array)."""
        p = _points(points, self.dim)
        _check(_native.load().vd_insert_points(self._h, _dp(p), p.shape[0], seed), "add_points_to_tree")

    def add_points_device(self, ptr, n, seed=0):
        """Insert ``n`` points already in device memory (row-major f64, ``dim`` per point)."""
        _check(_native.load().vd_insert_points_device(self._h, ctypes.c_void_p(ptr), n, seed),
               "add_points_device")

    def insert_point(self, point):
        p = _points(point, self.dim)
        _check(_native.load().vd_insert_point(self._h, _dp(p)), "insert_point")

    # -- queries ----------------------------------------------------------------
    def _i64(self, fn):
        out = ctypes.c_int64(0)
        _check(fn(self._h, ctypes.byref(out)), fn.__name__)
        return out.value

    @property
    def max_simplex_id(self):
        return self._i64(_native.load().vd_max_simplex_id)

    @property
    def num_vertices(self):
        return self._i64(_native.load().vd_num_vertices)

    @property
    def num_simplices(self):
        return self._i64(_native.load().vd_num_simplices)

    def edges(self):
        """Sorted (u, v) input-index pairs, u < v, as an (m, 2) int64 array."""
        L = _native.load()
        m = ctypes.c_int64(0)
        _check(L.vd_edges(self._h, None, 0, ctypes.byref(m)), "edges")
        out = np.zeros((m.value, 2), dtype=np.int64)
        _check(L.vd_edges(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), m.value,
                          ctypes.byref(m)), "edges")
        return out

    def edges_device(self, ptr, cap):
        """Write the edge list as uint32 pairs to device memory; returns the count."""
        m = ctypes.c_int64(0)
        _check(_native.load().vd_edges_device(self._h, ctypes.c_void_p(ptr), cap, ctypes.byref(m)),
               "edges_device")
        return m.value

    def num_edges(self):
        return self._i64(_native.load().vd_num_edges)

    def simplices(self):
        """(verts, nbrs) int32 arrays of shape (s, 4).  Super vertices are -1-k;
        neighbour -1 is the super-simplex hull."""
        L = _native.load()
        n = ctypes.c_int64(0)
        _check(L.vd_simplices(self._h, None, None, 0, ctypes.byref(n)), "simplices")
        v = np.zeros((n.value, 4), dtype=np.int32)
        nb = np.zeros((n.value, 4), dtype=np.int32)
        i32p = ctypes.POINTER(ctypes.c_int32)
        _check(L.vd_simplices(self._h, v.ctypes.data_as(i32p), nb.ctypes.data_as(i32p), n.value,
                              ctypes.byref(n)), "simplices")
        return v, nb

    def check_delaunay(self, details=False):
        ok = ctypes.c_int(0)
        viol = (ctypes.c_int64 * 6)()
        _check(_native.load().vd_check_delaunay(self._h, ctypes.byref(ok), viol), "check_delaunay")
        if details:
            keys = ["non_positive", "asymmetric", "not_delaunay", "not_perturbed_delaunay",
                    "hull_facets", "facets"]
            return bool(ok.value), dict(zip(keys, list(viol)))
        return bool(ok.value)

    def duplicates(self):
        L = _native.load()
        n = ctypes.c_int64(0)
        _check(L.vd_duplicates(self._h, None, 0, ctypes.byref(n)), "duplicates")
        out = np.zeros((n.value, 2), dtype=np.int64)
        if n.value:
            _check(L.vd_duplicates(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                   n.value, ctypes.byref(n)), "duplicates")
        return out

    def set_schedule(self, first_prefix=64, growth=1.25, ratio=0.12):
        _check(_native.load().vd_set_schedule(self._h, int(first_prefix), float(growth), float(ratio)),
               "set_schedule")

    def set_tuning(self, passes=3, thin=1):
        _check(_native.load().vd_set_tuning(self._h, int(passes), int(thin)), "set_tuning")

    def set_graphs(self, on=True):
        _check(_native.load().vd_set_graphs(self._h, int(on)), "set_graphs")

    def set_profiling(self, on=True):
        _check(_native.load().vd_set_profiling(self._h, int(on)), "set_profiling")

    def profile(self):
        """{kernel: (milliseconds, launches)} summed since profiling was enabled."""
        L = _native.load()
        n = ctypes.c_int(0)
        _check(L.vd_profile(self._h, None, None, 0, ctypes.byref(n)), "profile")
        ms = np.zeros(n.value)
        cnt = np.zeros(n.value, dtype=np.int64)
        _check(L.vd_profile(self._h, _dp(ms), cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n.value,
                            ctypes.byref(n)), "profile")
        return {L.vd_profile_name(i).decode(): (float(ms[i]), int(cnt[i])) for i in range(n.value)}

    def set_trace(self, on=True):
        _check(_native.load().vd_set_trace(self._h, int(on)), "set_trace")

    def trace(self):
        L = _native.load()
        n = ctypes.c_int64(0)
        _check(L.vd_trace(self._h, None, 0, ctypes.byref(n)), "trace")
        out = np.zeros((n.value, 8), dtype=np.int64)
        if n.value:
            _check(L.vd_trace(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n.value,
                              ctypes.byref(n)), "trace")
        return out

    def stats(self):
        s = _native.VdStats()
        _check(_native.load().vd_get_stats(self._h, ctypes.byref(s)), "stats")
        return {k: getattr(s, k) for k, _ in s._fields_}


def delaunay(points, seed=0):
    """``voronoids.delaunay(points)``: new(points) + insert all points.

    The reference inserts the first 1e5 points one at a time and the rest
    with ``add_points_to_tree``; the result is the same triangulation, so
    every point goes through the round-parallel path here."""
    p = _points(points)
    t = DelaunayTree(p)
    t.add_points_to_tree(p, seed=seed)
    return t
