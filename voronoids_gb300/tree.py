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

    @classmethod
    def create(cls, dim, stream=None):
        """An empty tree (no super simplex yet), e.g. for :meth:`batch`."""
        L = _native.load()
        st = ctypes.c_int(0)
        h = L.vd_tree_create(int(dim), ctypes.c_void_p(stream) if stream is not None else None, ctypes.byref(st))
        if not h:
            raise VDError(3, "vd_tree_create")
        self = cls.__new__(cls)
        self.dim = int(dim)
        self._h = ctypes.c_void_p(h)
        if st.value != _native.VD_OK:
            L.vd_tree_free(self._h)
            self._h = None
            raise VDError(st.value, "vd_tree_create")
        return self

    # -- batched build ------------------------------------------------------------
    def batch(self, points, offsets, seed=0):
        """Triangulate the sets ``points[offsets[s]:offsets[s+1]]`` together.

        Returns ``(uv, edge_offsets)``: uint32 pairs numbered within each set
        and the (nsets + 1) bounds of each set's edges."""
        p = _points(points, self.dim)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nsets = off.shape[0] - 1
        eoff = np.zeros(nsets + 1, dtype=np.int64)
        L = _native.load()
        i64p = ctypes.POINTER(ctypes.c_int64)
        cap = (10 if self.dim == 3 else 4) * p.shape[0] + 64  # above any uniform-density edge count
        for _ in range(2):
            uv = np.zeros((cap, 2), dtype=np.uint32)
            rc = L.vd_batch_delaunay(self._h, _dp(p), off.ctypes.data_as(i64p), nsets, seed,
                                     uv.ctypes.data_as(ctypes.c_void_p), cap, eoff.ctypes.data_as(i64p))
            if rc == 1 and eoff[-1] > cap:  # more edges than the first guess: exact size
                cap = int(eoff[-1])
                continue
            break
        if rc not in (_native.VD_OK, _native.VD_ERR_DUPLICATE):
            _check(rc, "batch")
        return uv[: int(eoff[-1])], eoff

    def batch_device(self, ptr, offsets, seed, out_ptr, cap):
        """Device variant of :meth:`batch`; returns the edge offsets."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        nsets = off.shape[0] - 1
        eoff = np.zeros(nsets + 1, dtype=np.int64)
        i64p = ctypes.POINTER(ctypes.c_int64)
        rc = _native.load().vd_batch_delaunay_device(self._h, ctypes.c_void_p(ptr), off.ctypes.data_as(i64p), nsets,
                                                     seed, ctypes.c_void_p(out_ptr), cap, eoff.ctypes.data_as(i64p))
        if rc not in (_native.VD_OK, _native.VD_ERR_DUPLICATE):
            _check(rc, "batch_device")
        return eoff

    def set_launch(self, warps_per_sm=20, blocks_per_sm=8):
        _check(_native.load().vd_set_launch(self._h, int(warps_per_sm), int(blocks_per_sm)), "set_launch")

    def autotune_batch(self, ptr, offsets, sample_points=2_000_000):
        """Tune launch shape and round settings on a sample of a device batch;
        returns the chosen setting."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        out = np.zeros(9, dtype=np.int64)
        i64p = ctypes.POINTER(ctypes.c_int64)
        _check(_native.load().vd_autotune_batch(self._h, ctypes.c_void_p(ptr), off.ctypes.data_as(i64p),
                                                 off.shape[0] - 1, int(sample_points), out.ctypes.data_as(i64p)),
               "autotune_batch")
        keys = ("warps_per_sm", "blocks_per_sm", "passes", "thin", "ratio_x1000", "sample_us", "sample_points",
                "sample_sets", "adjacent")
        return dict(zip(keys, out.tolist()))

    def locate(self, points):
        """Conflict regions (``locate``): for each query point the sorted ids
        (numbered as :meth:`simplices` returns them) of the simplices whose
        circumsphere strictly contains it.  One point -> one array; many ->
        a list of arrays."""
        q = np.asarray(points, dtype=np.float64)
        single = q.ndim == 1
        q = _points(q.reshape(1, -1) if single else q, self.dim)
        nq = q.shape[0]
        off = np.zeros(nq + 1, dtype=np.int64)
        L = _native.load()
        i64p = ctypes.POINTER(ctypes.c_int64)
        rc = L.vd_locate_points(self._h, _dp(q), nq, off.ctypes.data_as(i64p), None, 0)
        if rc not in (_native.VD_OK, 6):
            _check(rc, "locate")
        ids = np.zeros(max(int(off[-1]), 1), dtype=np.int64)
        rc = L.vd_locate_points(self._h, _dp(q), nq, off.ctypes.data_as(i64p), ids.ctypes.data_as(i64p), ids.shape[0])
        if rc not in (_native.VD_OK, 6):
            _check(rc, "locate")
        out = [ids[off[i]:off[i + 1]] for i in range(nq)]
        return out[0] if single else out

    def num_sets(self):
        n = ctypes.c_int(0)
        _check(_native.load().vd_num_sets(self._h, ctypes.byref(n)), "num_sets")
        return n.value

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

    def reset(self, points):
        """Empty the tree and size its super simplex from ``points`` (host),
        keeping its device allocations."""
        p = _points(points, self.dim)
        _check(_native.load().vd_tree_reset(self._h, _dp(p), p.shape[0]), "reset")

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

    def circumspheres(self):
        """Circumcentre (3 per simplex, z = 0 in 2D) and radius of every live
        simplex, in :meth:`simplices` order: the Voronoi vertices."""
        L = _native.load()
        n = ctypes.c_int64(0)
        _check(L.vd_circumspheres(self._h, None, None, 0, ctypes.byref(n)), "circumspheres")
        c = np.zeros((n.value, 3))
        r = np.zeros(n.value)
        _check(L.vd_circumspheres(self._h, _dp(c), _dp(r), n.value, ctypes.byref(n)), "circumspheres")
        return c, r

    def voronoi_edges(self):
        """(m, 2) int64 pairs (i, j), i < j, of simplices sharing a facet: the
        Voronoi edges between circumcentres i and j, sorted."""
        L = _native.load()
        n = ctypes.c_int64(0)
        _check(L.vd_voronoi_edges(self._h, None, 0, ctypes.byref(n)), "voronoi_edges")
        out = np.zeros((n.value, 2), dtype=np.int64)
        _check(L.vd_voronoi_edges(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), n.value,
                                  ctypes.byref(n)), "voronoi_edges")
        return out

    def voronoi_cells(self):
        """(offsets, ids): the sorted simplices incident to input vertex v (the
        vertices of its Voronoi cell) are ids[offsets[v]:offsets[v+1]]."""
        L = _native.load()
        i64p = ctypes.POINTER(ctypes.c_int64)
        off = np.zeros(self.num_vertices + 1, dtype=np.int64)
        _check(L.vd_voronoi_cells(self._h, off.ctypes.data_as(i64p), None, 0), "voronoi_cells")
        ids = np.zeros(max(int(off[-1]), 1), dtype=np.int64)
        _check(L.vd_voronoi_cells(self._h, off.ctypes.data_as(i64p), ids.ctypes.data_as(i64p), ids.shape[0]),
               "voronoi_cells")
        return off, ids[: int(off[-1])]

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

    def set_adjacent(self, on=True):
        """Round mode: 1 lets touching cavities win together (see vd_set_adjacent)."""
        _check(_native.load().vd_set_adjacent(self._h, int(on)), "set_adjacent")

    def set_early_phase(self, until_inserted=0, thin=0, ratio=0.5):
        """Rounds of the early phase (fewer than `until_inserted` points in): thinning radius and feed ratio."""
        _check(_native.load().vd_set_early_phase(self._h, int(until_inserted), int(thin), float(ratio)),
               "set_early_phase")

    def set_first_block(self, max_points):
        """First whole priority levels of a fresh call (at most ``max_points``, capped by the
        block's capacity of 320 points in 3D and 641 in 2D) inserted by one block before the
        rounds; 0 turns it off (default: 150)."""
        _check(_native.load().vd_set_first_block(self._h, int(max_points)), "set_first_block")

    def set_exact_tier(self, mode=0, switch_after=32):
        """Exact tier of the conflict tests: 0 automatic, 1 expansions only, 2 integer first (see vd_set_exact_tier)."""
        _check(_native.load().vd_set_exact_tier(self._h, int(mode), int(switch_after)), "set_exact_tier")

    def set_small_rounds(self, max_active=16384):
        """Run rounds in one cooperative launch while fewer points are active (0: never)."""
        _check(_native.load().vd_set_small_rounds(self._h, int(max_active)), "set_small_rounds")

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


def check_triangulation(points, verts, nbrs):
    """``check_delaunay`` on a caller's triangulation (``vd_check_triangulation``).

    ``points`` (npts, dim) are the vertices by id (any super vertices
    included), ``verts`` (ns, 4) int32 vertex ids oriented as
    :meth:`DelaunayTree.simplices` exports them, ``nbrs`` (ns, 4) the simplex
    across the face opposite each vertex (-1 on the hull).  Returns
    ``(ok, violations)``; the violations are counted on the GPU exactly as
    :meth:`DelaunayTree.check_delaunay` counts them."""
    p = _points(points)
    v = np.ascontiguousarray(verts, dtype=np.int32)
    nb = np.ascontiguousarray(nbrs, dtype=np.int32)
    if v.ndim != 2 or v.shape[1] != 4 or nb.shape != v.shape:
        raise ValueError("verts and nbrs must both have shape (ns, 4)")
    ok = ctypes.c_int(0)
    viol = (ctypes.c_int64 * 6)()
    i32p = ctypes.POINTER(ctypes.c_int32)
    _check(_native.load().vd_check_triangulation(p.shape[1], _dp(p), p.shape[0], v.ctypes.data_as(i32p),
                                                 nb.ctypes.data_as(i32p), v.shape[0], ctypes.byref(ok), viol),
           "check_triangulation")
    keys = ["non_positive", "asymmetric", "not_delaunay", "not_perturbed_delaunay", "hull_facets", "facets"]
    return bool(ok.value), dict(zip(keys, list(viol)))


def delaunay(points, seed=0):
    """``voronoids.delaunay(points)``: new(points) + insert all points.

    The reference inserts the first 1e5 points one at a time and the rest
    with ``add_points_to_tree``; the result is the same triangulation, so
    every point goes through the round-parallel path here."""
    p = _points(points)
    t = DelaunayTree(p)
    t.add_points_to_tree(p, seed=seed)
    return t


def delaunay_batch(point_sets, seed=0, tree=None):
    """Triangulate many independent point sets in one batched build.

    Returns one sorted (m, 2) int64 edge array per set, numbered within the
    set; each equals ``delaunay(points, seed).edges()`` of that set alone."""
    sets = [_points(p) for p in point_sets]
    dim = sets[0].shape[1]
    off = np.zeros(len(sets) + 1, dtype=np.int64)
    off[1:] = np.cumsum([p.shape[0] for p in sets])
    t = tree if tree is not None else DelaunayTree.create(dim)
    try:
        uv, eoff = t.batch(np.concatenate(sets, axis=0), off, seed=seed)
    finally:
        if tree is None:
            t.close()
    return [uv[eoff[s]:eoff[s + 1]].astype(np.int64) for s in range(len(sets))]


class Server:
    """Continuous-batching triangulation server (``vd_server_*``).

    ``submit(points)`` queues a request and returns its id; ``poll()`` returns
    the ids finished since the last call; ``result(id)`` returns the sorted
    (m, 2) int64 edge array of a finished request (numbered within it)."""

    def __init__(self, pool_bytes=64 << 30, slots=2, max_batch_points=0, seed=0):
        L = _native.load()
        st = ctypes.c_int(0)
        h = L.vd_server_new(int(pool_bytes), int(slots), int(max_batch_points), int(seed), ctypes.byref(st))
        if not h or st.value != _native.VD_OK:
            raise VDError(st.value or 3, "vd_server_new")
        self._h = ctypes.c_void_p(h)

    def submit(self, points):
        p = _points(points)
        i = ctypes.c_int64(0)
        _check(_native.load().vd_server_submit(self._h, p.shape[1], _dp(p), p.shape[0], ctypes.byref(i)), "submit")
        return i.value

    def poll(self, timeout_ms=0, cap=4096):
        ids = np.zeros(cap, dtype=np.int64)
        n = ctypes.c_int64(0)
        _check(_native.load().vd_server_poll(self._h, ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), cap,
                                             ctypes.byref(n), int(timeout_ms)), "poll")
        return ids[: n.value].tolist()

    def result(self, rid):
        L = _native.load()
        m = ctypes.c_int64(0)
        st = ctypes.c_int(0)
        _check(L.vd_server_result(self._h, rid, None, 0, ctypes.byref(m), ctypes.byref(st)), "result")
        uv = np.zeros((m.value, 2), dtype=np.uint32)
        _check(L.vd_server_result(self._h, rid, uv.ctypes.data_as(ctypes.c_void_p), m.value, ctypes.byref(m),
                                  ctypes.byref(st)), "result")
        if st.value != _native.VD_OK:
            raise VDError(st.value, f"request {rid}")
        return uv.astype(np.int64)

    def stats(self):
        out = np.zeros(8, dtype=np.int64)
        _check(_native.load().vd_server_stats(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))), "stats")
        keys = ("submitted", "finished", "batches", "bytes_in_flight", "peak_bytes_in_flight", "queued",
                "isolated", "budget")
        return dict(zip(keys, out.tolist()))

    def close(self):
        if getattr(self, "_h", None):
            _native.load().vd_server_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
