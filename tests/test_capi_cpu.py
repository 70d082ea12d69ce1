"""CPU: the C-ABI library loads, exports every symbol include/*.h declares,
and its host-only entry points behave (no device compute is called)."""
import ctypes
import glob
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(vd_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    from voronoids_gb300 import _native
    L = _native.load()
    declared = _declared()
    assert len(declared) >= 20
    missing = [s for s in sorted(declared) if not hasattr(L, s)]
    assert not missing, missing
    assert set(_native.EXPORTS) == declared


def test_status_strings():
    from voronoids_gb300 import _native
    L = _native.load()
    for code in _native.STATUS:
        assert L.vd_status_str(code).decode()
    assert L.vd_status_str(4).decode() == "duplicate points were skipped"


def test_super_simplex_matches_oracle(oracle):
    from voronoids_gb300 import _native
    L = _native.load()
    rng = np.random.default_rng(1)
    dp = ctypes.POINTER(ctypes.c_double)
    for dim in (2, 3):
        for n in (2, 7, 1000):
            p = np.ascontiguousarray(rng.random((n, dim)) * 3 - 1)
            out = np.zeros(12)
            r = ctypes.c_double()
            assert L.vd_super_simplex(dim, p.ctypes.data_as(dp), n, out.ctypes.data_as(dp), ctypes.byref(r)) == 0
            sv, R = oracle.super_vertices(p)
            assert r.value == R
            assert np.array_equal(out[: 3 * (dim + 1)].reshape(dim + 1, 3), sv)


def test_bad_arguments_are_rejected_on_host():
    from voronoids_gb300 import _native
    L = _native.load()
    dp = ctypes.POINTER(ctypes.c_double)
    p = np.zeros((3, 4))
    st = ctypes.c_int(-1)
    h = L.vd_tree_new(4, p.ctypes.data_as(dp), 3, ctypes.byref(st))
    assert st.value == 1  # VD_ERR_ARG, decided before any device call
    L.vd_tree_free(h)
    q = np.array([[0.0, np.nan]])
    out = np.zeros(12)
    r = ctypes.c_double()
    assert L.vd_super_simplex(2, q.ctypes.data_as(dp), 1, out.ctypes.data_as(dp), ctypes.byref(r)) == 5
    assert L.vd_insert_points(None, p.ctypes.data_as(dp), 3, 0) == 1


def test_profile_kernel_names():
    """The per-kernel profile slots have unique names, the round's kernels
    among them, and the roofline kernels' committed ncu summaries carry a
    traffic figure the bench can read."""
    import bench
    from voronoids_gb300 import _native
    L = _native.load()
    names = []
    i = 0
    while True:
        nm = L.vd_profile_name(i)
        if not nm:
            break
        names.append(nm.decode())
        i += 1
    assert len(names) == len(set(names))
    for k in ("k_pick", "k_thin", "k_cavity", "k_check", "k_reclaim", "k_relocate", "k_activate", "k_decide",
              "k_cavity_big", "k_commit_big", "edges"):
        assert k in names
    for k in ("k_cavity", "k_check", "k_decide"):
        t = bench.profile_traffic(k)
        assert t is not None and t > 1e6
