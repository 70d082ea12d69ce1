"""CPU: the device predicate tiers (host build of vd_predicates.cuh) against
the oracle's independent big-integer predicates, including exact ties
resolved by the symbolic perturbation."""
import ctypes

import numpy as np
import pytest

dp = ctypes.POINTER(ctypes.c_double)
ip = ctypes.POINTER(ctypes.c_int)


@pytest.fixture(scope="module")
def host():
    from voronoids_gb300 import build as B
    H = ctypes.CDLL(B.build_host())
    H.vdh_in_conflict.argtypes = [ctypes.c_int, dp, ip, ip, ip]
    H.vdh_insphere_exact.argtypes = [ctypes.c_int, dp, ip, ctypes.c_int, ip]
    H.vdh_insphere_exact_expansion.argtypes = [ctypes.c_int, dp, ip, ctypes.c_int, ip]
    H.vdh_orient_exact.argtypes = [ctypes.c_int, dp, ip]
    H.vdh_exit_face.argtypes = [ctypes.c_int, dp, ctypes.c_uint, ctypes.c_int, ip]
    return H


def _pad(pts, dim):
    p = np.zeros((len(pts), 3))
    p[:, :dim] = pts
    return np.ascontiguousarray(p)


def _tuples(rng, dim, kind):
    if kind == 0:
        return rng.random((dim + 2, dim))
    if kind == 1:  # coarse lattice: many exact zeros
        return np.round(rng.random((dim + 2, dim)) * 4) / 4
    if kind == 2:  # query within 1e-13 of a vertex
        p = rng.random((dim + 2, dim))
        p[-1] = p[0] + (rng.random(dim) - 0.5) * 1e-13
        return p
    return np.round(rng.random((dim + 2, dim)) * 8) / 8 + rng.choice([0, 1e-12, -1e-12], size=(dim + 2, dim))


@pytest.mark.parametrize("dim", [2, 3])
def test_conflict_matches_oracle(host, oracle, dim):
    rng = np.random.default_rng(100 + dim)
    tiers = [0, 0, 0]
    checked = 0
    for trial in range(6000):
        pts = _tuples(rng, dim, trial % 4)
        s = pts[: dim + 1]
        o = oracle.orient(s)
        if o == 0:
            continue
        if o < 0:
            s = s[[1, 0] + list(range(2, dim + 1))]
        pts = np.vstack([s, pts[dim + 1:]])
        keys = np.ascontiguousarray(rng.permutation(64)[: dim + 2], dtype=np.int32)
        P = _pad(pts, dim)
        tier, err = ctypes.c_int(), ctypes.c_int()
        g = host.vdh_in_conflict(dim, P.ctypes.data_as(dp), keys.ctypes.data_as(ip), ctypes.byref(tier),
                                 ctypes.byref(err))
        gx = host.vdh_insphere_exact(dim, P.ctypes.data_as(dp), keys.ctypes.data_as(ip), 1, ctypes.byref(err))
        want = oracle.insphere_sos(pts[: dim + 1], pts[dim + 1], keys)
        assert err.value == 0
        assert g == want and gx == want, (pts.tolist(), keys.tolist())
        tiers[tier.value] += 1
        checked += 1
    assert checked > 5000
    assert all(t > 0 for t in tiers), tiers  # every tier exercised


@pytest.mark.parametrize("dim", [2, 3])
def test_unperturbed_exact_sign(host, oracle, dim):
    rng = np.random.default_rng(7 + dim)
    for trial in range(2000):
        pts = _tuples(rng, dim, 1 + trial % 3)
        if oracle.orient(pts[: dim + 1]) == 0:
            continue
        keys = np.zeros(dim + 2, dtype=np.int32)
        P = _pad(pts, dim)
        err = ctypes.c_int()
        g = host.vdh_insphere_exact(dim, P.ctypes.data_as(dp), keys.ctypes.data_as(ip), 0, ctypes.byref(err))
        assert g == oracle.insphere_exact(pts[: dim + 1], pts[dim + 1])


@pytest.mark.parametrize("dim", [2, 3])
def test_orient_exact(host, oracle, dim):
    rng = np.random.default_rng(17 + dim)
    for trial in range(3000):
        pts = np.round(rng.random((dim + 1, dim)) * 4) / 4 if trial % 2 else rng.random((dim + 1, dim))
        P = _pad(pts, dim)
        err = ctypes.c_int()
        assert host.vdh_orient_exact(dim, P.ctypes.data_as(dp), ctypes.byref(err)) == oracle.orient(pts)


def test_exit_face_convention(host):
    # positive 3D simplex (b, a, c, d) of the unit corner; a point beyond face 2
    v = np.array([[1, 0, 0], [0, 0, 0], [0, 1, 0], [0, 0, 1], [0.2, -0.5, 0.2]], dtype=np.float64)
    err = ctypes.c_int()
    f = host.vdh_exit_face(3, np.ascontiguousarray(v).ctypes.data_as(dp), 0xF, 0, ctypes.byref(err))
    assert f == 2  # the face opposite vertex (0,1,0)
    inside = v.copy()
    inside[4] = [0.1, 0.1, 0.1]
    assert host.vdh_exit_face(3, np.ascontiguousarray(inside).ctypes.data_as(dp), 0xF, 1, ctypes.byref(err)) == -1
    onface = v.copy()
    onface[4] = [0.1, 0.0, 0.1]
    assert host.vdh_exit_face(3, np.ascontiguousarray(onface).ctypes.data_as(dp), 0xF, 0, ctypes.byref(err)) == -1
    assert host.vdh_exit_face(3, np.ascontiguousarray(onface).ctypes.data_as(dp), 0xF, 1, ctypes.byref(err)) == 2


def _hl(host):
    host.vdh_in_conflict_hl.argtypes = [ctypes.c_int, dp, ip, ip, ip]
    host.vdh_insphere_hl.argtypes = [ctypes.c_int, dp]
    host.vdh_exit_face_hl.argtypes = [ctypes.c_int, dp, ctypes.c_uint, ctypes.c_int, ip]
    return host


def _hl_tuples(rng, dim, kind):
    if kind < 4:
        return _tuples(rng, dim, kind)
    if kind == 4:  # differences ~1e-6 on coordinates ~0.5: the split's absolute error matters
        return 0.5 + (rng.random((dim + 2, dim)) - 0.5) * 1e-6
    return rng.random((dim + 2, dim)) * 1000 + 1e5  # far from the origin


@pytest.mark.parametrize("dim", [2, 3])
def test_split_tier_is_sound(host, oracle, dim):
    """The f32 tier on hi/lo split coordinates never certifies a wrong sign,
    and the full tiered test agrees with the oracle."""
    H = _hl(host)
    rng = np.random.default_rng(300 + dim)
    certified = 0
    total = 0
    for trial in range(6000):
        pts = _hl_tuples(rng, dim, trial % 6)
        s = pts[: dim + 1]
        o = oracle.orient(s)
        if o == 0:
            continue
        if o < 0:
            s = s[[1, 0] + list(range(2, dim + 1))]
        pts = np.vstack([s, pts[dim + 1:]])
        keys = np.ascontiguousarray(rng.permutation(64)[: dim + 2], dtype=np.int32)
        P = _pad(pts, dim)
        f = H.vdh_insphere_hl(dim, P.ctypes.data_as(dp))
        total += 1
        if f != 0:
            certified += 1
            assert f == oracle.insphere_exact(pts[: dim + 1], pts[dim + 1]), pts.tolist()
        tier, err = ctypes.c_int(), ctypes.c_int()
        g = H.vdh_in_conflict_hl(dim, P.ctypes.data_as(dp), keys.ctypes.data_as(ip), ctypes.byref(tier),
                                 ctypes.byref(err))
        assert g == oracle.insphere_sos(pts[: dim + 1], pts[dim + 1], keys)
    assert certified > total // 2


@pytest.mark.parametrize("dim", [2, 3])
def test_split_tier_near_sphere(host, oracle, dim):
    """Queries a relative 1e-9 .. 1e-2 off the circumsphere, at coordinate
    scales 2^-10 .. 2^8: the first (cheap, permanent-free) bound of the
    split tier and the tight one both certify only correct signs."""
    H = _hl(host)
    rng = np.random.default_rng(500 + dim)
    certified = checked = 0
    for trial in range(6000):
        scale = 2.0 ** rng.uniform(-10, 8)
        s = rng.random((dim + 1, dim)) * scale
        o = oracle.orient(s)
        if o == 0:
            continue
        if o < 0:
            s = s[[1, 0] + list(range(2, dim + 1))]
        # circumcentre c (least squares on the bisector system) and radius r
        A = 2 * (s[1:] - s[0])
        b = (s[1:] ** 2).sum(1) - (s[0] ** 2).sum()
        c = np.linalg.solve(A, b)
        r = np.linalg.norm(s[0] - c)
        u = rng.normal(size=dim)
        u /= np.linalg.norm(u)
        eps = 10.0 ** rng.uniform(-9, -2) * rng.choice([-1.0, 1.0])
        q = c + u * r * (1 + eps)
        pts = np.vstack([s, q[None, :]])
        f = H.vdh_insphere_hl(dim, _pad(pts, dim).ctypes.data_as(dp))
        checked += 1
        if f != 0:
            certified += 1
            assert f == oracle.insphere_exact(pts[: dim + 1], pts[dim + 1]), (scale, eps, pts.tolist())
    assert checked > 5000 and certified > checked // 3


@pytest.mark.parametrize("dim", [2, 3])
def test_split_exit_face(host, oracle, dim):
    H = _hl(host)
    rng = np.random.default_rng(400 + dim)
    for trial in range(3000):
        pts = _hl_tuples(rng, dim, [0, 1, 4, 5][trial % 4])
        s = pts[: dim + 1]
        o = oracle.orient(s)
        if o == 0:
            continue
        if o < 0:
            s = s[[1, 0] + list(range(2, dim + 1))]
        pts = np.vstack([s, pts[dim + 1:]])
        P = _pad(pts, dim)
        err = ctypes.c_int()
        for strict in (0, 1):
            got = H.vdh_exit_face_hl(dim, P.ctypes.data_as(dp), (1 << (dim + 1)) - 1, strict, ctypes.byref(err))
            want = -1
            for j in range(dim + 1):
                q = pts[: dim + 1].copy()
                q[j] = pts[dim + 1]
                sg = oracle.orient(q)
                if sg < 0 or (strict and sg == 0):
                    want = j
                    break
            assert got == want


@pytest.mark.parametrize("dim", [2, 3])
def test_exact_tier_integer_and_expansion_paths(host, oracle, dim):
    # The exact tier works on integers when every coordinate is a multiple of
    # a common power of two within 126 bits, and on floating-point expansions
    # otherwise.  Near-cospherical lattices, exact ties (perturbation), small
    # and huge coordinates mixed (beyond the integer budget) all against the
    # oracle's big integers.
    rng = np.random.default_rng(900 + dim)
    checked = 0
    for trial in range(4000):
        kind = trial % 5
        if kind == 0:  # jittered lattice (near-degenerate, integer path)
            pts = np.round(rng.random((dim + 2, dim)) * 64) / 64 + rng.uniform(-1e-12, 1e-12, (dim + 2, dim))
        elif kind == 1:  # exact lattice (ties: perturbation on exact minors)
            pts = np.round(rng.random((dim + 2, dim)) * 6) / 6
        elif kind == 2:  # super-simplex scale next to unit-cube points
            pts = rng.random((dim + 2, dim))
            pts[0] = pts[0] * 40 - 20
        elif kind == 3:  # exponents spread wider than 126 bits: expansion path
            pts = rng.random((dim + 2, dim))
            pts[1, 0] = 1e-30 + pts[1, 0] * 1e-31
            pts[2, 0] = 3.0e9
        else:  # tiny query offsets from a vertex
            pts = rng.random((dim + 2, dim))
            pts[-1] = pts[1] + rng.uniform(-1e-14, 1e-14, dim)
        s = pts[: dim + 1]
        o = oracle.orient(s)
        if o == 0:
            continue
        if o < 0:
            s = s[[1, 0] + list(range(2, dim + 1))]
        pts = np.vstack([s, pts[dim + 1:]])
        keys = np.ascontiguousarray(rng.permutation(64)[: dim + 2], dtype=np.int32)
        P = _pad(pts, dim)
        err = ctypes.c_int()
        want_g = oracle.insphere_sos(pts[: dim + 1], pts[dim + 1], keys)
        want_u = oracle.insphere_exact(pts[: dim + 1], pts[dim + 1])
        for fn in (host.vdh_insphere_exact, host.vdh_insphere_exact_expansion):
            g = fn(dim, P.ctypes.data_as(dp), keys.ctypes.data_as(ip), 1, ctypes.byref(err))
            u = fn(dim, P.ctypes.data_as(dp), keys.ctypes.data_as(ip), 0, ctypes.byref(err))
            assert err.value == 0
            assert g == want_g, (fn.__name__, kind, pts.tolist(), keys.tolist())
            assert u == want_u, (fn.__name__, kind, pts.tolist())
        checked += 1
    assert checked > 3500
