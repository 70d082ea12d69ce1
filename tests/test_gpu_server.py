"""GPU: the continuous-batching server.

Each request's result in the mix must be bit-identical to the same points
triangulated alone; admission keeps the estimated bytes in flight within the
budget; a failing request does not take its batch down.
"""
import time
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def alone(vd, p):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t = vd.delaunay(p)
    e = t.edges()
    t.close()
    return e


def drain(srv, ids, timeout=120.0):
    got = {}
    t0 = time.time()
    while len(got) < len(ids) and time.time() - t0 < timeout:
        for i in srv.poll(timeout_ms=100):
            got[i] = True
    assert len(got) == len(ids)


def test_mixed_stream_same_as_alone(vd):
    reqs = W.c5_requests(48, lo=100, hi=20_000, seed=12345)
    srv = vd.Server(pool_bytes=8 << 30, slots=3, max_batch_points=60_000)
    ids, pts = [], []
    for k, r in enumerate(reqs):  # arrivals in bursts while batches run
        p = W.c5_points(r)
        pts.append(p)
        ids.append(srv.submit(p))
        if k % 8 == 7:
            time.sleep(0.01)
    drain(srv, ids)
    st = srv.stats()
    assert st["finished"] == len(reqs) and st["batches"] >= 2
    for i, p in zip(ids, pts):
        assert np.array_equal(srv.result(i), alone(vd, p))
    srv.close()


def test_admission_respects_budget(vd):
    reqs = W.c5_requests(24, lo=1000, hi=5000, seed=777)
    budget = 3 * 1850 * 5000  # room for about three of the largest 3D requests
    srv = vd.Server(pool_bytes=budget, slots=4)
    ids = [srv.submit(W.c5_points(r)) for r in reqs]
    drain(srv, ids)
    st = srv.stats()
    assert 0 < st["peak_bytes_in_flight"] <= budget
    assert st["bytes_in_flight"] == 0
    for i, r in zip(ids, reqs):
        assert np.array_equal(srv.result(i), alone(vd, W.c5_points(r)))
    srv.close()


def test_failing_request_is_isolated(vd):
    srv = vd.Server(pool_bytes=1 << 30, slots=1)
    good = [np.random.default_rng(k).random((300 + 50 * k, 3)) for k in range(3)]
    bad = np.full((10, 3), 0.5)  # all points equal: degenerate super simplex
    huge = np.random.default_rng(9).random((10, 2))
    ids = [srv.submit(good[0]), srv.submit(bad), srv.submit(good[1]), srv.submit(good[2])]
    drain(srv, ids)
    assert np.array_equal(srv.result(ids[0]), alone(vd, good[0]))
    with pytest.raises(vd.VDError):
        srv.result(ids[1])
    assert np.array_equal(srv.result(ids[2]), alone(vd, good[1]))
    assert np.array_equal(srv.result(ids[3]), alone(vd, good[2]))
    srv.close()
    small = vd.Server(pool_bytes=1000, slots=1)  # below any request's estimate
    i = small.submit(huge)
    drain(small, [i])
    with pytest.raises(vd.VDError):
        small.result(i)
    small.close()
