"""GPU: batched build of many independent point sets in one pass of rounds.

Parity bar: every set's sorted edge list is bit-identical to the single-set
build of that set alone (and to the oracle where the oracle is run), and the
exact validator passes on the whole batched tree.
"""
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def single(vd, p, seed):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t = vd.delaunay(p, seed=seed)
    e = t.edges()
    t.close()
    return e


def sets_of(sizes, dim, seed):
    return [W.uniform_points(int(n), dim, seed + 17 * i) for i, n in enumerate(sizes)]


@pytest.mark.parametrize("dim", [2, 3])
def test_batch_matches_oracle_and_single(vd, oracle, dim):
    sizes = [2, 3, 4, 5, 9, 40, 333, 1200, 2500, 7, 64]
    sets = sets_of(sizes, dim, 500 + dim)
    got = vd.delaunay_batch(sets, seed=11)
    assert len(got) == len(sets)
    for p, e in zip(sets, got):
        o = oracle.Triangulation(p, seed=11)
        assert np.array_equal(e, o.edges())
        assert np.array_equal(e, single(vd, p, 11))


def test_batch_c4_shaped_sample(vd):
    # log-uniform sizes 32..65536, uniform [0,1)^3: the batched-build workload
    sizes = W.c4_sizes(48, seed=W.config_seed(4) + 1)
    sets = sets_of(sizes, 3, 900)
    t = vd.DelaunayTree.create(3)
    got = vd.delaunay_batch(sets, seed=5, tree=t)
    assert t.num_sets() == len(sets)
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    assert t.num_vertices == int(np.sum(sizes))
    t.close()
    for p, e in zip(sets, got):
        assert np.array_equal(e, single(vd, p, 5))


def test_batch_order_and_seed_independent(vd):
    sets = sets_of([800, 50, 3000, 12], 3, 77)
    a = vd.delaunay_batch(sets, seed=1)
    b = vd.delaunay_batch(sets[::-1], seed=99)[::-1]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_batch_duplicates_and_lattice(vd):
    rng = np.random.default_rng(3)
    p = rng.random((400, 3))
    p[10] = p[20]  # one duplicate inside the set
    lat = W.lattice_points(6, 3)  # exact cospherical configurations
    sets = [p, lat, rng.random((100, 3))]
    got = vd.delaunay_batch(sets, seed=2)
    for s, e in zip(sets, got):
        assert np.array_equal(e, single(vd, s, 2))


def test_batch_device_entry(vd):
    torch = pytest.importorskip("torch")
    sets = sets_of([700, 30, 1500], 3, 41)
    pts = np.concatenate(sets)
    off = np.concatenate([[0], np.cumsum([len(s) for s in sets])])
    d = torch.from_numpy(pts).cuda()
    cap = 16 * len(pts)
    out = torch.zeros((cap, 2), dtype=torch.int32, device="cuda")
    t = vd.DelaunayTree.create(3)
    eoff = t.batch_device(d.data_ptr(), off, 4, out.data_ptr(), cap)
    torch.cuda.synchronize()
    uv = out[: int(eoff[-1])].cpu().numpy().astype(np.int64)
    for s, p in enumerate(sets):
        assert np.array_equal(uv[eoff[s]:eoff[s + 1]], single(vd, p, 4))
    # the same handle then serves a single-set build
    t.close()


def test_batch_tree_reuse_switches_modes(vd):
    t = vd.DelaunayTree.create(2)
    a = sets_of([300, 20], 2, 5)
    r1 = vd.delaunay_batch(a, seed=3, tree=t)
    b = sets_of([50, 600, 7], 2, 9)
    r2 = vd.delaunay_batch(b, seed=3, tree=t)
    for p, e in zip(a, r1):
        assert np.array_equal(e, single(vd, p, 3))
    for p, e in zip(b, r2):
        assert np.array_equal(e, single(vd, p, 3))
    t.close()


def test_batch_errors_are_statuses(vd):
    with pytest.raises(vd.VDError):
        t = vd.DelaunayTree.create(3)
        t.batch(np.zeros((4, 3)), [0, 2, 2, 4])  # an empty set
    bad = np.random.default_rng(0).random((10, 3))
    bad[4, 1] = np.nan
    with pytest.raises(vd.VDError):
        vd.delaunay_batch([bad[:5], bad[5:]])
    with pytest.raises(vd.VDError):
        t = vd.DelaunayTree.create(3)
        t.add_points_to_tree(np.random.default_rng(1).random((10, 3)))  # no super simplex yet


def test_autotuned_batch_same_result(vd):
    torch = pytest.importorskip("torch")
    sizes = W.c4_sizes(40, seed=W.config_seed(4) + 7)
    sets = sets_of(sizes, 3, 1300)
    pts = np.concatenate(sets)
    off = np.concatenate([[0], np.cumsum(sizes)])
    d = torch.from_numpy(pts).cuda()
    t = vd.DelaunayTree.create(3)
    cfg = t.autotune_batch(d.data_ptr(), off, sample_points=60_000)
    assert 4 <= cfg["warps_per_sm"] <= 32 and cfg["passes"] in (1, 2, 3) and cfg["sample_sets"] >= 1
    uv, eoff = t.batch(pts, off, seed=8)
    for s, p in enumerate(sets):
        assert np.array_equal(uv[eoff[s]:eoff[s + 1]].astype(np.int64), single(vd, p, 8))
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    t.close()
