"""GPU: the two forms of the conflict-test kernels (exact tier on expansions
alone, or an integer evaluation first) and the automatic switch between
them give the same triangulation: bit-identical edges against the oracle,
validator clean, on inputs that reach the exact tier often."""
import warnings

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def build(vd, p, seed, mode, switch_after=32):
    t = vd.DelaunayTree(p)
    t.set_exact_tier(mode, switch_after)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t.add_points_to_tree(p, seed=seed)
    return t


@pytest.mark.parametrize("mode,switch_after", [(1, 0), (2, 0), (0, 0), (0, 32), (0, 5000)])
def test_exact_tier_forms_match_oracle(vd, oracle, mode, switch_after):
    p = W.c3_points(n=30000)
    t = build(vd, p, 11, mode, switch_after)
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    assert t.stats()["pred_exact"] > 0  # the input does reach the exact tier
    assert np.array_equal(t.edges(), oracle.Triangulation(p, seed=11).edges())


@pytest.mark.parametrize("dim", [2, 3])
def test_exact_tier_lattice(vd, oracle, dim):
    # exact ties everywhere: every cospherical decision goes to the perturbation
    p = W.lattice_points(12 if dim == 3 else 40, dim)
    ref = oracle.Triangulation(p, seed=6).edges()
    for mode in (1, 2):
        t = build(vd, p, 6, mode)
        assert t.check_delaunay()
        assert np.array_equal(t.edges(), ref), mode


def test_exact_tier_arg_errors(vd):
    t = vd.DelaunayTree(W.uniform_points(100, 3, 1))
    with pytest.raises(vd.VDError):
        t.set_exact_tier(3)
    with pytest.raises(vd.VDError):
        t.set_exact_tier(0, -1)


@pytest.mark.parametrize("small_rounds", [0, 1 << 30])
def test_large_regions_block_search(vd, oracle, small_rounds):
    """Near-degenerate points whose conflict regions outgrow a warp's shared
    memory: the searches are redone in the pool, by a whole block
    (k_cavity_big) in the default path and by the warp inside the
    cooperative small-round kernel.  Same edges as the oracle either way."""
    p = W.c3_points(n=60000)
    t = vd.DelaunayTree(p)
    t.set_small_rounds(small_rounds)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        t.add_points_to_tree(p, seed=5)
    st = t.stats()
    assert st["spilled"] > 0 and st["max_cavity"] > 128
    ok, det = t.check_delaunay(details=True)
    assert ok, det
    assert np.array_equal(t.edges(), oracle.Triangulation(p, seed=5).edges())
