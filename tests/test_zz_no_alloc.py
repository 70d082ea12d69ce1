"""GPU: the allocation-free edge extraction (vd_edges_from_simplices_noalloc).

Callers that may not allocate device memory -- an application whose memory
manager owns the GPU, or a loop that cannot take the synchronisation of a
cudaMalloc -- hand this entry point their simplices and an output buffer;
its scratch is a static device array.  The test exports the simplices of a
tree built by the library, runs the entry point twice in a row on them and
checks that each output equals the tree's own edge list (vd_edges), exactly.
This file is collected last so that a run stopping at its first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _noalloc(L, dim, simp_dev, ns, nverts, out_dev, cap):
    import torch
    m = ctypes.c_int64(-1)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.vd_edges_from_simplices_noalloc(dim, ctypes.c_void_p(simp_dev.data_ptr() if ns else 0), ns, nverts,
                                           ctypes.c_void_p(out_dev.data_ptr()), cap, ctypes.byref(m),
                                           ctypes.c_void_p(stream))
    return rc, m.value


@pytest.mark.parametrize("dim,n", [(3, 4000), (2, 6000)])
def test_noalloc_edges_match_tree_edges_twice(vd, dim, n):
    import torch
    from voronoids_gb300 import _native
    L = _native.load()
    p = W.uniform_points(n, dim, 7100 + dim)
    t = vd.delaunay(p, seed=3)
    want = t.edges()
    verts, _ = t.simplices()
    simp = torch.from_numpy(np.ascontiguousarray(verts, dtype=np.int32)).cuda()
    cap = 8 * n
    for call in range(2):
        out = torch.full((2 * cap,), -7, dtype=torch.int32, device="cuda")
        rc, m = _noalloc(L, dim, simp, verts.shape[0], n, out, cap)
        assert rc == 0, (call, rc)
        got = out[: 2 * m].view(-1, 2).cpu().numpy().astype(np.int64)
        assert m == len(want)
        assert np.array_equal(got, want), call


def test_noalloc_rejects_sizes_beyond_its_scratch(vd):
    import torch
    from voronoids_gb300 import _native
    L = _native.load()
    dummy = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc, _ = _noalloc(L, 3, dummy, 131072 + 1, 10, dummy, 4)
    assert rc == 1  # VD_ERR_ARG: more simplices than the static scratch holds
    rc, _ = _noalloc(L, 3, dummy, 1, 65536 + 1, dummy, 4)
    assert rc == 1  # VD_ERR_ARG: vertex ids beyond the static scratch


def test_noalloc_long_bucket_fan_matches_numpy(vd):
    """Vertex 0 in 1,500 tetrahedra: its bucket (4,500 entries, most of them
    repeated edges) is longer than one warp sorts, so the block-per-bucket
    path runs; the result must equal np.unique of the same edges."""
    import torch
    from voronoids_gb300 import _native
    L = _native.load()
    k = 1500
    i = np.arange(1, k + 1)
    tets = np.stack([np.zeros(k, np.int64), i, i + 1, i + 2], axis=1)
    nverts = k + 3
    pairs = np.concatenate([np.sort(tets[:, [a, b]], axis=1) for a in range(4) for b in range(a + 1, 4)])
    want = np.unique(pairs, axis=0)
    simp = torch.from_numpy(tets.astype(np.int32)).cuda()
    cap = len(pairs)
    for call in range(2):
        out = torch.full((2 * cap,), -1, dtype=torch.int32, device="cuda")
        rc, m = _noalloc(L, 3, simp, k, nverts, out, cap)
        assert rc == 0, (call, rc)
        got = out[: 2 * m].view(-1, 2).cpu().numpy().astype(np.int64)
        assert np.array_equal(got, want), call


def test_noalloc_reports_bad_ids_and_short_output(vd):
    import torch
    from voronoids_gb300 import _native
    L = _native.load()
    tets = np.array([[0, 1, 2, 3], [1, 2, 3, 4]], dtype=np.int32)
    simp = torch.from_numpy(tets).cuda()
    out = torch.zeros(64, dtype=torch.int32, device="cuda")
    rc, m = _noalloc(L, 3, simp, 2, 5, out, 32)
    assert rc == 0 and m == 9
    rc, m = _noalloc(L, 3, simp, 2, 5, out, 4)
    assert rc == 1 and m == 9  # VD_ERR_ARG: output too short; the count is still reported
    rc, m = _noalloc(L, 3, simp, 2, 4, out, 32)
    assert rc == 1  # VD_ERR_ARG: vertex id 4 is not below nverts = 4
    rc, m = _noalloc(L, 3, simp, 2, 5, out, 32)
    assert rc == 0 and m == 9  # a good call after the rejected ones
