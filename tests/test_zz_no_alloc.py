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
