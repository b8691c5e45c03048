"""The allocation-free BFS entry point (gg_bfs_noalloc) against gg_bfs.

gg_bfs_noalloc serves callers that cannot allocate device memory while they run
(for example code living inside another framework's pre-sized memory pool, or a
real-time loop that cannot afford an allocation stall); it keeps its scratch in
a static device array.  This test calls it through the C ABI with device
buffers, twice in a row (the second call must not see the first call's
leftovers), and compares each result with the regular entry point's.  The file
sorts last so that a run stopping at the first failure has already run every
other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bfs_noalloc_matches_gg_bfs_twice():
    import torch

    from easy_graphit_gb300 import GraphT, HostGraph, bfs
    from easy_graphit_gb300 import _lib as L

    dev = torch.device("cuda", 0)
    hg = HostGraph.rmat(16, 16, symmetrize=True)
    off = torch.from_numpy(np.array(hg.offsets)).to(dev)
    dst = torch.from_numpy(np.array(hg.dst)).to(dev)
    V, E = hg.num_vertices, hg.num_edges
    g = GraphT(hg, symmetric=True)
    deg = np.diff(hg.offsets)
    sources = [int(np.argmax(deg)), int(np.nonzero(deg)[0][7])]
    stream = torch.cuda.current_stream(dev)
    wants = [bfs(g, src)[0] for src in sources]  # the regular entry point (which allocates)
    import oracle
    np.testing.assert_array_equal(wants[0], oracle.bfs(np.array(hg.offsets), np.array(hg.dst), sources[0]))
    outs = [torch.full((V,), 123, dtype=torch.int32, device=dev) for _ in sources]

    def call(src, out):
        st = L.lib().gg_bfs_noalloc(C.c_void_p(off.data_ptr()), C.c_void_p(dst.data_ptr()), V, E, src,
                                    C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert st == L.GG_OK, L.last_error()

    call(sources[0], outs[0])  # set-up: looks up the scratch array's address
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(dev)[0]
    for src, out, want in zip(sources, outs, wants):  # two calls in a row, different sources
        call(src, out)
        np.testing.assert_array_equal(out.cpu().numpy(), want)  # BFS depths: exact
    torch.cuda.synchronize()
    # nothing was allocated on the device by those calls
    assert torch.cuda.mem_get_info(dev)[0] == free_before
    g.close()


def test_bfs_noalloc_rejects_oversized_graphs():
    from easy_graphit_gb300 import _lib as L

    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    st = L.lib().gg_bfs_noalloc(dummy, dummy, (1 << 20) + 1, 10, 0, dummy, None)
    assert st == L.GG_ERR_INVALID
    assert "1048576" in L.last_error()
