"""Batched mode parity: every source's result equals the oracle's single-source
result (bit-exact), for BFS (bit-parallel, 64 sources per pass) and SSSP
(32 sources per pass, per-source delta-stepping)."""
import numpy as np
import pytest

import oracle
from easy_graphit_gb300 import GraphT, HostGraph, bfs_batch, sssp_batch

pytestmark = pytest.mark.gpu

INT_MAX = 2**31 - 1
_G = {}


def graph(kind):
    if kind not in _G:
        if kind == "dir14":
            hg = HostGraph.rmat(14, 16)
        elif kind == "sym14":
            hg = HostGraph.rmat(14, 16, symmetrize=True)
        elif kind == "grid":
            hg = HostGraph.grid(40, 70)
        elif kind == "dir17":
            hg = HostGraph.rmat(17, 16)
        sym = kind.startswith("sym") or kind == "grid"
        _G[kind] = (hg, GraphT(hg, symmetric=sym),
                    (np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)))
    return _G[kind]


@pytest.mark.parametrize("kind", ["dir14", "sym14", "grid"])
@pytest.mark.parametrize("nsrc", [1, 5, 64, 100])
def test_bfs_batch(kind, nsrc):
    hg, g, (off, dst, _) = graph(kind)
    srcs = hg.pick_sources(nsrc, seed=11)
    depth, st = bfs_batch(g, srcs)
    for i, s in enumerate(srcs):
        np.testing.assert_array_equal(depth[i], oracle.bfs(off, dst, int(s)), err_msg=f"source {s}")


def test_bfs_batch_duplicate_sources():
    hg, g, (off, dst, _) = graph("sym14")
    s = int(hg.pick_sources(1)[0])
    depth, _ = bfs_batch(g, [s, s, s])
    ref = oracle.bfs(off, dst, s)
    for i in range(3):
        np.testing.assert_array_equal(depth[i], ref)


@pytest.mark.parametrize("kind", ["dir14", "sym14", "grid"])
@pytest.mark.parametrize("delta", [1, 8, 32, 128])
@pytest.mark.parametrize("nsrc", [3, 32, 40])
def test_sssp_batch(kind, delta, nsrc):
    hg, g, (off, dst, w) = graph(kind)
    srcs = hg.pick_sources(nsrc, seed=5)
    dist, st = sssp_batch(g, srcs, delta)
    for i, s in enumerate(srcs):
        np.testing.assert_array_equal(dist[i], oracle.sssp_dijkstra(off, dst, w, int(s)),
                                      err_msg=f"source {s} delta {delta}")


def test_sssp_batch_larger_graph_device_output():
    import torch
    hg, g, (off, dst, w) = graph("dir17")
    srcs = hg.pick_sources(32)
    out = torch.empty((32, hg.num_vertices), dtype=torch.int32, device="cuda")
    sssp_batch(g, srcs, 32, out=out)
    got = out.cpu().numpy()
    for i in [0, 7, 31]:
        np.testing.assert_array_equal(got[i], oracle.sssp_dijkstra(off, dst, w, int(srcs[i])))
