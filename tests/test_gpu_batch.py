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


# ------------------------------------------------ multi-source / multi-graph
def test_multi_source_equals_min_over_sources():
    from easy_graphit_gb300 import bfs_multi, sssp_multi
    hg, g, (off, dst, w) = graph("dir14")
    srcs = hg.pick_sources(7, seed=3)
    depth, _ = bfs_multi(g, srcs)
    bref = np.stack([oracle.bfs(off, dst, int(s)) for s in srcs]).astype(np.int64)
    bref[bref < 0] = 2**40
    bmin = bref.min(axis=0)
    bmin[bmin == 2**40] = -1
    np.testing.assert_array_equal(depth, bmin)
    for delta in (1, 32):
        dist, _ = sssp_multi(g, srcs, delta)
        sref = np.stack([oracle.sssp_dijkstra(off, dst, w, int(s)) for s in srcs]).min(axis=0)
        np.testing.assert_array_equal(dist, sref)


@pytest.mark.parametrize("app", ["bfs", "sssp"])
def test_multigraph_batch_uneven_graphs(app):
    from easy_graphit_gb300 import multigraph_batch
    rng = np.random.default_rng(27491095)
    parts = []
    for i in range(10):
        if i % 3 == 2:
            n = int(rng.integers(8, 40))
            parts.append(HostGraph.grid(n, n, seed=100 + i))
        else:
            parts.append(HostGraph.rmat(int(rng.integers(6, 13)), int(rng.integers(4, 33)), seed=200 + i))
    local = [int(p.pick_sources(1, seed=i)[0]) for i, p in enumerate(parts)]
    res, st = multigraph_batch(parts, app, local, delta=16)
    for p, s, r in zip(parts, local, res):
        off, dst, w = np.array(p.offsets), np.array(p.dst), np.array(p.weights)
        ref = oracle.bfs(off, dst, s) if app == "bfs" else oracle.sssp_dijkstra(off, dst, w, s)
        np.testing.assert_array_equal(r, ref)


@pytest.mark.parametrize("app", ["bfs", "sssp"])
def test_batch_plan_cuda_graph_replay(app):
    import torch
    from easy_graphit_gb300 import BatchPlan
    hg, g, (off, dst, w) = graph("dir14")
    srcs = hg.pick_sources(70, seed=9)
    out = torch.full((70, hg.num_vertices), -7, dtype=torch.int32, device="cuda")
    plan = BatchPlan(g, app, srcs, out, delta=32)
    for _ in range(2):  # replay twice: the second run must not see the first's state
        st = plan.run()
        got = out.cpu().numpy()
        for i in [0, 33, 63, 64, 69]:
            ref = oracle.bfs(off, dst, int(srcs[i])) if app == "bfs" else \
                oracle.sssp_dijkstra(off, dst, w, int(srcs[i]))
            np.testing.assert_array_equal(got[i], ref)
        out.fill_(-7)
    plan.close()
