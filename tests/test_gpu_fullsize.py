"""The named workloads at their full sizes, through the C ABI on the GPU.

  BFS    symmetrized R-MAT 16, highest-degree source, bfs.cpp's push TWCE
  SSSP   directed R-MAT 22 and the 4096 x 4096 grid, delta in {1, 8, 32, 128}
  PR     directed R-MAT 24, 20 iterations (1e-6 relative L1 against FP64)
  CC     symmetrized R-MAT 24 (labels = minimum id per component)
  batch  256 BFS and 256 SSSP sources on R-MAT 22, BC from 64 sources on the
         symmetrized R-MAT 22, and the mix of 64 uneven graphs

The oracle runs in full on sampled sources; every other source is held to a
size-independent property: its batched row equals the engine's single-source
run of the same source (itself held to the oracle at smaller sizes), or SSSP
rows carry a shortest-path certificate (no edge improves them, and every
reached vertex has a tight in-edge).
"""
import numpy as np
import pytest

import oracle
from easy_graphit_gb300 import (GraphT, HostGraph, SimpleGPUSchedule as T, bc, bc_batch, bfs,
                                bfs_batch, cc, default_schedule, multigraph_batch, pagerank,
                                sssp, sssp_batch)
from tests.conftest import rel_l1, shortest_paths_certified

pytestmark = pytest.mark.gpu

INT_MAX = 2**31 - 1
TOL = 1e-6
_G = {}


def graph(name):
    if name not in _G:
        if name == "rmat16s":
            hg = HostGraph.rmat(16, 16, symmetrize=True)
        elif name == "rmat22":
            hg = HostGraph.rmat(22, 16)
        elif name == "rmat22s":
            hg = HostGraph.rmat(22, 16, symmetrize=True)
        elif name == "grid4096":
            hg = HostGraph.grid(4096, 4096)
        elif name == "grid1024":
            hg = HostGraph.grid(1024, 1024)
        sym = name.endswith("s")  # grid weights differ per direction: not symmetric
        _G[name] = (hg, GraphT(hg, symmetric=sym),
                    (np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)))
    return _G[name]


def release(name):
    if name in _G:
        _G.pop(name)[1].close()


def test_bfs_rmat16_symmetrized_highest_degree_source():
    hg, g, (off, dst, _) = graph("rmat16s")
    src = int(np.argmax(np.diff(off)))
    sch, fuse = default_schedule("bfs")
    depth, parent, _ = bfs(g, src, sch, fuse, with_parent=True)
    np.testing.assert_array_equal(depth, oracle.bfs(off, dst, src))
    assert oracle.bfs_check_parent(off, dst, src, depth, parent) == 0
    release("rmat16s")


@pytest.mark.parametrize("delta", [1, 8, 32, 128])
def test_sssp_rmat22_32_sources(delta):
    hg, g, (off, dst, w) = graph("rmat22")
    srcs = hg.pick_sources(32)
    dist, _ = sssp_batch(g, srcs, delta)
    for i in (0, 1):  # the oracle in full on two sources
        key = ("dijkstra22", int(srcs[i]))
        if key not in _G:
            _G[key] = oracle.sssp_dijkstra(off, dst, w, int(srcs[i]))
        np.testing.assert_array_equal(dist[i], _G[key])
    twce = T().configLoadBalancing(T.load_balancing_type.TWCE)
    for i in range(0, 32, 1 if delta == 32 else 8):  # every source against the engine's single run
        one, _ = sssp(g, int(srcs[i]), delta, twce, True)
        np.testing.assert_array_equal(dist[i], one)
    assert shortest_paths_certified(off, dst, w, dist[31], int(srcs[31]))


GRID_DELTAS = [1, 8, 32, 128]


def grid_ref(i):
    """Dijkstra distances of the i-th SourcePicker source of the 4096 x 4096 grid."""
    hg, g, (off, dst, w) = graph("grid4096")
    s = int(hg.pick_sources(2)[i])
    key = ("grid4096", s)
    if key not in _G:
        _G[key] = oracle.sssp_dijkstra(off, dst, w, s)
    return s, _G[key]


@pytest.mark.parametrize("delta", GRID_DELTAS)
def test_sssp_grid4096_batched(delta):
    """Two sources in one batched call: on a mesh every source runs the
    bucket queue in a CTA of its own."""
    hg, g, _ = graph("grid4096")
    srcs = hg.pick_sources(2)
    dist, st = sssp_batch(g, srcs, delta)
    for i in range(2):
        np.testing.assert_array_equal(dist[i], grid_ref(i)[1])


@pytest.mark.parametrize("delta", GRID_DELTAS)
def test_sssp_grid4096_single_source_fused(delta):
    """sssp.cpp's own schedule (PUSH SPARSE VERTEX_BASED, fused) from two
    sources; the bucket advances follow the reference rule exactly."""
    hg, g, (off, dst, w) = graph("grid4096")
    sch, fuse = default_schedule("sssp")
    for i in range(2):
        s, ref = grid_ref(i)
        dist, st = sssp(g, s, delta, sch, fuse)
        np.testing.assert_array_equal(dist, ref)
        assert st["fused"] == 1


@pytest.mark.parametrize("delta", [32, 128])
def test_sssp_grid4096_single_source_unfused(delta):
    """The host-driven queue (one frontier-size read and one minimum read-back
    per bucket, as the reference's host loop) from one source.  At delta 1 and
    8 the 4096 x 4096 grid has 10^5 to 10^6 buckets, one host round trip each
    (16 s and 95 s): those deltas run on the 1024 x 1024 grid below."""
    hg, g, _ = graph("grid4096")
    s, ref = grid_ref(0)
    dist, st = sssp(g, s, delta, T().configLoadBalancing(T.load_balancing_type.TWCE), False)
    np.testing.assert_array_equal(dist, ref)
    assert st["fused"] == 0


@pytest.mark.parametrize("delta", [1, 8])
def test_sssp_grid1024_single_source_unfused_small_delta(delta):
    hg, g, (off, dst, w) = graph("grid1024")
    s = int(hg.pick_sources(1)[0])
    dist, st = sssp(g, s, delta, T().configLoadBalancing(T.load_balancing_type.TWCE), False)
    np.testing.assert_array_equal(dist, oracle.sssp_dijkstra(off, dst, w, s))
    assert st["fused"] == 0


def test_sssp_grid_lane_per_source_kernel():
    """The lane-per-source batched kernel (the R-MAT choice) on a mesh as well,
    by tuning: 32 sources of the 1024 x 1024 grid at delta 128."""
    from easy_graphit_gb300 import set_batch_tuning
    hg, g, (off, dst, w) = graph("grid1024")
    srcs = hg.pick_sources(32)
    set_batch_tuning(g, "sssp", per_source_cta=-1)
    lane, _ = sssp_batch(g, srcs, 128)
    set_batch_tuning(g, "sssp")
    cta, _ = sssp_batch(g, srcs, 128)
    np.testing.assert_array_equal(lane, cta)
    for i in (0, 31):
        np.testing.assert_array_equal(cta[i], oracle.sssp_dijkstra(off, dst, w, int(srcs[i])))
    release("grid1024")


def test_pagerank_rmat24():
    hg = HostGraph.rmat(24, 16)
    g = GraphT(hg)
    off, dst = np.array(hg.offsets), np.array(hg.dst)
    ref = oracle.pagerank(off, dst, 20, float(np.float32(0.85)))
    sch, _ = default_schedule("pr")
    r, st = pagerank(g, 20, 0.85, sch)
    assert rel_l1(r, ref) <= TOL, rel_l1(r, ref)
    tw = T().configDirection(T.direction_type.PULL).configLoadBalancing(T.load_balancing_type.TWC)
    r2, _ = pagerank(g, 20, 0.85, tw)
    assert rel_l1(r2, ref) <= TOL, rel_l1(r2, ref)
    assert st["edges_traversed"] == 20 * len(dst)
    g.close()


def test_cc_rmat24_symmetrized():
    hg = HostGraph.rmat(24, 16, symmetrize=True)
    g = GraphT(hg, symmetric=True)
    off, dst = np.array(hg.offsets), np.array(hg.dst)
    labels, _ = cc(g)
    np.testing.assert_array_equal(labels, oracle.cc_omp(off, dst))
    g.close()


def test_batched_256_bfs_and_256_sssp_sources_rmat22():
    hg, g, (off, dst, w) = graph("rmat22")
    srcs = hg.pick_sources(256, seed=7)
    depth, _ = bfs_batch(g, srcs)
    bsch, bfuse = default_schedule("bfs")
    for i in range(0, 256, 5):
        one, _, _ = bfs(g, int(srcs[i]), bsch, bfuse)
        np.testing.assert_array_equal(depth[i], one)
    for i in range(3, 256, 16):  # the oracle itself on 16 rows
        np.testing.assert_array_equal(depth[i], oracle.bfs(off, dst, int(srcs[i])))
    del depth
    dist, _ = sssp_batch(g, srcs, 32)
    twce = T().configLoadBalancing(T.load_balancing_type.TWCE)
    for i in range(0, 256, 5):
        one, _ = sssp(g, int(srcs[i]), 32, twce, True)
        np.testing.assert_array_equal(dist[i], one)
    for i in (7, 100, 200, 255):  # Dijkstra on four rows, one in each group of 64
        np.testing.assert_array_equal(dist[i], oracle.sssp_dijkstra(off, dst, w, int(srcs[i])))
    release("rmat22")


def test_bc_64_sources_rmat22_symmetrized():
    hg, g, (off, dst, _) = graph("rmat22s")
    srcs = hg.pick_sources(64, seed=3)
    dep, st = bc_batch(g, srcs)
    for i in (0, 33, 63):
        assert rel_l1(dep[i], oracle.bc(off, dst, int(srcs[i]))) <= TOL
    for i in range(0, 64, 4):
        one, _ = bc(g, int(srcs[i]))
        assert rel_l1(dep[i], one) <= TOL
    release("rmat22s")


@pytest.mark.parametrize("app", ["bfs", "sssp"])
def test_mix_of_64_uneven_graphs(app):
    parts = HostGraph.mix(64)
    spec = HostGraph.mix_spec(64)
    assert (spec[:, 0] == 1).any() and (spec[:, 0] == 0).any()
    local = [int(p.pick_sources(1, seed=i)[0]) for i, p in enumerate(parts)]
    res, st = multigraph_batch(parts, app, local, delta=32)
    # the same traversal captured into a CUDA graph (one persistent launch per replay)
    import torch
    from easy_graphit_gb300 import BatchPlan
    hg, offs = HostGraph.union(parts)
    g = GraphT(hg)
    srcs = np.array([offs[i] + s for i, s in enumerate(local)], dtype=np.int32)
    out = torch.empty((hg.num_vertices,), dtype=torch.int32, device="cuda")
    plan = BatchPlan(g, app + "_multi", srcs, out, delta=32)
    plan.run()
    np.testing.assert_array_equal(out.cpu().numpy(), np.concatenate(res))
    plan.close()
    g.close()
    for i, (p, s, r) in enumerate(zip(parts, local, res)):
        off, dst, w = np.array(p.offsets), np.array(p.dst), np.array(p.weights)
        if app == "bfs":
            np.testing.assert_array_equal(r, oracle.bfs(off, dst, s))
        elif i % 4 == 0:  # Dijkstra on every fourth graph, the certificate on the others
            np.testing.assert_array_equal(r, oracle.sssp_dijkstra(off, dst, w, s))
        else:
            assert shortest_paths_certified(off, dst, w, r, s)
