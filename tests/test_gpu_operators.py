"""The operator-level boundary, driven the way GraphIt's generated code drives
the runtime: each app's testcase() loop (apps/bfs.cpp:36-62, sssp.cpp:34-57,
bc.cpp:64-123, pr.cpp:49-69, cc.cpp:53-77) composed from edgeset_apply(s)
.from_(f).to(filter).apply / apply_modified / apply_priority, vertexset_apply,
the priority queue, the frontier list and the frontier conversions, and
compared with the oracle: BFS parents form a valid BFS tree, SSSP distances
and CC labels are bit-exact, PageRank and BC are within 1e-6 relative L1 of
FP64.  Every call goes through the C ABI (gg_edgeset_apply,
gg_vertexset_apply, gg_pq_*, gg_edgeset_apply_priority, gg_frontier_*,
gg_frontier_list_*).
"""
import numpy as np
import pytest

import oracle
from easy_graphit_gb300 import (UDF, VUDF, Filter, GraphT, HostGraph, HybridGPUSchedule, PriorityQueue,
                                SimpleGPUSchedule as T, VertexData, VertexFrontierList, VertexSubset,
                                edgeset_apply, vertexset_apply)
from tests.conftest import INT_MAX, rel_l1

pytestmark = pytest.mark.gpu

TOL = 1e-6  # PageRank and BC: relative L1 against the FP64 oracle
D, LB, FC, PR_ = T.direction_type, T.load_balancing_type, T.frontier_creation_type, T.pull_frontier_rep_type
_G = {}


def graph(name):
    if name not in _G:
        hg = {"sym12": lambda: HostGraph.rmat(12, 16, symmetrize=True),
              "dir12": lambda: HostGraph.rmat(12, 16),
              "grid": lambda: HostGraph.grid(48, 64)}[name]()
        # the grid has every edge both ways but with independent weights, so it is
        # not symmetric in the GG_GRAPH_SYMMETRIC sense (a weighted pull needs its transpose)
        sym = name == "sym12"
        _G[name] = (GraphT(hg, symmetric=sym), np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights))
    return _G[name]


def dev(n, dtype, fill=0):
    import torch
    return torch.full((n,), fill, dtype=dtype, device="cuda")


def hub(off):
    return int(np.argmax(np.diff(off)))


def sched(direction=D.PUSH, lb=LB.TWCE, creation=FC.SPARSE, pull_rep=PR_.BITMAP, dedup_unfused=False):
    s = T().configDirection(direction, pull_rep).configLoadBalancing(lb).configFrontierCreation(creation)
    if dedup_unfused:
        s.configDeduplication(T.deduplication_type.ENABLED, T.deduplication_strategy_type.UNFUSED)
    return s


# ------------------------------------------------------------------- BFS
def bfs_testcase(g, V, src, s1):
    """apps/bfs.cpp:36-62 (one trial)."""
    import torch
    parent = dev(V, torch.int32)
    vd = VertexData(parent=parent, src=src)
    vertexset_apply(g, VUDF.BFS_RESET, vd)          # reset; parent[src] = src
    frontier = VertexSubset(g)
    frontier.addVertex(src)
    while frontier.size() != 0:
        edgeset_apply(s1).from_(frontier).to(Filter.PARENT_UNSET).apply_modified(g, frontier, vd,
                                                                                 UDF.BFS_PARENT)
    return parent.cpu().numpy()


@pytest.mark.parametrize("s1", [
    sched(),
    sched(lb=LB.VERTEX_BASED),
    sched(lb=LB.CM, creation=FC.BITMAP),
    sched(lb=LB.WM, creation=FC.BOOLMAP),
    sched(lb=LB.EDGE_ONLY),
    sched(direction=D.PULL, lb=LB.VERTEX_BASED, creation=FC.BITMAP),
    sched(direction=D.PULL, lb=LB.TWCE, pull_rep=PR_.BOOLMAP),
    HybridGPUSchedule(sched(), sched(direction=D.PULL, lb=LB.VERTEX_BASED, creation=FC.BITMAP))
    .configThreshold(0.05),
], ids=["push_twce", "push_vertex", "push_cm_bitmap_out", "push_wm_boolmap_out", "push_edge_only",
        "pull_vertex_bitmap", "pull_twce_boolmap", "hybrid_power"])
@pytest.mark.parametrize("name", ["sym12", "grid"])
def test_bfs_testcase_through_operators(name, s1):
    g, off, dst, _ = graph(name)
    V = len(off) - 1
    src = hub(off)
    parent = bfs_testcase(g, V, src, s1)
    depth = oracle.bfs(off, dst, src)
    np.testing.assert_array_equal(parent >= 0, depth >= 0)
    assert oracle.bfs_check_parent(off, dst, src, depth, parent) == 0


def test_bfs_hybrid_threshold_bound_at_run_time():
    """bindThreshold binds a value the caller changes between trials
    (bfs.cpp:38-39): 0 runs every level with s2, 1 every level with s1; both
    give a valid BFS tree."""
    g, off, dst, _ = graph("sym12")
    V = len(off) - 1
    src = hub(off)
    t = [0.0]
    h = HybridGPUSchedule(sched(), sched(direction=D.PULL, lb=LB.VERTEX_BASED, creation=FC.BITMAP))
    h.bindThreshold(t)
    depth = oracle.bfs(off, dst, src)
    for value in (0.0, 1.0, 0.02):
        t[0] = value
        assert h.threshold == value
        parent = bfs_testcase(g, V, src, h)
        assert oracle.bfs_check_parent(off, dst, src, depth, parent) == 0


# ------------------------------------------------------------------ SSSP
def sssp_testcase(g, V, src, delta, s1):
    """apps/sssp.cpp:34-57 (one trial)."""
    import torch
    SP = dev(V, torch.int32)
    pq = PriorityQueue(g, SP, 0, delta, src)        # pq.init(edges, SP, 0, delta, src)
    vertexset_apply(g, VUDF.SSSP_RESET, VertexData(dist=SP, src=src))  # reset; SP[src] = 0
    rounds = 0
    while not pq.finished():
        frontier = pq.dequeue()
        edgeset_apply(s1).from_(frontier).apply_priority(g, UDF.SSSP_RELAX, pq)
        rounds += 1
    pq.close()
    return SP.cpu().numpy(), rounds


@pytest.mark.parametrize("s1", [
    sched(lb=LB.VERTEX_BASED),
    sched(lb=LB.TWCE),
    sched(lb=LB.CM),
    sched(lb=LB.WM),
    sched(lb=LB.ETWC),
    sched(lb=LB.TWC),
    sched(lb=LB.STRICT),
    sched(lb=LB.TWCE, creation=FC.BOOLMAP),
    sched(lb=LB.VERTEX_BASED, creation=FC.BITMAP),
    sched(direction=D.PULL, lb=LB.VERTEX_BASED),
], ids=["vertex", "twce", "cm", "wm", "etwc", "twc", "strict", "twce_boolmap", "vertex_bitmap",
        "pull_vertex"])
@pytest.mark.parametrize("delta", [1, 32])
@pytest.mark.parametrize("name", ["dir12", "grid"])
def test_sssp_testcase_through_operators(name, delta, s1):
    g, off, dst, w = graph(name)
    V = len(off) - 1
    src = hub(off)
    d, rounds = sssp_testcase(g, V, src, delta, s1)
    np.testing.assert_array_equal(d, oracle.sssp_dijkstra(off, dst, w, src))
    assert rounds >= 1


@pytest.mark.parametrize("fuse", [False, True], ids=["host_driven", "persistent"])
def test_sssp_queue_advances_by_the_reference_bucket_rule(fuse):
    """Both queues (the host-driven one behind dequeue() and the persistent
    loop's) move their windows exactly as gpu_priority_queue.h does: the same
    number of bucket advances as the sequential restatement of the reference
    loop, which scans all V per advance."""
    from easy_graphit_gb300 import sssp
    for name in ("grid", "dir12"):
        g, off, dst, w = graph(name)
        src = 100 if name == "grid" else hub(off)
        for delta in (1, 3, 8, 64, 1000):
            d, st = sssp(g, src, delta, sched(lb=LB.TWCE), fuse)
            ref, adv = oracle.sssp_delta_gpu(off, dst, w, src, delta)
            np.testing.assert_array_equal(d, ref)
            assert st["bucket_advances"] == adv, (name, delta)


# -------------------------------------------------------------------- BC
def bc_testcase(g, V, src, s1):
    """apps/bc.cpp:64-123 (one trial), fp32 dependences as in the reference."""
    import torch
    num_paths = dev(V, torch.float64)
    dependences = dev(V, torch.float32)
    visited = dev(V, torch.uint8)
    vd = VertexData(num_paths=num_paths, dependences=dependences, visited=visited, src=src)
    vertexset_apply(g, VUDF.BC_RESET, vd)            # reset; num_paths[src] = 1; visited[src] = 1
    frontier = VertexSubset(g)
    frontier.addVertex(src)
    rnd = 0
    frontier_list = VertexFrontierList(g)
    frontier_list.insert(frontier)
    while frontier.size() != 0:
        rnd += 1
        edgeset_apply(s1).from_(frontier).to(Filter.UNVISITED).apply_modified(
            g, frontier, vd, UDF.BC_FORWARD, allow_dupes=False)
        vertexset_apply(frontier, VUDF.BC_MARK_VISITED, vd)
        frontier_list.insert(frontier)
    vertexset_apply(g, VUDF.BC_MARK_UNVISITED, vd)
    frontier_list.retrieve(frontier)
    frontier_list.retrieve(frontier)
    vertexset_apply(frontier, VUDF.BC_BACKWARD_VERTEX, vd)
    rnd -= 1
    while rnd > 0:
        edgeset_apply(s1).from_(frontier).to(Filter.UNVISITED).apply(g, UDF.BC_BACKWARD, vd)
        frontier_list.retrieve(frontier)
        vertexset_apply(frontier, VUDF.BC_BACKWARD_VERTEX, vd)
        rnd -= 1
    vertexset_apply(g, VUDF.BC_FINAL, vd)
    frontier_list.close()
    return dependences.cpu().numpy()


@pytest.mark.parametrize("s1", [
    sched(),                                  # bc.cpp default: PUSH TWCE, fused dedup
    sched(dedup_unfused=True),                # dedup_frontier_perfect after the apply
    sched(lb=LB.VERTEX_BASED, dedup_unfused=True),
    sched(lb=LB.CM),
    HybridGPUSchedule(sched(), sched(direction=D.PULL, lb=LB.TWCE, creation=FC.BITMAP)).configThreshold(0.1),
], ids=["push_twce_fused_dedup", "push_twce_unfused_dedup", "push_vertex_unfused_dedup", "push_cm",
        "hybrid_power"])
@pytest.mark.parametrize("name", ["sym12", "grid"])
def test_bc_testcase_through_operators(name, s1):
    g, off, dst, _ = graph(name)
    V = len(off) - 1
    src = hub(off)
    dep = bc_testcase(g, V, src, s1)
    assert rel_l1(dep, oracle.bc(off, dst, src)) <= TOL


# ------------------------------------------------------------- PageRank
@pytest.mark.parametrize("s1", [
    sched(direction=D.PULL, lb=LB.EDGE_ONLY),
    sched(direction=D.PUSH, lb=LB.TWCE),
    sched(direction=D.PULL, lb=LB.WM),
], ids=["pull_edge_only", "push_twce", "pull_wm"])
def test_pagerank_testcase_through_operators(s1):
    """apps/pr.cpp:49-69 (one trial, 20 iterations)."""
    import torch
    g, off, dst, _ = graph("dir12")
    V = len(off) - 1
    old_rank, new_rank, contrib = dev(V, torch.float32), dev(V, torch.float32), dev(V, torch.float32)
    vd = VertexData(old_rank=old_rank, new_rank=new_rank, contrib=contrib, damping=0.85)
    vertexset_apply(g, VUDF.PR_RESET, vd)
    for _ in range(20):
        vertexset_apply(g, VUDF.PR_CONTRIB, vd)
        edgeset_apply(s1).apply(g, UDF.PR_ADD, vd)
        vertexset_apply(g, VUDF.PR_UPDATE, vd)
    ref = oracle.pagerank(off, dst, 20, float(np.float32(0.85)))
    assert rel_l1(old_rank.cpu().numpy(), ref) <= TOL


# ------------------------------------------------------------------- CC
def test_cc_testcase_through_operators():
    """apps/cc.cpp:53-77 (one trial): hook rounds, pointer jumping until stable."""
    import torch
    g, off, dst, _ = graph("sym12")
    V = len(off) - 1
    ids, updates = dev(V, torch.int32), dev(2, torch.int32)
    vd = VertexData(ids=ids, updates=updates)
    vertexset_apply(g, VUDF.CC_INIT, vd)
    updates[0] = 1
    s1 = sched(lb=LB.EDGE_ONLY)
    while int(updates[0]):
        updates[0] = 0
        edgeset_apply(s1).apply(g, UDF.CC_HOOK, vd)
        updates[1] = 1
        while int(updates[1]):
            updates[1] = 0
            vertexset_apply(g, VUDF.CC_PJUMP, vd)
    np.testing.assert_array_equal(ids.cpu().numpy(), oracle.cc(off, dst))


# -------------------------------------------------------- frontier formats
def test_frontier_conversions_and_unfused_dedup():
    """to_bitmap / to_boolmap / to_sparse keep the member set; dedup
    (dedup_frontier_perfect, vertex_frontier.h:382-386) removes repeats."""
    g, off, dst, _ = graph("sym12")
    V = len(off) - 1
    f = VertexSubset(g)
    members = [5, 17, 17, 100, 5, V - 1, 2048, 17]
    for v in members:
        f.addVertex(v)
    assert f.size() == len(members)
    f.dedup()
    want = np.array(sorted(set(members)), dtype=np.int32)
    assert f.size() == len(want)
    np.testing.assert_array_equal(f.read(), want)
    for conv, fmt in ((f.to_bitmap, VertexSubset.BITMAP), (f.to_boolmap, VertexSubset.BOOLMAP),
                      (f.to_sparse, VertexSubset.SPARSE), (f.to_boolmap, VertexSubset.BOOLMAP),
                      (f.to_bitmap, VertexSubset.BITMAP)):
        conv()
        assert f.format() == fmt
        assert f.size() == len(want)
        np.testing.assert_array_equal(f.read(), want)
    f.clear()
    assert f.size() == 0


def test_frontier_of_a_bfs_level_survives_every_conversion():
    import torch
    g, off, dst, _ = graph("sym12")
    V = len(off) - 1
    src = hub(off)
    parent = dev(V, torch.int32)
    vd = VertexData(parent=parent, src=src)
    vertexset_apply(g, VUDF.BFS_RESET, vd)
    f = VertexSubset(g)
    f.addVertex(src)
    edgeset_apply(sched()).from_(f).to(Filter.PARENT_UNSET).apply_modified(g, f, vd, UDF.BFS_PARENT)
    depth = oracle.bfs(off, dst, src)
    want = np.nonzero(depth == 1)[0].astype(np.int32)
    np.testing.assert_array_equal(f.read(), want)
    for conv in (f.to_boolmap, f.to_bitmap, f.to_sparse):
        conv()
        np.testing.assert_array_equal(f.read(), want)
