"""GPU parity of the five apps against the oracle, through the C ABI.

Bit-exact: BFS depths (and a valid parent tree), SSSP int32 distances, CC
labels.  PageRank and BC: relative L1 <= 1e-6 against the FP64 oracle.
Every load-balancing strategy, both directions, every frontier representation
and the fused/unfused loops must give the same results.
"""
import numpy as np
import pytest

import oracle
from easy_graphit_gb300 import (GraphT, HostGraph, HybridGPUSchedule, SimpleGPUSchedule, bc, bfs,
                                cc, default_schedule, pagerank, sssp)
from tests.conftest import rel_l1

pytestmark = pytest.mark.gpu

T = SimpleGPUSchedule
LBS = [T.load_balancing_type.VERTEX_BASED, T.load_balancing_type.TWC, T.load_balancing_type.TWCE,
       T.load_balancing_type.WM, T.load_balancing_type.CM, T.load_balancing_type.STRICT,
       T.load_balancing_type.EDGE_ONLY, T.load_balancing_type.ETWC]
PR_TOL = 1e-6
BC_TOL = 1e-6


def sched(direction=T.direction_type.PUSH, lb=T.load_balancing_type.TWCE,
          creation=T.frontier_creation_type.SPARSE, pull_rep=T.pull_frontier_rep_type.BITMAP,
          blocked=0, cta=512):
    s = SimpleGPUSchedule()
    s.configDirection(direction, pull_rep)
    if lb == T.load_balancing_type.EDGE_ONLY and blocked:
        s.configLoadBalancing(lb, T.edge_blocking_type.BLOCKED, blocked)
    else:
        s.configLoadBalancing(lb)
    s.configFrontierCreation(creation)
    s.cta_size = cta
    return s


_CACHE = {}


def graph(kind):
    if kind not in _CACHE:
        if kind == "sym12":
            hg = HostGraph.rmat(12, 16, symmetrize=True)
        elif kind == "dir12":
            hg = HostGraph.rmat(12, 16)
        elif kind == "sym16":
            hg = HostGraph.rmat(16, 16, symmetrize=True)
        elif kind == "dir16":
            hg = HostGraph.rmat(16, 16)
        elif kind == "grid":
            hg = HostGraph.grid(64, 48)
        else:
            raise KeyError(kind)
        sym = kind.startswith("sym") or kind == "grid"
        _CACHE[kind] = (hg, GraphT(hg, symmetric=sym),
                        (np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)))
    return _CACHE[kind]


def hub(off):
    return int(np.argmax(np.diff(off)))


# ------------------------------------------------------------------ BFS
@pytest.mark.parametrize("lb", LBS, ids=lambda x: x.name)
@pytest.mark.parametrize("kind", ["sym12", "dir12"])
def test_bfs_push_every_lb(kind, lb):
    hg, g, (off, dst, _) = graph(kind)
    s = hub(off)
    ref = oracle.bfs(off, dst, s)
    depth, parent, st = bfs(g, s, sched(lb=lb), fuse=False, with_parent=True)
    np.testing.assert_array_equal(depth, ref)
    assert oracle.bfs_check_parent(off, dst, s, depth, parent) == 0
    assert st["iterations"] == ref.max() + 1


@pytest.mark.parametrize("lb", [T.load_balancing_type.VERTEX_BASED, T.load_balancing_type.TWCE,
                                T.load_balancing_type.WM, T.load_balancing_type.CM],
                         ids=lambda x: x.name)
@pytest.mark.parametrize("kind", ["sym16", "dir16", "grid"])
def test_bfs_fused(kind, lb):
    hg, g, (off, dst, _) = graph(kind)
    s = hub(off)
    ref = oracle.bfs(off, dst, s)
    depth, parent, st = bfs(g, s, sched(lb=lb), fuse=True, with_parent=True)
    np.testing.assert_array_equal(depth, ref)
    assert oracle.bfs_check_parent(off, dst, s, depth, parent) == 0
    assert st["edges_traversed"] == oracle.reached_edges(off, ref)


@pytest.mark.parametrize("creation", list(T.frontier_creation_type), ids=lambda x: x.name)
@pytest.mark.parametrize("pull_rep", list(T.pull_frontier_rep_type), ids=lambda x: x.name)
@pytest.mark.parametrize("lb", [T.load_balancing_type.VERTEX_BASED, T.load_balancing_type.WM,
                                T.load_balancing_type.TWCE, T.load_balancing_type.EDGE_ONLY],
                         ids=lambda x: x.name)
def test_bfs_pull_every_representation(creation, pull_rep, lb):
    hg, g, (off, dst, _) = graph("dir12")
    s = hub(off)
    ref = oracle.bfs(off, dst, s)
    sc = sched(direction=T.direction_type.PULL, lb=lb, creation=creation, pull_rep=pull_rep)
    depth, parent, _ = bfs(g, s, sc, fuse=False, with_parent=True)
    np.testing.assert_array_equal(depth, ref)
    assert oracle.bfs_check_parent(off, dst, s, depth, parent) == 0


@pytest.mark.parametrize("threshold", [0.0, 0.01, 0.12, 1.0])
def test_bfs_hybrid_power_schedule(threshold):
    hg, g, (off, dst, _) = graph("sym16")
    s = hub(off)
    ref = oracle.bfs(off, dst, s)
    hs, _ = default_schedule("bfs", power=True, threshold=threshold)
    depth, parent, st = bfs(g, s, hs, fuse=False, with_parent=True)
    np.testing.assert_array_equal(depth, ref)
    assert oracle.bfs_check_parent(off, dst, s, depth, parent) == 0
    if threshold == 0.0:
        assert st["push_iterations"] <= 1
    if threshold == 1.0:
        assert st["pull_iterations"] == 0


def test_bfs_golden_reference_depths(golden):
    hg = HostGraph.rmat(12, 16)
    g = GraphT(hg)
    for i, s in enumerate(golden["sources/rmat12_k16_dir"]):
        depth, _, _ = bfs(g, int(s))
        np.testing.assert_array_equal(depth, golden["bfs/rmat12_k16_dir"][i])


# ------------------------------------------------------------------ SSSP
@pytest.mark.parametrize("delta", [1, 8, 32, 128])
def test_sssp_golden_reference_distances(golden, delta):
    for name, (scale, sym) in {"rmat10_k16_sym": (10, True), "rmat12_k16_dir": (12, False)}.items():
        hg = HostGraph.rmat(scale, 16, symmetrize=sym)
        g = GraphT(hg, symmetric=sym)
        for fuse in (True, False):
            for i, s in enumerate(golden[f"sources/{name}"]):
                d, _ = sssp(g, int(s), delta, fuse=fuse)
                np.testing.assert_array_equal(d, golden[f"sssp/{name}/d{delta}"][i])


@pytest.mark.parametrize("lb", LBS, ids=lambda x: x.name)
@pytest.mark.parametrize("creation", list(T.frontier_creation_type), ids=lambda x: x.name)
def test_sssp_every_lb_and_creation(lb, creation):
    hg, g, (off, dst, w) = graph("dir12")
    s = hub(off)
    ref = oracle.sssp_dijkstra(off, dst, w, s)
    d, st = sssp(g, s, 32, sched(lb=lb, creation=creation), fuse=False)
    np.testing.assert_array_equal(d, ref)


@pytest.mark.parametrize("lb", [T.load_balancing_type.VERTEX_BASED, T.load_balancing_type.TWCE,
                                T.load_balancing_type.WM, T.load_balancing_type.CM],
                         ids=lambda x: x.name)
@pytest.mark.parametrize("delta", [1, 128])
def test_sssp_fused_larger(lb, delta):
    hg, g, (off, dst, w) = graph("dir16")
    s = hub(off)
    ref = oracle.sssp_dijkstra(off, dst, w, s)
    d, st = sssp(g, s, delta, sched(lb=lb), fuse=True)
    np.testing.assert_array_equal(d, ref)
    _, adv = oracle.sssp_delta_gpu(off, dst, w, s, delta)
    assert st["bucket_advances"] == adv


def test_sssp_grid_and_power_schedule():
    hg, g, (off, dst, w) = graph("grid")
    for s in [0, 1000, 3071]:
        ref = oracle.sssp_dijkstra(off, dst, w, s)
        for delta in [8, 128]:
            d, _ = sssp(g, s, delta)  # default: PUSH SPARSE VERTEX_BASED fused
            np.testing.assert_array_equal(d, ref)
            ps, fuse = default_schedule("sssp", power=True)
            d, _ = sssp(g, s, delta, ps, fuse=fuse)
            np.testing.assert_array_equal(d, ref)


# --------------------------------------------------------------- PageRank
@pytest.mark.parametrize("sc", [
    "default",
    sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.EDGE_ONLY),
    sched(direction=T.direction_type.PUSH, lb=T.load_balancing_type.EDGE_ONLY, blocked=1000),
    sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.WM),
    sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.VERTEX_BASED),
    sched(direction=T.direction_type.PUSH, lb=T.load_balancing_type.TWCE),
    sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.CM),
    sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.TWC),
], ids=["default", "pull_edge_only", "push_edge_only_blocked", "pull_wm", "pull_vertex",
        "push_twce", "pull_cm", "pull_twc_static"])
def test_pagerank(sc):
    hg, g, (off, dst, _) = graph("dir16")
    ref = oracle.pagerank(off, dst, 20, float(np.float32(0.85)))
    r, st = pagerank(g, 20, 0.85, None if sc == "default" else sc)
    assert rel_l1(r, ref) <= PR_TOL, rel_l1(r, ref)


@pytest.mark.parametrize("kind", ["sym16", "dir16"])
def test_pagerank_static_pull_is_bitwise_deterministic(kind):
    """PULL + TWC runs the static pull gather: one owner per vertex, fixed
    summation order, so two runs agree bit for bit."""
    hg, g, (off, dst, _) = graph(kind)
    sc = sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.TWC)
    ref = oracle.pagerank(off, dst, 20, float(np.float32(0.85)))
    r1, st = pagerank(g, 20, 0.85, sc)
    r2, _ = pagerank(g, 20, 0.85, sc)
    np.testing.assert_array_equal(r1, r2)
    assert rel_l1(r1, ref) <= PR_TOL, rel_l1(r1, ref)
    assert st["iterations"] == 20 and st["edges_traversed"] == 20 * len(dst)


# --------------------------------------------------------------------- CC
@pytest.mark.parametrize("lb", LBS, ids=lambda x: x.name)
@pytest.mark.parametrize("kind", ["sym12", "dir12"])
def test_cc(kind, lb):
    hg, g, (off, dst, _) = graph(kind)
    ref = oracle.cc(off, dst)
    labels, _ = cc(g, sched(lb=lb))
    np.testing.assert_array_equal(labels, ref)


def test_cc_default_large():
    hg, g, (off, dst, _) = graph("sym16")
    labels, st = cc(g)
    np.testing.assert_array_equal(labels, oracle.cc(off, dst))


# --------------------------------------------------------------------- BC
@pytest.mark.parametrize("power", [False, True])
@pytest.mark.parametrize("kind", ["sym12", "sym16", "grid"])
def test_bc(kind, power):
    hg, g, (off, dst, _) = graph(kind)
    s = hub(off)
    ref = oracle.bc(off, dst, s)
    sch, fuse = default_schedule("bc", power=power, threshold=0.05)
    dep, st = bc(g, s, sch, fuse=fuse)
    assert rel_l1(dep, ref) <= BC_TOL, rel_l1(dep, ref)


@pytest.mark.parametrize("lb", LBS, ids=lambda x: x.name)
def test_bc_every_lb(lb):
    hg, g, (off, dst, _) = graph("sym12")
    s = hub(off)
    ref = oracle.bc(off, dst, s)
    dep, _ = bc(g, s, sched(lb=lb), fuse=False)
    assert rel_l1(dep, ref) <= BC_TOL, rel_l1(dep, ref)


# ------------------------------------------------------------- edge cases
def test_edge_cases():
    # isolated source, empty edge set, self-loops and duplicates kept by from_csr
    hg = HostGraph.from_csr([0, 0, 0, 0], [], None)
    g = GraphT(hg)
    depth, _, _ = bfs(g, 1)
    np.testing.assert_array_equal(depth, [-1, 0, -1])
    d, _ = sssp(g, 2, 4)
    np.testing.assert_array_equal(d, [2**31 - 1, 2**31 - 1, 0])
    labels, _ = cc(g)
    np.testing.assert_array_equal(labels, [0, 1, 2])
    off = [0, 3, 4, 4]
    dst = [0, 1, 1, 2]  # self-loop 0->0, duplicate 0->1
    hg = HostGraph.from_csr(off, dst, [1, 5, 2, 1])
    g = GraphT(hg)
    depth, parent, _ = bfs(g, 0, with_parent=True)
    np.testing.assert_array_equal(depth, [0, 1, 2])
    d, _ = sssp(g, 0, 1)
    np.testing.assert_array_equal(d, [0, 2, 3])
    # path graph: deep
    n = 3000
    hg = HostGraph.from_edges(n, np.arange(n - 1), np.arange(1, n), symmetrize=True)
    g = GraphT(hg, symmetric=True)
    depth, _, st = bfs(g, 0)
    np.testing.assert_array_equal(depth, np.arange(n))
    dep, _ = bc(g, 0)
    ref = oracle.bc(np.array(hg.offsets), np.array(hg.dst), 0)
    assert rel_l1(dep, ref) <= BC_TOL
    # star: one hub with a huge degree
    n = 200000
    hg = HostGraph.from_edges(n, np.zeros(n - 1, dtype=np.int32), np.arange(1, n), symmetrize=True)
    g = GraphT(hg, symmetric=True)
    for lb in LBS:
        depth, _, _ = bfs(g, 5, sched(lb=lb), fuse=False)
        assert depth[0] == 1 and depth[5] == 0 and (depth[1:] == 2).sum() == n - 2


def test_deterministic_outputs():
    hg, g, (off, dst, w) = graph("dir16")
    s = hub(off)
    r1, _ = pagerank(g, 20, 0.85, sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.WM))
    r2, _ = pagerank(g, 20, 0.85, sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.WM))
    d1, _ = sssp(g, s, 8)
    d2, _ = sssp(g, s, 8)
    np.testing.assert_array_equal(d1, d2)
    assert rel_l1(r1, r2) < 1e-6


@pytest.mark.parametrize("kind", ["sym12", "dir12", "sym16", "dir16", "grid"])
def test_cc_fused_union_find_matches_the_rounds(kind):
    """fuse = 1 runs CC as one union-find pass; labels equal cc.cpp's rounds
    and the oracle's (minimum id per weakly connected component)."""
    hg, g, (off, dst, _) = graph(kind)
    sch, _ = default_schedule("cc")
    fused, st = cc(g, sch, True)
    rounds, _ = cc(g, sch)
    np.testing.assert_array_equal(fused, oracle.cc(off, dst))
    np.testing.assert_array_equal(fused, rounds)
    assert st["fused"] == 1


@pytest.mark.parametrize("symmetrize", [False, True])
def test_cc_fused_when_the_giant_tree_joins_a_smaller_root_late(symmetrize):
    """The union-find pass skips the vertices of the most frequent sampled root
    c after two sampling rounds.  Here component B = {0..99} (a path) reaches the
    giant component A = {1000..4999} only through edges 50 -> 3000 and 60 -> 4000
    that come after the first two entries of their out-lists, so on the directed
    graph they are never sampled and c's tree must be hooked under B's root 0
    during the finishing pass.  Vertices 100..999 are isolated, 5000..5009 form a
    ring of their own."""
    rng = np.random.default_rng(5)
    u = [np.arange(1000, 4999), rng.integers(1000, 5000, 20000)]
    v = [np.arange(1001, 5000), rng.integers(1000, 5000, 20000)]
    u += [np.arange(0, 99), np.array([50, 50, 50, 60, 60, 60])]
    v += [np.arange(1, 100), np.array([0, 1, 3000, 2, 3, 4000])]
    u += [np.arange(5000, 5010)]
    v += [np.array([5001, 5002, 5003, 5004, 5005, 5006, 5007, 5008, 5009, 5000])]
    hg = HostGraph.from_edges(5010, np.concatenate(u), np.concatenate(v), symmetrize=symmetrize)
    g = GraphT(hg, symmetric=symmetrize)
    off, dst = np.array(hg.offsets), np.array(hg.dst)
    sch, _ = default_schedule("cc")
    fused, st = cc(g, sch, True)
    ref = oracle.cc(off, dst)
    np.testing.assert_array_equal(fused, ref)
    assert fused[3000] == 0 and fused[4999] == 0 and fused[500] == 500 and fused[5005] == 5000
    g.close()


# ------------------------------------------------- the reference's own apps
@pytest.mark.parametrize("name", ["rmat10_k16_sym", "rmat11_k8_dir", "grid32"])
def test_engine_matches_the_reference_apps(app_golden, name):
    """The engine against what easy_graphit's own apps/*.cpp compute on the
    same graphs (tests/golden/ref_apps.npz, made by running those sources on
    the CPU): each app's default schedule and the batched / fused forms."""
    from easy_graphit_gb300 import bc_batch, bfs_batch, sssp_batch
    from tests.conftest import app_graph
    off, dst, w = app_graph(app_golden, name)
    g = GraphT(HostGraph.from_csr(off, dst, w), symmetric=name.endswith("_sym"))
    srcs = [int(s) for s in app_golden[f"sources/{name}"]]
    want = app_golden[f"pr/{name}"]
    r, _ = pagerank(g, 20, 0.85)  # pr.cpp's PULL EDGE_ONLY blocked schedule
    assert rel_l1(r, want) <= PR_TOL, rel_l1(r, want)
    r, _ = pagerank(g, 20, 0.85, sched(direction=T.direction_type.PULL, lb=T.load_balancing_type.TWC))
    assert rel_l1(r, want) <= PR_TOL, rel_l1(r, want)
    np.testing.assert_array_equal(cc(g)[0], app_golden[f"cc/{name}"])
    np.testing.assert_array_equal(cc(g, None, True)[0], app_golden[f"cc/{name}"])
    rows, _ = bc_batch(g, srcs)
    for k, s in enumerate(srcs):
        want = app_golden[f"bc/{name}/s{k}"]
        dep, _ = bc(g, s)
        assert rel_l1(dep, want) <= BC_TOL, (s, rel_l1(dep, want))
        assert rel_l1(rows[k], want) <= BC_TOL, (s, rel_l1(rows[k], want))
    want = app_golden[f"bfs/{name}"]
    np.testing.assert_array_equal(bfs(g, srcs[0])[0], want)
    np.testing.assert_array_equal(bfs_batch(g, srcs[:1])[0][0], want)
    for d in (1, 8, 32):
        want = app_golden[f"sssp/{name}/d{d}"]
        np.testing.assert_array_equal(sssp(g, srcs[0], d)[0], want)
        np.testing.assert_array_equal(sssp_batch(g, srcs[:1], d)[0][0], want)
    g.close()
