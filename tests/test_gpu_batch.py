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
@pytest.mark.parametrize("bottom_up", [0, -1, 4096])
def test_bfs_batch(kind, nsrc, bottom_up):
    from easy_graphit_gb300 import set_batch_tuning
    hg, g, (off, dst, _) = graph(kind)
    srcs = hg.pick_sources(nsrc, seed=11)
    set_batch_tuning(g, "bfs", bottom_up_div=bottom_up)
    try:
        depth, st = bfs_batch(g, srcs)
    finally:
        set_batch_tuning(g, "bfs")
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


@pytest.mark.parametrize("delta", [1, 16, 128])
def test_sssp_parts_one_cta_per_graph(delta):
    """gg_sssp_parts on a union of grids, paths and small R-MAT graphs: every
    part's loop in its own CTA, each part's distances equal to Dijkstra's."""
    from easy_graphit_gb300 import sssp_parts
    parts = [HostGraph.grid(n, m, seed=300 + n) for n, m in ((1, 1), (3, 50), (40, 40), (97, 13))]
    parts += [HostGraph.rmat(sc, ef, seed=400 + sc) for sc, ef in ((6, 4), (10, 16), (12, 8))]
    n = 700  # a weighted path: 700 buckets at delta 1
    parts.append(HostGraph.from_edges(n, np.arange(n - 1, dtype=np.int32), np.arange(1, n, dtype=np.int32),
                                      np.full(n - 1, 3, dtype=np.int32), symmetrize=True))
    hg, offs = HostGraph.union(parts)
    g = GraphT(hg)
    local = [int(p.pick_sources(1, seed=i)[0]) if p.num_edges else 0 for i, p in enumerate(parts)]
    srcs = np.array([offs[i] + s for i, s in enumerate(local)], dtype=np.int32)
    for _ in range(2):  # twice: the second call must not see the first's state
        dist, st = sssp_parts(g, offs, srcs, delta)
        for i, (p, s_) in enumerate(zip(parts, local)):
            off, dst, w = np.array(p.offsets), np.array(p.dst), np.array(p.weights)
            np.testing.assert_array_equal(dist[offs[i]:offs[i + 1]], oracle.sssp_dijkstra(off, dst, w, s_))
        assert st["fused"] == 1 and st["bucket_advances"] > 0
    g.close()


def test_sssp_parts_rejects_edges_across_parts():
    from easy_graphit_gb300 import _lib as L, sssp_parts
    hg = HostGraph.grid(8, 8)
    g = GraphT(hg)
    with pytest.raises(L.GGError) as e:  # rows 0-3 and 4-7 of one grid are not separate graphs
        sssp_parts(g, np.array([0, 32, 64]), np.array([0, 40]), 8)
    assert e.value.status == L.GG_ERR_INVALID
    with pytest.raises(L.GGError):
        sssp_parts(g, np.array([0, 64]), np.array([64]), 8)  # source outside its part
    g.close()


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


# ---------------------------------------------------------------- batched BC
BC_TOL = 1e-6  # relative L1 against the FP64 oracle, per source


@pytest.mark.parametrize("kind", ["sym14", "dir14", "grid"])
@pytest.mark.parametrize("nsrc", [1, 17, 64, 70])
def test_bc_batch_matches_fp64_oracle(kind, nsrc):
    from easy_graphit_gb300 import bc_batch
    from tests.conftest import rel_l1
    hg, g, (off, dst, _) = graph(kind)
    srcs = hg.pick_sources(nsrc, seed=13)
    dep, st = bc_batch(g, srcs)
    assert dep.dtype == np.float32 and dep.shape == (nsrc, hg.num_vertices)
    er = 0
    for i, s in enumerate(srcs):
        ref = oracle.bc(off, dst, int(s))
        assert rel_l1(dep[i], ref) <= BC_TOL, (i, rel_l1(dep[i], ref))
        er += oracle.reached_edges(off, oracle.bfs(off, dst, int(s)))
    assert st["edges_traversed"] == 2 * er


def test_bc_batch_equals_single_source_app():
    from easy_graphit_gb300 import bc, bc_batch
    from tests.conftest import rel_l1
    hg, g, (off, dst, _) = graph("sym14")
    srcs = hg.pick_sources(9, seed=21)
    dep, _ = bc_batch(g, srcs)
    for i, s in enumerate(srcs):
        one, _ = bc(g, int(s))
        assert rel_l1(dep[i], one) <= BC_TOL


def test_bc_batch_duplicate_and_isolated_sources():
    from easy_graphit_gb300 import bc_batch
    from tests.conftest import rel_l1
    # vertex 5 has no edges: its row is all zeros
    edges = [(0, 1), (1, 2), (2, 3), (3, 0), (1, 3), (4, 0)]
    src = [a for a, b in edges] + [b for a, b in edges]
    dst_ = [b for a, b in edges] + [a for a, b in edges]
    hg = HostGraph.from_edges(6, src, dst_, [1] * len(src))
    g = GraphT(hg, symmetric=True)
    off, dst = np.array(hg.offsets), np.array(hg.dst)
    dep, _ = bc_batch(g, [1, 1, 5, 0])
    for i, s in enumerate([1, 1, 5, 0]):
        ref = oracle.bc(off, dst, s)
        assert rel_l1(dep[i], ref) <= BC_TOL, (s, dep[i], ref)
    assert not dep[2].any()


def test_batch_plan_bc_replay():
    import torch
    from easy_graphit_gb300 import BatchPlan
    from tests.conftest import rel_l1
    hg, g, (off, dst, _) = graph("sym14")
    srcs = hg.pick_sources(66, seed=4)
    out = torch.full((66, hg.num_vertices), -7.0, dtype=torch.float32, device="cuda")
    plan = BatchPlan(g, "bc", srcs, out)
    for _ in range(2):
        st = plan.run()
        got = out.cpu().numpy()
        for i in [0, 40, 63, 64, 65]:
            assert rel_l1(got[i], oracle.bc(off, dst, int(srcs[i]))) <= BC_TOL
        assert st["edges_traversed"] > 0
        out.fill_(-7.0)
    plan.close()


# ------------------------------------------------------------- launch tuning
@pytest.mark.parametrize("tuning", [dict(blocks_per_sm=1), dict(chunk=32), dict(chunk=4096),
                                    dict(edge_parallel_max=-1), dict(edge_parallel_max=32),
                                    dict(blocks_per_sm=2, chunk=64, edge_parallel_max=2),
                                    dict(bottom_up_div=-1), dict(bottom_up_div=4096),
                                    dict(bottom_up_div=2, blocks_per_sm=1)])
def test_batched_results_do_not_depend_on_tuning(tuning):
    from easy_graphit_gb300 import bc_batch, set_batch_tuning
    from tests.conftest import rel_l1
    hg, g, (off, dst, w) = graph("dir14")
    srcs = hg.pick_sources(33, seed=17)
    for app in ("bfs", "sssp", "bc"):
        set_batch_tuning(g, app, **tuning)
    try:
        dist, _ = sssp_batch(g, srcs, 8)
        depth, _ = bfs_batch(g, srcs)
        dep, _ = bc_batch(g, srcs[:5])
        for i in [0, 16, 32]:
            s = int(srcs[i])
            np.testing.assert_array_equal(dist[i], oracle.sssp_dijkstra(off, dst, w, s))
            np.testing.assert_array_equal(depth[i], oracle.bfs(off, dst, s))
        for i in range(5):
            assert rel_l1(dep[i], oracle.bc(off, dst, int(srcs[i]))) <= BC_TOL
    finally:
        for app in ("bfs", "sssp", "bc"):
            set_batch_tuning(g, app)


def test_invalid_tuning_is_rejected():
    from easy_graphit_gb300 import set_batch_tuning
    hg, g, _ = graph("dir14")
    for bad in (dict(chunk=48), dict(chunk=16), dict(chunk=8192), dict(edge_parallel_max=33),
                dict(blocks_per_sm=-1), dict(bottom_up_div=5000), dict(bottom_up_div=-2)):
        with pytest.raises(Exception, match="out of range"):
            set_batch_tuning(g, "sssp", **bad)


@pytest.mark.parametrize("app", ["bfs", "sssp", "bc"])
def test_autotune_sets_the_fastest_candidate(app):
    from easy_graphit_gb300 import autotune_batch, get_batch_tuning, set_batch_tuning
    hg, g, (off, dst, w) = graph("sym14")
    srcs = hg.pick_sources(32, seed=2)
    best, rows = autotune_batch(g, app, srcs, delta=32)
    try:
        assert len(rows) >= 2 and all(ms > 0 for _, ms in rows)
        assert min(rows, key=lambda r: r[1])[0] == best
        assert get_batch_tuning(g, app) == best
        if app == "sssp":  # the tuned graph still gives exact results
            dist, _ = sssp_batch(g, srcs[:3], 32)
            for i in range(3):
                np.testing.assert_array_equal(dist[i], oracle.sssp_dijkstra(off, dst, w, int(srcs[i])))
    finally:
        set_batch_tuning(g, app)


@pytest.mark.parametrize("app", ["bfs", "sssp"])
def test_multigraph_plan_is_one_captured_launch(app):
    """The mix of uneven graphs as one multi-source traversal captured into a
    CUDA graph: replays equal the per-graph oracle results."""
    import torch
    from easy_graphit_gb300 import BatchPlan
    parts = [HostGraph.rmat(9 + i % 4, 4 + 5 * i, seed=300 + i) if i % 3 else HostGraph.grid(20 + i, 20 + i, seed=400 + i)
             for i in range(9)]
    local = [int(p.pick_sources(1, seed=i)[0]) for i, p in enumerate(parts)]
    hg, offs = HostGraph.union(parts)
    g = GraphT(hg)
    srcs = np.array([offs[i] + s for i, s in enumerate(local)], dtype=np.int32)
    out = torch.full((hg.num_vertices,), -7, dtype=torch.int32, device="cuda")
    plan = BatchPlan(g, app + "_multi", srcs, out, delta=16)
    for _ in range(2):
        st = plan.run()
        assert st["launches"] >= 1 and st["iterations"] > 0
        got = out.cpu().numpy()
        for i, (p, s) in enumerate(zip(parts, local)):
            off, dst, w = np.array(p.offsets), np.array(p.dst), np.array(p.weights)
            ref = oracle.bfs(off, dst, s) if app == "bfs" else oracle.sssp_dijkstra(off, dst, w, s)
            np.testing.assert_array_equal(got[offs[i]:offs[i + 1]], ref)
        out.fill_(-7)
    plan.close()
    g.close()


@pytest.mark.parametrize("delta", [1, 10, 1000])
def test_sssp_batch_window_from_a_settled_far_value(delta):
    """0 -> 1 costs 100 (far), but 0 -> 2 -> 1 costs 2: vertex 1's far value 100
    is the smallest one recorded when source 0 advances, though 1 was settled at
    2 meanwhile.  The window then starts at 100 and holds nothing; the next
    advance must still reach 3 (202).  Sources 4 (isolated) and a duplicate of 0
    ride along."""
    u = np.array([0, 0, 2, 1], dtype=np.int32)
    v = np.array([1, 2, 1, 3], dtype=np.int32)
    w = np.array([100, 1, 1, 200], dtype=np.int32)
    hg = HostGraph.from_edges(5, u, v, w)
    g = GraphT(hg)
    off, dst, ww = np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)
    srcs = [0, 4, 0, 2]
    dist, _ = sssp_batch(g, srcs, delta)
    np.testing.assert_array_equal(dist[0], [0, 2, 1, 202, INT_MAX])
    for i, s in enumerate(srcs):
        np.testing.assert_array_equal(dist[i], oracle.sssp_dijkstra(off, dst, ww, s))
    g.close()


@pytest.mark.parametrize("delta", [4, 64])
def test_sssp_batch_light_and_heavy_edges(delta):
    """Weights 1 or 1000 on a random graph: far values recorded through heavy
    edges are often undercut later through chains of light ones."""
    rng = np.random.default_rng(3)
    n, m = 20000, 160000
    u = rng.integers(0, n, m).astype(np.int32)
    v = rng.integers(0, n, m).astype(np.int32)
    w = np.where(rng.random(m) < 0.5, 1, 1000).astype(np.int32)
    hg = HostGraph.from_edges(n, u, v, w)
    g = GraphT(hg)
    off, dst, ww = np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)
    srcs = hg.pick_sources(32, seed=9)
    dist, _ = sssp_batch(g, srcs, delta)
    for i, s in enumerate(srcs):
        np.testing.assert_array_equal(dist[i], oracle.sssp_dijkstra(off, dst, ww, int(s)),
                                      err_msg=f"source {s}")
    g.close()


@pytest.mark.parametrize("delta", [1, 32, 1000])
def test_sssp_one_cta_per_source_forced_on_a_graph_with_hubs(delta):
    """The per-source form (one CTA per source, bucket ring) forced onto a
    directed R-MAT 12 (hubs of hundreds of edges; at delta 1000 one window
    holds most of the graph): ring slots fill and spill, relax lists overflow
    into the per-step queue, edge ranges exceed a group of four -- the
    distances still equal Dijkstra's, and equal the lane-per-source kernel's."""
    from easy_graphit_gb300 import set_batch_tuning
    hg = HostGraph.rmat(12, 16)
    g = GraphT(hg)
    off, dst, w = np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)
    srcs = hg.pick_sources(8, seed=5)
    set_batch_tuning(g, "sssp", per_source_cta=1)
    cta, _ = sssp_batch(g, srcs, delta)
    set_batch_tuning(g, "sssp", per_source_cta=-1)
    lane, _ = sssp_batch(g, srcs, delta)
    np.testing.assert_array_equal(cta, lane)
    for i, s in enumerate(srcs):
        np.testing.assert_array_equal(cta[i], oracle.sssp_dijkstra(off, dst, w, int(s)), err_msg=f"source {s}")
    g.close()
