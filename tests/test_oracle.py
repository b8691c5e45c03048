"""The oracle against the reference's golden data and hand-computed answers (CPU)."""
import numpy as np
import pytest

import oracle
from tests.conftest import INT_MAX, rel_l1

DELTAS = [1, 8, 32, 128]


def _g(golden, name):
    from easy_graphit_gb300 import HostGraph
    scale, deg, sym = {"rmat10_k16_sym": (10, 16, True), "rmat12_k16_dir": (12, 16, False)}[name]
    hg = HostGraph.rmat(scale, deg, symmetrize=sym)
    return np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)


GOLDEN_GRAPHS = {"rmat10_k16_sym": (10, 16, True), "rmat11_k8_dir": (11, 8, False),
                 "rmat12_k16_dir": (12, 16, False), "rmat12_k16_sym": (12, 16, True),
                 "rmat14_k16_dir": (14, 16, False)}


@pytest.mark.parametrize("name", sorted(GOLDEN_GRAPHS))
def test_oracle_rmat_generator_matches_reference_builder(golden, name):
    """The oracle's own restatement of GAPBS's generator and builder (used by the
    benchmark's CPU legs) against the CSR digests made by the reference's code."""
    import hashlib
    scale, deg, sym = GOLDEN_GRAPHS[name]
    off, dst, w = oracle.rmat(scale, deg, sym)
    assert len(off) - 1 == int(golden[f"graph/{name}/V"])
    assert len(dst) == int(golden[f"graph/{name}/E"])
    h = hashlib.sha256()
    for a in (off, dst, w):
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    assert h.hexdigest() == str(golden[f"graph/{name}/sha256"])


def test_oracle_rmat_small_full_arrays(golden):
    off, dst, w = oracle.rmat(10, 16, True)
    np.testing.assert_array_equal(off, golden["graph_small/offsets"])
    np.testing.assert_array_equal(dst, golden["graph_small/dst"])
    np.testing.assert_array_equal(w, golden["graph_small/w"])


@pytest.mark.parametrize("name", ["rmat10_k16_sym", "rmat12_k16_dir"])
@pytest.mark.parametrize("delta", DELTAS)
def test_sssp_oracles_match_reference(golden, name, delta):
    off, dst, w = _g(golden, name)
    ref = golden[f"sssp/{name}/d{delta}"]
    for i, s in enumerate(golden[f"sources/{name}"]):
        np.testing.assert_array_equal(oracle.sssp_dijkstra(off, dst, w, int(s)), ref[i])
        d, adv = oracle.sssp_delta_gpu(off, dst, w, int(s), delta)
        np.testing.assert_array_equal(d, ref[i])
        assert adv >= 1
        np.testing.assert_array_equal(oracle.sssp_ordered(off, dst, w, int(s), delta, 4), ref[i])


@pytest.mark.parametrize("name", ["rmat10_k16_sym", "rmat12_k16_dir"])
def test_bfs_oracle_matches_reference_unit_weight_sssp(golden, name):
    off, dst, _ = _g(golden, name)
    ref = golden[f"bfs/{name}"]
    for i, s in enumerate(golden[f"sources/{name}"]):
        np.testing.assert_array_equal(oracle.bfs(off, dst, int(s)), ref[i])
        np.testing.assert_array_equal(oracle.bfs_omp(off, dst, int(s), 4), ref[i])


def test_bfs_parent_checker_catches_bad_parent(golden):
    off, dst, _ = _g(golden, "rmat10_k16_sym")
    s = int(golden["sources/rmat10_k16_sym"][0])
    depth = oracle.bfs(off, dst, s)
    # Build a valid parent array on the CPU, then plant one mistake.
    parent = np.full(len(depth), -1, dtype=np.int32)
    parent[s] = s
    for u in range(len(depth)):
        for k in range(off[u], off[u + 1]):
            v = dst[k]
            if depth[v] == depth[u] + 1 and parent[v] == -1:
                parent[v] = u
    assert oracle.bfs_check_parent(off, dst, s, depth, parent) == 0
    v = int(np.where(depth == 2)[0][0])
    parent[v] = s
    assert oracle.bfs_check_parent(off, dst, s, depth, parent) == 1


def _csr(V, edges, sym=False):
    from easy_graphit_gb300 import HostGraph
    u = [a for a, b in edges]
    v = [b for a, b in edges]
    hg = HostGraph.from_edges(V, u, v, symmetrize=sym)
    return np.array(hg.offsets), np.array(hg.dst)


def test_pagerank_known_answers():
    off, dst = _csr(3, [(0, 1), (1, 2), (2, 0)])
    np.testing.assert_allclose(oracle.pagerank(off, dst, 20), [1 / 3] * 3, rtol=1e-12)
    off, dst = _csr(2, [(0, 1)])  # vertex 1 is a sink: no dangling redistribution
    r1 = oracle.pagerank(off, dst, 1)
    np.testing.assert_allclose(r1, [0.075, 0.075 + 0.85 * 0.5], rtol=1e-12)
    r2 = oracle.pagerank(off, dst, 2)
    np.testing.assert_allclose(r2, [0.075, 0.075 + 0.85 * 0.075], rtol=1e-12)


def test_cc_known_answers():
    off, dst = _csr(6, [(2, 1), (1, 0), (4, 3)])
    np.testing.assert_array_equal(oracle.cc(off, dst), [0, 0, 0, 3, 3, 5])
    lab, rounds = oracle.cc_labelprop(off, dst)
    np.testing.assert_array_equal(lab, [0, 0, 0, 3, 3, 5])
    assert rounds >= 1


@pytest.mark.parametrize("name", ["rmat10_k16_sym", "rmat12_k16_dir"])
def test_cc_labelprop_restatement_equals_union_find(golden, name):
    off, dst, _ = _g(golden, name)
    lab, _ = oracle.cc_labelprop(off, dst)
    np.testing.assert_array_equal(lab, oracle.cc(off, dst))
    np.testing.assert_array_equal(oracle.cc_omp(off, dst, 4), oracle.cc(off, dst))


def test_bc_known_answers():
    off, dst = _csr(3, [(0, 1), (1, 2)], sym=True)  # path 0-1-2
    np.testing.assert_allclose(oracle.bc(off, dst, 0), [2, 1, 0])
    off, dst = _csr(4, [(0, 1), (0, 2), (0, 3)], sym=True)  # star, source = leaf 1
    np.testing.assert_allclose(oracle.bc(off, dst, 1), [2, 3, 0, 0])
    off, dst = _csr(4, [(0, 1), (0, 2), (1, 3), (2, 3)], sym=True)  # diamond
    np.testing.assert_allclose(oracle.bc(off, dst, 0), [3, 0.5, 0.5, 0])
    off, dst = _csr(3, [(1, 2)], sym=True)  # isolated source
    np.testing.assert_allclose(oracle.bc(off, dst, 0), [0, 0, 0])


def test_bc_matches_brandes_dependencies(golden):
    nx = pytest.importorskip("networkx")
    from networkx.algorithms.centrality import betweenness as B
    off, dst, _ = _g(golden, "rmat10_k16_sym")
    G = nx.DiGraph()
    G.add_nodes_from(range(len(off) - 1))
    for u in range(len(off) - 1):
        for k in range(off[u], off[u + 1]):
            G.add_edge(u, int(dst[k]))
    for s in golden["sources/rmat10_k16_sym"][:2]:
        s = int(s)
        S, P, sigma, _ = B._single_source_shortest_path_basic(G, s)
        acc = dict.fromkeys(G, 0.0)
        acc, _ = B._accumulate_basic(acc, S, P, sigma, s)
        ref = np.array([acc[v] for v in range(len(off) - 1)])
        got = oracle.bc(off, dst, s)
        mask = np.arange(len(ref)) != s
        assert rel_l1(got[mask], ref[mask]) < 1e-12


def test_sssp_matches_scipy(golden):
    sp = pytest.importorskip("scipy.sparse")
    csg = pytest.importorskip("scipy.sparse.csgraph")
    off, dst, w = _g(golden, "rmat12_k16_dir")
    V = len(off) - 1
    A = sp.csr_matrix((w.astype(np.float64), dst, off), shape=(V, V))
    s = int(golden["sources/rmat12_k16_dir"][0])
    d = csg.dijkstra(A, indices=s)
    ref = np.where(np.isinf(d), INT_MAX, d).astype(np.int64)
    np.testing.assert_array_equal(oracle.sssp_dijkstra(off, dst, w, s), ref)


def test_shortest_path_certificate_accepts_exact_and_rejects_wrong_distances():
    from easy_graphit_gb300 import HostGraph
    from tests.conftest import shortest_paths_certified
    hg = HostGraph.rmat(10, 8)
    off, dst, w = np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)
    s = int(hg.pick_sources(1)[0])
    d = oracle.sssp_dijkstra(off, dst, w, s)
    assert shortest_paths_certified(off, dst, w, d, s)
    reached = np.flatnonzero((d != 2**31 - 1) & (np.arange(len(d)) != s))
    bad = d.copy()
    bad[reached[0]] -= 1                      # too small: no tight in-edge
    assert not shortest_paths_certified(off, dst, w, bad, s)
    bad = d.copy()
    bad[reached[-1]] += 1                     # too large: an edge improves it
    assert not shortest_paths_certified(off, dst, w, bad, s)
    assert not shortest_paths_certified(off, dst, w, np.zeros_like(d), s)


@pytest.mark.parametrize("name", ["rmat10_k16_sym", "rmat12_k16_dir"])
def test_cc_matches_scipy_weak_components(golden, name):
    """An independent implementation: scipy's weakly connected components,
    relabelled to the smallest vertex id of each component (cc.cpp's fixpoint)."""
    sp = pytest.importorskip("scipy.sparse")
    csg = pytest.importorskip("scipy.sparse.csgraph")
    off, dst, _ = _g(golden, name)
    V = len(off) - 1
    A = sp.csr_matrix((np.ones(len(dst)), dst, off), shape=(V, V))
    n, comp = csg.connected_components(A, directed=True, connection="weak")
    smallest = np.full(n, V, dtype=np.int64)
    np.minimum.at(smallest, comp, np.arange(V))
    np.testing.assert_array_equal(oracle.cc(off, dst), smallest[comp])


@pytest.mark.parametrize("name", ["rmat10_k16_sym", "rmat12_k16_dir"])
def test_pagerank_matches_sparse_power_iteration(golden, name):
    """pr.cpp's iteration written as a sparse matrix product in FP64:
    new = (1-d)/V + d * A^T (old / outdeg), 20 times, no dangling redistribution
    (a sink's contribution is never read: it has no out-edges)."""
    sp = pytest.importorskip("scipy.sparse")
    off, dst, _ = _g(golden, name)
    V = len(off) - 1
    A = sp.csr_matrix((np.ones(len(dst)), dst, off), shape=(V, V))
    outdeg = np.diff(off).astype(np.float64)
    r = np.full(V, 1.0 / V)
    for _ in range(20):
        contrib = np.divide(r, outdeg, out=np.zeros(V), where=outdeg > 0)
        r = (1.0 - 0.85) / V + 0.85 * (A.T @ contrib)
    assert rel_l1(oracle.pagerank(off, dst, 20, 0.85), r) < 1e-12


# ------------------------------------------------- the reference's own apps
@pytest.mark.parametrize("name", ["rmat10_k16_sym", "rmat11_k8_dir", "grid32"])
def test_oracle_matches_the_reference_apps(app_golden, name):
    """tests/golden/ref_apps.npz holds what easy_graphit's apps/{pr,cc,bc,bfs,
    sssp}.cpp compute when they run on the CPU (their UDFs, loops and constants;
    float vertex data in double): the oracle's restatements give the same
    values -- PageRank and BC to rounding, the integer apps exactly."""
    from tests.conftest import app_graph
    off, dst, w = app_graph(app_golden, name)
    srcs = [int(s) for s in app_golden[f"sources/{name}"]]
    # pr.cpp: damp is a float constant (0.85f), used in double here as there
    pr = oracle.pagerank(off, dst, 20, float(np.float32(0.85)))
    assert rel_l1(pr, app_golden[f"pr/{name}"]) <= 1e-12
    np.testing.assert_array_equal(oracle.cc(off, dst), app_golden[f"cc/{name}"])
    for k, s in enumerate(srcs):
        assert rel_l1(oracle.bc(off, dst, s), app_golden[f"bc/{name}/s{k}"]) <= 1e-12, (name, s)
    np.testing.assert_array_equal(oracle.bfs(off, dst, srcs[0]), app_golden[f"bfs/{name}"])
    for d in (1, 8, 32):
        want = app_golden[f"sssp/{name}/d{d}"]
        np.testing.assert_array_equal(oracle.sssp_dijkstra(off, dst, w, srcs[0]), want)
        # the bucket rule: as many window moves as sssp.cpp's own loop makes
        dist, adv = oracle.sssp_delta_gpu(off, dst, w, srcs[0], d)
        np.testing.assert_array_equal(dist, want)
        assert adv == int(app_golden[f"sssp/{name}/adv{d}"][0]), (name, d)


def test_reference_app_golden_is_not_trivial(app_golden):
    """The fixtures exercise the apps: reached sets are large, BC has nonzero
    dependencies, CC finds components, PageRank sums to about one."""
    for name in ["rmat10_k16_sym", "rmat11_k8_dir", "grid32"]:
        assert (app_golden[f"bfs/{name}"] > 1).sum() > 100
        assert (app_golden[f"sssp/{name}/d8"] != INT_MAX).sum() > 100
        assert np.abs(app_golden[f"bc/{name}/s0"]).sum() > 0
        assert 0.5 < app_golden[f"pr/{name}"].sum() <= 1.0 + 1e-9
    assert len(np.unique(app_golden["cc/rmat11_k8_dir"])) > 1


def test_reference_apps_reproduce_the_golden(app_golden, tmp_path):
    """Where the reference apps were built here (oracle/_ref/app_*, made from
    the reference tree by `make -C oracle apps`), running them again on the
    grid reproduces the stored outputs exactly."""
    from pathlib import Path

    from tests.conftest import app_graph
    ref = Path(oracle.__file__).resolve().parent / "_ref"
    if not all((ref / f"app_{a}").exists() for a in ("pr", "cc", "bc", "bfs", "sssp")):
        pytest.skip("reference apps not built here (they need the reference tree)")
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_app_golden", Path(__file__).resolve().parent / "golden" / "make_app_golden.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    off, dst, w = app_graph(app_golden, "grid32")
    gf = str(tmp_path / "grid32.graphit_bin")
    mk.write_graphit_bin(gf, off, dst, w)
    s = int(app_golden["sources/grid32"][0])
    np.testing.assert_array_equal(mk.run_app("pr", gf)["old_rank"], app_golden["pr/grid32"])
    np.testing.assert_array_equal(mk.run_app("cc", gf)["ID"], app_golden["cc/grid32"])
    np.testing.assert_array_equal(mk.run_app("bc", gf, s, 0.0)["dependences"], app_golden["bc/grid32/s0"])
    np.testing.assert_array_equal(mk.run_app("sssp", gf, s, 8)["SP"], app_golden["sssp/grid32/d8"])
    parent = mk.run_app("bfs", gf, s, 0.0)["parent"]
    np.testing.assert_array_equal(mk.depths_from_parents(parent, s), app_golden["bfs/grid32"])


def test_oracle_bfs_matches_the_reference_app_on_the_bfs_workload(app_golden):
    """The BFS workload as stated -- symmetrized R-MAT 16, edge factor 16, from
    its highest-degree vertex -- run by bfs.cpp itself: the oracle's depths are
    the same, bit for bit (the GPU's are held to the oracle on this graph)."""
    import hashlib
    off, dst, w = (np.asarray(a, dtype=np.int32) for a in oracle.rmat(16, 16, symmetrize=True))
    h = hashlib.sha256()
    for a in (off, dst, w):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(app_golden["config1/sha256"])
    src = int(app_golden["config1/source"])
    assert src == int(np.argmax(np.diff(off)))
    np.testing.assert_array_equal(oracle.bfs(off, dst, src), app_golden["config1/depth"])


def test_oracle_sssp_matches_the_reference_app_on_the_sssp_workload(app_golden):
    """The SSSP workload's directed R-MAT 22 (weights U[1,255]) from its first
    two SourcePicker sources, run by sssp.cpp itself at delta 8, 32, 128: the
    oracle's Dijkstra distances hash the same, and its restatement of the
    bucket rule makes as many window moves as the app's own queue."""
    import hashlib
    off, dst, w = (np.asarray(a, dtype=np.int32) for a in oracle.rmat(22, 16))
    h = hashlib.sha256()
    for a in (off, dst, w):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.hexdigest() == str(app_golden["config2/sha256"])
    srcs = [int(x) for x in oracle.pick_sources(off, 2)]
    assert srcs == [int(x) for x in app_golden["config2/sources"]]
    for k, s in enumerate(srcs):
        d = oracle.sssp_dijkstra(off, dst, w, s)
        assert hashlib.sha256(np.ascontiguousarray(d, dtype=np.int32).tobytes()).hexdigest() == \
            str(app_golden[f"config2/s{k}_sha256"])
        for delta in (8, 32, 128):
            dist, adv = oracle.sssp_delta_gpu(off, dst, w, s, delta)
            np.testing.assert_array_equal(dist, d)
            assert adv == int(app_golden[f"config2/s{k}_adv{delta}"][0]), (s, delta)
