"""Host-side logic of libgg.so (no GPU): graph generation and I/O, the schedule
mirror, and the C ABI's exported symbols."""
import ctypes as C
import hashlib
import re
from pathlib import Path

import numpy as np
import pytest

from easy_graphit_gb300 import HostGraph, SimpleGPUSchedule, HybridGPUSchedule, default_schedule
from easy_graphit_gb300 import _lib as L
from tests.conftest import ROOT

GRAPHS = {
    "rmat10_k16_sym": (10, 16, True),
    "rmat11_k8_dir": (11, 8, False),
    "rmat12_k16_dir": (12, 16, False),
    "rmat12_k16_sym": (12, 16, True),
    "rmat14_k16_dir": (14, 16, False),
}


def _digest(hg):
    h = hashlib.sha256()
    for a in (hg.offsets, hg.dst, hg.weights):
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("name", sorted(GRAPHS))
def test_rmat_generator_matches_reference_builder(golden, name):
    scale, deg, sym = GRAPHS[name]
    hg = HostGraph.rmat(scale, deg, symmetrize=sym)
    assert hg.num_vertices == int(golden[f"graph/{name}/V"])
    assert hg.num_edges == int(golden[f"graph/{name}/E"])
    assert _digest(hg) == str(golden[f"graph/{name}/sha256"])


def test_rmat_small_full_arrays(golden):
    hg = HostGraph.rmat(10, 16, symmetrize=True)
    np.testing.assert_array_equal(hg.offsets, golden["graph_small/offsets"])
    np.testing.assert_array_equal(hg.dst, golden["graph_small/dst"])
    np.testing.assert_array_equal(hg.weights, golden["graph_small/w"])


def test_csr_invariants_and_determinism():
    a = HostGraph.rmat(12, 8, symmetrize=True)
    b = HostGraph.rmat(12, 8, symmetrize=True)
    assert _digest(a) == _digest(b)
    off, dst, w = a.offsets, a.dst, a.weights
    for v in range(a.num_vertices):
        nb = dst[off[v]:off[v + 1]]
        assert np.all(np.diff(nb) > 0)  # sorted, no duplicates
        assert v not in nb               # no self-loops
    assert w.min() >= 1 and w.max() <= 255
    # symmetric: every edge has its reverse with the same weight
    E = {(u, int(x)): int(ww) for u in range(a.num_vertices)
         for x, ww in zip(dst[off[u]:off[u + 1]], w[off[u]:off[u + 1]])}
    assert all(E.get((v, u)) == ww for (u, v), ww in E.items())


def test_rmat_seed_and_skew_change_the_graph():
    a = HostGraph.rmat(10, 8)
    b = HostGraph.rmat(10, 8, seed=1)
    c = HostGraph.rmat(10, 8, a=0.45, b=0.25, c=0.25)
    assert _digest(a) != _digest(b) and _digest(a) != _digest(c)


def test_grid_generator():
    g = HostGraph.grid(5, 7, wmin=1, wmax=1000)
    assert g.num_vertices == 35
    assert g.num_edges == 2 * (5 * 6 + 4 * 7)
    off, dst, w = g.offsets, g.dst, g.weights
    deg = np.diff(off)
    assert deg[0] == 2 and deg[8] == 4 and deg[1] == 3
    np.testing.assert_array_equal(dst[off[8]:off[9]], [1, 7, 9, 15])
    assert w.min() >= 1 and w.max() <= 1000
    assert _digest(g) == _digest(HostGraph.grid(5, 7, wmin=1, wmax=1000))


def test_from_edges_squish_semantics():
    # duplicates keep the smallest weight, self-loops vanish, lists sorted
    hg = HostGraph.from_edges(4, [0, 0, 0, 2, 1], [3, 1, 3, 2, 0], [9, 5, 4, 7, 1])
    np.testing.assert_array_equal(hg.offsets, [0, 2, 3, 3, 3])
    np.testing.assert_array_equal(hg.dst, [1, 3, 0])
    np.testing.assert_array_equal(hg.weights, [5, 4, 1])
    sym = HostGraph.from_edges(3, [0], [2], [6], symmetrize=True)
    np.testing.assert_array_equal(sym.offsets, [0, 1, 1, 2])
    np.testing.assert_array_equal(sym.dst, [2, 0])


def test_graphit_bin_roundtrip(tmp_path):
    hg = HostGraph.rmat(9, 8)
    p = tmp_path / "g.int.graphit_bin"
    hg.save_bin(str(p))
    raw = np.fromfile(p, dtype=np.int32)
    V, E = int(raw[0]), int(raw[1])
    assert (V, E) == (hg.num_vertices, hg.num_edges)
    # [V][E][src E][dst E][w E][offsets V+1]  (graph.h:295-302)
    np.testing.assert_array_equal(raw[2:2 + E], np.repeat(np.arange(V), np.diff(hg.offsets)))
    np.testing.assert_array_equal(raw[2 + E:2 + 2 * E], hg.dst)
    np.testing.assert_array_equal(raw[2 + 3 * E:], hg.offsets)
    back = HostGraph.load(str(p))
    assert _digest(back) == _digest(hg)


def test_graphit_bin_truncated_and_corrupt(tmp_path):
    hg = HostGraph.rmat(8, 4)
    p = tmp_path / "g.graphit_bin"
    hg.save_bin(str(p))
    data = p.read_bytes()
    (tmp_path / "t.graphit_bin").write_bytes(data[:-4])
    with pytest.raises(L.GGError) as e:
        HostGraph.load(str(tmp_path / "t.graphit_bin"))
    assert e.value.status == L.GG_ERR_IO
    bad = bytearray(data)
    E = hg.num_edges
    bad[8 + 4 * E: 8 + 4 * E + 4] = np.int32(10**6).tobytes()  # dst[0] out of range
    (tmp_path / "c.graphit_bin").write_bytes(bytes(bad))
    with pytest.raises(L.GGError) as e:
        HostGraph.load(str(tmp_path / "c.graphit_bin"))
    assert e.value.status == L.GG_ERR_IO
    with pytest.raises(L.GGError) as e:
        HostGraph.load(str(tmp_path / "missing.graphit_bin"))
    assert e.value.status == L.GG_ERR_IO


def _gapbs_sg(path, directed, V, out_lists, in_lists=None, weighted=False):
    """Writes GAPBS's serialized layout by hand (writer.h:39-70): [bool directed]
    [i64 E][i64 V][i64 offsets[V+1]][neighbours] (+ the in-lists if directed)."""
    def block(lists):
        off = np.zeros(V + 1, dtype=np.int64)
        off[1:] = np.cumsum([len(l) for l in lists])
        if weighted:
            nb = np.array([x for l in lists for pair in l for x in pair], dtype=np.int32)
        else:
            nb = np.array([x for l in lists for x in l], dtype=np.int32)
        return off.tobytes() + nb.tobytes()
    E = sum(len(l) for l in out_lists)
    data = bytes([1 if directed else 0]) + np.int64(E).tobytes() + np.int64(V).tobytes() + block(out_lists)
    if directed:
        data += block(in_lists)
    path.write_bytes(data)


def test_gapbs_serialized_graphs_by_hand(tmp_path):
    # directed 0->1, 0->2, 2->1 ; in-lists 1:{0,2} 2:{0}
    _gapbs_sg(tmp_path / "d.sg", True, 3, [[1, 2], [], [1]], [[], [0, 2], [0]])
    g = HostGraph.load(str(tmp_path / "d.sg"))
    np.testing.assert_array_equal(g.offsets, [0, 2, 2, 3])
    np.testing.assert_array_equal(g.dst, [1, 2, 1])
    np.testing.assert_array_equal(g.weights, [1, 1, 1])
    _gapbs_sg(tmp_path / "u.wsg", False, 3, [[(1, 7)], [(0, 7), (2, 4)], [(1, 4)]], weighted=True)
    g = HostGraph.load(str(tmp_path / "u.wsg"))
    np.testing.assert_array_equal(g.offsets, [0, 1, 3, 4])
    np.testing.assert_array_equal(g.dst, [1, 0, 2, 1])
    np.testing.assert_array_equal(g.weights, [7, 7, 4, 4])


@pytest.mark.parametrize("suffix,directed", [(".sg", True), (".wsg", True), (".wsg", False)])
def test_gapbs_serialized_roundtrip(tmp_path, suffix, directed):
    hg = HostGraph.rmat(9, 8, symmetrize=not directed)
    p = tmp_path / ("g" + suffix)
    hg.save_sg(str(p), directed=directed)
    back = HostGraph.load(str(p))
    np.testing.assert_array_equal(back.offsets, hg.offsets)
    np.testing.assert_array_equal(back.dst, hg.dst)
    if suffix == ".wsg":
        np.testing.assert_array_equal(back.weights, hg.weights)
    else:
        assert np.all(back.weights == 1)
    raw = p.read_bytes()
    assert raw[0] == int(directed)
    V, E = hg.num_vertices, hg.num_edges
    nb = 8 if suffix == ".wsg" else 4
    assert len(raw) == 17 + (8 * (V + 1) + nb * E) * (2 if directed else 1)
    if directed:  # the stored in-lists are the transpose
        o = 17 + 8 * (V + 1) + nb * E
        in_off = np.frombuffer(raw, dtype=np.int64, count=V + 1, offset=o)
        np.testing.assert_array_equal(np.diff(in_off), np.bincount(hg.dst, minlength=V))


def test_gapbs_serialized_truncated_and_corrupt(tmp_path):
    hg = HostGraph.rmat(8, 4)
    p = tmp_path / "g.sg"
    hg.save_sg(str(p), directed=False)
    data = p.read_bytes()
    (tmp_path / "t.sg").write_bytes(data[:-4])
    with pytest.raises(L.GGError) as e:
        HostGraph.load(str(tmp_path / "t.sg"))
    assert e.value.status == L.GG_ERR_IO
    bad = bytearray(data)
    V = hg.num_vertices
    o = 17 + 8 * (V + 1)
    bad[o:o + 4] = np.int32(V + 5).tobytes()  # first neighbour out of range
    (tmp_path / "c.sg").write_bytes(bytes(bad))
    with pytest.raises(L.GGError) as e:
        HostGraph.load(str(tmp_path / "c.sg"))
    assert e.value.status == L.GG_ERR_IO
    bad = bytearray(data)
    bad[17 + 8:17 + 16] = np.int64(10**9).tobytes()  # offsets not monotone
    (tmp_path / "m.sg").write_bytes(bytes(bad))
    with pytest.raises(L.GGError) as e:
        HostGraph.load(str(tmp_path / "m.sg"))
    assert e.value.status == L.GG_ERR_IO


def test_text_readers(tmp_path):
    (tmp_path / "a.el").write_text("0 1\n1 2\n2 0\n1 1\n0 1\n")
    g = HostGraph.load(str(tmp_path / "a.el"))
    np.testing.assert_array_equal(g.offsets, [0, 1, 2, 3])
    np.testing.assert_array_equal(g.weights, [1, 1, 1])
    (tmp_path / "a.wel").write_text("0 1 5\n0 1 3\n1 0 7\n")
    g = HostGraph.load(str(tmp_path / "a.wel"))
    np.testing.assert_array_equal(g.dst, [1, 0])
    np.testing.assert_array_equal(g.weights, [3, 7])
    (tmp_path / "a.gr").write_text("c comment\np sp 3 2\na 1 2 4\na 2 3 6\n")
    g = HostGraph.load(str(tmp_path / "a.gr"))
    assert g.num_vertices == 4  # DIMACS ids kept as written (reader.h:74-87)
    (tmp_path / "a.mtx").write_text("%%MatrixMarket matrix coordinate integer symmetric\n% c\n3 3 2\n1 2 4\n2 3 6\n")
    g = HostGraph.load(str(tmp_path / "a.mtx"))
    np.testing.assert_array_equal(g.offsets, [0, 1, 3, 4])
    np.testing.assert_array_equal(g.dst, [1, 0, 2, 1])
    (tmp_path / "bad.el").write_text("0 x\n")
    with pytest.raises(L.GGError):
        HostGraph.load(str(tmp_path / "bad.el"))


def test_schedule_mirror_defaults():
    s = SimpleGPUSchedule()
    c = L.gg_schedule()
    L.lib().gg_schedule_init(C.byref(c))
    assert bytes(s.to_c()) == bytes(c)
    T = SimpleGPUSchedule
    assert [e.value for e in T.load_balancing_type] == list(range(8))
    assert T.load_balancing_type.EDGE_ONLY == 6 and T.direction_type.PULL == 1
    s.configDirection(T.direction_type.PULL, T.pull_frontier_rep_type.BITMAP)
    assert s.pull_frontier_rep == T.pull_frontier_rep_type.BITMAP
    s.configLoadBalancing(T.load_balancing_type.EDGE_ONLY, T.edge_blocking_type.BLOCKED, 0x42000)
    assert s.block_size == 0x42000
    h = HybridGPUSchedule(T(), s).configThreshold(0.25)
    assert h.threshold == 0.25
    for app in ["bfs", "sssp", "pr", "cc", "bc"]:
        default_schedule(app)
    sch, fuse = default_schedule("bfs")
    assert sch.load_balancing == T.load_balancing_type.TWCE and fuse


def test_abi_exports_every_declared_symbol():
    header = (ROOT / "include" / "gg.h").read_text()
    body = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    names = set(re.findall(r"\b(gg_[a-z0-9_]+)\s*\(", body))
    assert len(names) > 40
    lib = C.CDLL(str(L.LIB_PATH))
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(L.SIGNATURES) == names


def test_errors_are_reported_not_fatal():
    h = C.c_void_p()
    st = L.lib().gg_host_graph_rmat(0, 16, 0.57, 0.19, 0.19, 1, 0, 1, 255, C.byref(h))
    assert st == L.GG_ERR_INVALID
    assert "scale" in L.last_error()


def test_host_graph_union():
    a = HostGraph.rmat(6, 4)
    b = HostGraph.grid(3, 4)
    u, offs = HostGraph.union([a, b])
    assert list(offs) == [0, a.num_vertices, a.num_vertices + b.num_vertices]
    assert u.num_edges == a.num_edges + b.num_edges
    np.testing.assert_array_equal(u.dst[:a.num_edges], a.dst)
    np.testing.assert_array_equal(u.dst[a.num_edges:], b.dst + a.num_vertices)
    np.testing.assert_array_equal(u.weights[a.num_edges:], b.weights)
    np.testing.assert_array_equal(np.diff(u.offsets), np.concatenate([np.diff(a.offsets), np.diff(b.offsets)]))
