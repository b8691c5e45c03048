"""Python mirror of the GraphIt GPU algorithm and scheduling API.

Names follow easy_graphit's `include/graphit/schedule.h` (SimpleGPUSchedule,
HybridGPUSchedule and their enums/config methods), `include/graphit/operators.h`
(edgeset_apply(...).from_(...).to(...).apply / apply_modified / apply_priority,
vertexset_apply) and the runtime objects of `runtime/infra_gpu/` (GraphT,
VertexFrontier, GPUPriorityQueue, VertexFrontierList).  Everything executes in
libgg.so on the GPU; this module only marshals arguments.
"""
from __future__ import annotations

import ctypes as C
import weakref
from enum import IntEnum
from pathlib import Path
from typing import Optional

import numpy as np

from . import _lib as L
from ._lib import call, lib


# --------------------------------------------------------------- schedules
class SimpleGPUSchedule:
    """graphit::SimpleGPUSchedule (schedule.h:26-118)."""

    default_max_cta = 60   # schedule.cpp:6
    default_cta_size = 512  # schedule.cpp:5

    class direction_type(IntEnum):
        PUSH = 0
        PULL = 1

    class pull_frontier_rep_type(IntEnum):
        BITMAP = 0
        BOOLMAP = 1

    class frontier_creation_type(IntEnum):
        SPARSE = 0
        BITMAP = 1
        BOOLMAP = 2

    class deduplication_type(IntEnum):
        DISABLED = 0
        ENABLED = 1

    class deduplication_strategy_type(IntEnum):
        FUSED = 0
        UNFUSED = 1

    class load_balancing_type(IntEnum):
        VERTEX_BASED = 0
        TWC = 1
        TWCE = 2
        WM = 3
        CM = 4
        STRICT = 5
        EDGE_ONLY = 6
        ETWC = 7  # not in the reference enum

    class edge_blocking_type(IntEnum):
        BLOCKED = 0
        UNBLOCKED = 1

    class kernel_fusion_type(IntEnum):
        DISABLED = 0
        ENABLED = 1

    def __init__(self):
        T = SimpleGPUSchedule
        self.direction = T.direction_type.PUSH
        self.load_balancing = T.load_balancing_type.VERTEX_BASED
        self.edge_blocking = T.edge_blocking_type.UNBLOCKED
        self.frontier_creation = T.frontier_creation_type.SPARSE
        self.pull_frontier_rep = T.pull_frontier_rep_type.BOOLMAP
        self.deduplication = T.deduplication_type.DISABLED
        self.deduplication_strategy = T.deduplication_strategy_type.FUSED
        self.kernel_fusion = T.kernel_fusion_type.DISABLED
        self.block_size = -1
        self.max_cta = T.default_max_cta
        self.cta_size = T.default_cta_size

    def configDirection(self, dir, pf=None):
        self.direction = SimpleGPUSchedule.direction_type(dir)
        if self.direction == SimpleGPUSchedule.direction_type.PULL:
            self.pull_frontier_rep = SimpleGPUSchedule.pull_frontier_rep_type(
                SimpleGPUSchedule.pull_frontier_rep_type.BOOLMAP if pf is None else pf)
        return self

    def configFrontierCreation(self, fc):
        self.frontier_creation = SimpleGPUSchedule.frontier_creation_type(fc)
        return self

    def configDeduplication(self, dedup, strategy=None):
        self.deduplication = SimpleGPUSchedule.deduplication_type(dedup)
        if strategy is not None:
            self.deduplication_strategy = SimpleGPUSchedule.deduplication_strategy_type(strategy)
        return self

    def configLoadBalancing(self, lb, eb=None, bs=-1):
        self.load_balancing = SimpleGPUSchedule.load_balancing_type(lb)
        if self.load_balancing == SimpleGPUSchedule.load_balancing_type.EDGE_ONLY:
            self.edge_blocking = SimpleGPUSchedule.edge_blocking_type(
                SimpleGPUSchedule.edge_blocking_type.UNBLOCKED if eb is None else eb)
            self.block_size = bs
        return self

    def configKernelFusion(self, kf):
        self.kernel_fusion = SimpleGPUSchedule.kernel_fusion_type(kf)
        return self

    def to_c(self) -> L.gg_schedule:
        return L.gg_schedule(int(self.direction), int(self.pull_frontier_rep),
                             int(self.frontier_creation), int(self.deduplication),
                             int(self.deduplication_strategy), int(self.load_balancing),
                             int(self.edge_blocking), int(self.block_size),
                             int(self.kernel_fusion), int(self.max_cta), int(self.cta_size))

    def __repr__(self):
        return (f"SimpleGPUSchedule({self.direction.name}, {self.load_balancing.name}, "
                f"creation={self.frontier_creation.name}, pull_rep={self.pull_frontier_rep.name}, "
                f"blocking={self.edge_blocking.name}:{self.block_size}, cta={self.cta_size})")


class HybridGPUSchedule:
    """graphit::HybridGPUSchedule (schedule.h:122-139): s1 when
    |frontier| <= threshold * V, else s2 (operators.cpp:526).

    configThreshold(t) fixes the threshold; bindThreshold(ref) binds it to a
    value the caller keeps changing (schedule.cpp:9-12 binds a dyn_var<float>):
    a one-element list or array, a ctypes float, or a callable, read every
    time the schedule decides."""

    def __init__(self, s1: SimpleGPUSchedule, s2: SimpleGPUSchedule):
        self.s1, self.s2 = s1, s2
        self._static = 0.0
        self._bound = None

    def configThreshold(self, t: float):
        self._static = float(t)
        self._bound = None
        return self

    def bindThreshold(self, ref):
        if isinstance(ref, (int, float)):  # a plain number cannot be rebound later: same as config
            return self.configThreshold(ref)
        self._bound = ref
        return self

    @property
    def threshold(self) -> float:
        r = self._bound
        if r is None:
            return self._static
        if callable(r):
            return float(r())
        if hasattr(r, "value"):
            return float(r.value)
        return float(r[0])


D, LB, FC, PR_ = (SimpleGPUSchedule.direction_type, SimpleGPUSchedule.load_balancing_type,
                  SimpleGPUSchedule.frontier_creation_type, SimpleGPUSchedule.pull_frontier_rep_type)


class LearnedGPUSchedule:
    """Per-iteration schedule from the learned selector; `fallback` (the
    hand-written GraphIt schedule) is used when no selector is attached.
    Unfused, each iteration's (direction, load balancing, frontier) comes from
    the network on the host.  Fused (BFS): one persistent loop pushes with the
    fallback's load balancing or pulls, level by level, as the network's
    direction head decides on the device (Selector.pretrained_fused_bfs() is
    trained for that loop)."""

    def __init__(self, selector: "Selector", fallback: SimpleGPUSchedule | None = None):
        self.selector = selector
        self.fallback = fallback or SimpleGPUSchedule().configLoadBalancing(
            SimpleGPUSchedule.load_balancing_type.TWCE)


def app_schedule(s, fuse: bool = False) -> L.gg_app_schedule:
    a = L.gg_app_schedule()
    a.fuse = int(bool(fuse))
    if isinstance(s, LearnedGPUSchedule):
        a.kind = 2
        a.s1 = s.fallback.to_c()
        a.s2 = s.fallback.to_c()
        a.selector = s.selector._h if s.selector is not None else None
        return a
    if isinstance(s, HybridGPUSchedule):
        a.kind = 1
        a.s1, a.s2, a.threshold = s.s1.to_c(), s.s2.to_c(), s.threshold
    else:
        s = s or SimpleGPUSchedule()
        a.kind = 0
        a.s1 = s.to_c()
        a.s2 = s.to_c()
    return a


def default_schedule(app: str, power: bool = False, threshold: float = 0.12):
    """The schedules chosen in each app's main() (apps/*.cpp) as
    (schedule, fuse).  `power` selects the alternative ("power") schedule."""
    def s():
        return SimpleGPUSchedule()
    if app == "bfs":  # bfs.cpp:69-92
        if power:
            s1 = s().configDirection(D.PUSH).configLoadBalancing(LB.TWCE)
            s2 = (s().configDirection(D.PULL, PR_.BITMAP).configLoadBalancing(LB.VERTEX_BASED)
                  .configFrontierCreation(FC.BITMAP))
            return HybridGPUSchedule(s1, s2).bindThreshold(threshold), False
        return s().configDirection(D.PUSH).configLoadBalancing(LB.TWCE), True
    if app == "sssp":  # sssp.cpp:65-83
        if power:
            return (s().configDirection(D.PUSH).configLoadBalancing(LB.TWCE)
                    .configFrontierCreation(FC.BOOLMAP)), False
        return s().configDirection(D.PUSH).configFrontierCreation(FC.SPARSE), True
    if app == "pr":  # pr.cpp:79-81
        return (s().configDirection(D.PULL).configLoadBalancing(
            LB.EDGE_ONLY, SimpleGPUSchedule.edge_blocking_type.BLOCKED, 0x42000)), False
    if app == "cc":  # cc.cpp:86-88
        return s().configDirection(D.PUSH).configLoadBalancing(LB.EDGE_ONLY), False
    if app == "bc":  # bc.cpp:131-156
        if power:
            s1 = s().configDirection(D.PUSH).configLoadBalancing(LB.TWCE)
            s2 = (s().configDirection(D.PULL, PR_.BITMAP).configLoadBalancing(LB.TWCE)
                  .configFrontierCreation(FC.BITMAP))
            return HybridGPUSchedule(s1, s2).bindThreshold(threshold), False
        return s().configDirection(D.PUSH).configLoadBalancing(LB.TWCE), True
    raise ValueError(f"unknown app {app!r}")


# ------------------------------------------------------------------ graphs
K_RAND_SEED = 27491095  # GAPBS kRandSeed (infra_gapbs/util.h:22)


def _np_ptr(a: Optional[np.ndarray]):
    return None if a is None else C.c_void_p(a.ctypes.data)


class HostGraph:
    """Host CSR built like GAPBS's builder (sorted, deduplicated, no self-loops)."""

    def __init__(self, handle: C.c_void_p):
        self._h = handle

    @classmethod
    def _make(cls, fn: str, *args) -> "HostGraph":
        h = C.c_void_p()
        call(fn, *args, C.byref(h))
        return cls(h)

    @classmethod
    def rmat(cls, scale: int, degree: int = 16, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, seed: int = K_RAND_SEED, symmetrize: bool = False,
             wmin: int = 1, wmax: int = 255) -> "HostGraph":
        return cls._make("gg_host_graph_rmat", scale, degree, a, b, c, seed, int(symmetrize),
                         wmin, wmax)

    @classmethod
    def grid(cls, rows: int, cols: int, seed: int = K_RAND_SEED, wmin: int = 1,
             wmax: int = 1000) -> "HostGraph":
        return cls._make("gg_host_graph_grid", rows, cols, seed, wmin, wmax)

    @classmethod
    def from_edges(cls, num_vertices: int, u, v, w=None, symmetrize: bool = False) -> "HostGraph":
        u = np.ascontiguousarray(u, dtype=np.int32)
        v = np.ascontiguousarray(v, dtype=np.int32)
        w = None if w is None else np.ascontiguousarray(w, dtype=np.int32)
        return cls._make("gg_host_graph_from_edges", num_vertices, len(u), _np_ptr(u), _np_ptr(v),
                         _np_ptr(w), int(symmetrize))

    @classmethod
    def from_csr(cls, offsets, dst, weights=None) -> "HostGraph":
        off = np.ascontiguousarray(offsets, dtype=np.int32)
        dst = np.ascontiguousarray(dst, dtype=np.int32)
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.int32)
        return cls._make("gg_host_graph_from_csr", len(off) - 1, len(dst), _np_ptr(off),
                         _np_ptr(dst), _np_ptr(w))

    @classmethod
    def load(cls, path: str, symmetrize: bool = False) -> "HostGraph":
        return cls._make("gg_host_graph_load", str(path).encode(), int(symmetrize))

    def save_sg(self, path: str, directed: bool = True) -> None:
        """GAPBS serialized graph: .sg (ids) or .wsg (ids and weights)."""
        call("gg_host_graph_save_sg", self._h, str(path).encode(), int(directed))

    def save_bin(self, path: str) -> None:
        call("gg_host_graph_save_bin", self._h, str(path).encode())

    @property
    def num_vertices(self) -> int:
        v, e = C.c_int32(), C.c_int64()
        call("gg_host_graph_info", self._h, C.byref(v), C.byref(e))
        return v.value

    @property
    def num_edges(self) -> int:
        v, e = C.c_int32(), C.c_int64()
        call("gg_host_graph_info", self._h, C.byref(v), C.byref(e))
        return e.value

    def _view(self, fn: str, n: int) -> np.ndarray:
        p = getattr(lib(), fn)(self._h)
        if n == 0:
            return np.zeros(0, dtype=np.int32)
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_int32)), shape=(n,))

    @property
    def offsets(self) -> np.ndarray:
        """Zero-copy view (valid while this object lives)."""
        return self._view("gg_host_graph_offsets", self.num_vertices + 1)

    @property
    def dst(self) -> np.ndarray:
        return self._view("gg_host_graph_dst", self.num_edges)

    @property
    def weights(self) -> np.ndarray:
        return self._view("gg_host_graph_weights", self.num_edges)

    def out_degrees(self) -> np.ndarray:
        return np.diff(self.offsets)

    @classmethod
    def union(cls, parts) -> tuple["HostGraph", np.ndarray]:
        """Disjoint union; returns (graph, vertex_offsets[len(parts)+1])."""
        arr = (C.c_void_p * len(parts))(*[p._h for p in parts])
        offs = np.empty(len(parts) + 1, dtype=np.int32)
        h = C.c_void_p()
        call("gg_host_graph_union", arr, len(parts), _np_ptr(offs), C.byref(h))
        return cls(h), offs

    @staticmethod
    def mix_spec(count: int = 64, seed: int = K_RAND_SEED) -> np.ndarray:
        """[count, 3] rows (0 R-MAT | 1 grid, scale | side, edge factor | 0) of the
        batched mode's mix of uneven graphs, drawn from std::mt19937(seed)."""
        spec = np.empty((count, 3), dtype=np.int32)
        call("gg_host_graph_mix_spec", seed, count, _np_ptr(spec))
        return spec

    @classmethod
    def mix(cls, count: int = 64, seed: int = K_RAND_SEED, symmetrize: bool = False) -> list["HostGraph"]:
        """The graphs of mix_spec(count, seed); graph i uses generator seed
        seed + 1 + i (grids are symmetric by construction)."""
        out = []
        for i, (kind, size, ef) in enumerate(cls.mix_spec(count, seed)):
            if kind == 1:
                out.append(cls.grid(int(size), int(size), seed=seed + 1 + i))
            else:
                out.append(cls.rmat(int(size), int(ef), seed=seed + 1 + i, symmetrize=symmetrize))
        return out

    def pick_sources(self, n: int, seed: int = K_RAND_SEED) -> np.ndarray:
        """GAPBS SourcePicker (benchmark.h:50-71): n non-zero-degree vertices."""
        out = np.empty(n, dtype=np.int32)
        call("gg_host_graph_pick_sources", self._h, n, seed, _np_ptr(out))
        return out

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and lib is not None:
            try:
                lib().gg_host_graph_destroy(h)
            except Exception:
                pass
            self._h = None


class GraphT:
    """A graph resident in HBM (graphit_runtime::GraphT<int>)."""

    def __init__(self, host: HostGraph | None = None, *, offsets=None, dst=None, weights=None,
                 symmetric: bool = False):
        if host is not None:
            offsets, dst, weights = host.offsets, host.dst, host.weights
        self._keep = (offsets, dst, weights)
        V = (offsets.numel() if hasattr(offsets, "numel") else len(offsets)) - 1
        E = dst.numel() if hasattr(dst, "numel") else len(dst)
        h = C.c_void_p()
        call("gg_graph_create", _ptr(offsets), _ptr(dst), _ptr(weights), V, E,
             1 if symmetric else 0, C.byref(h))
        self._h = h
        self._keep = None
        self._deps = weakref.WeakSet()  # frontiers, queues, lists and plans made on this graph
        self.num_vertices, self.num_edges, self.symmetric = V, E, symmetric

    @property
    def handle(self):
        return self._h

    def get_transposed_graph(self) -> "GraphT":
        call("gg_graph_transpose", self._h)
        return self

    def get_blocked_graph(self, block_size: int) -> "GraphT":
        call("gg_graph_blocked", self._h, block_size)
        return self

    def set_stream(self, stream_ptr: int | None) -> None:
        call("gg_graph_set_stream", self._h, C.c_void_p(stream_ptr) if stream_ptr else None)

    def sync(self) -> None:
        call("gg_graph_sync", self._h)

    def _adopt(self, obj) -> None:
        self._deps.add(obj)

    def close(self) -> None:
        """Releases the graph and, first, every object still open on it (their
        device memory is tied to the graph's)."""
        if getattr(self, "_h", None):
            for d in list(getattr(self, "_deps", ())):
                try:
                    d.close()
                except Exception:
                    pass
            lib().gg_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _ptr(a):
    """Raw pointer of a numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return C.c_void_p(np.ascontiguousarray(a).ctypes.data)


# ----------------------------------------------------------- vertex subsets
class VertexSubset:
    """graphit_runtime::VertexFrontier."""

    SPARSE, BITMAP, BOOLMAP = 0, 1, 2

    def __init__(self, g: GraphT, init_all: bool = False):
        self.g = g
        h = C.c_void_p()
        call("gg_frontier_create", g.handle, int(init_all), C.byref(h))
        self._h = h
        self._owned = True
        g._adopt(self)

    @classmethod
    def _view(cls, g: GraphT, handle) -> "VertexSubset":
        """A frontier owned by someone else (a priority queue's)."""
        v = cls.__new__(cls)
        v.g, v._h, v._owned = g, handle, False
        g._adopt(v)
        return v

    @property
    def handle(self):
        return self._h

    def addVertex(self, v: int) -> None:
        call("gg_frontier_add", self._h, v)

    def size(self) -> int:
        n = C.c_int32()
        call("gg_frontier_size", self._h, C.byref(n))
        return n.value

    def format(self) -> int:
        n = C.c_int32()
        call("gg_frontier_format", self._h, C.byref(n))
        return n.value

    def to_sparse(self):
        call("gg_frontier_to_sparse", self._h)

    def to_bitmap(self):
        call("gg_frontier_to_bitmap", self._h)

    def to_boolmap(self):
        call("gg_frontier_to_boolmap", self._h)

    def dedup(self):
        call("gg_frontier_dedup", self._h)

    def clear(self):
        call("gg_frontier_clear", self._h)

    def read(self) -> np.ndarray:
        n = C.c_int32()
        call("gg_frontier_read", self._h, None, 0, C.byref(n))
        out = np.empty(n.value, dtype=np.int32)
        call("gg_frontier_read", self._h, _ptr(out), n.value, C.byref(n))
        return out

    def close(self) -> None:
        # a view of a priority queue's frontier is released with the queue
        if getattr(self, "_h", None) and getattr(self, "_owned", True):
            lib().gg_frontier_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ the operators
class UDF(IntEnum):
    """Edge UDFs of the five apps (gg.h GG_UDF_*)."""
    BFS_PARENT = 0   # bfs.cpp:23-25
    SSSP_RELAX = 1   # sssp.cpp:24-27
    PR_ADD = 2       # pr.cpp:32-34
    CC_HOOK = 3      # cc.cpp:23-36
    BC_FORWARD = 4   # bc.cpp:34-36
    BC_BACKWARD = 5  # bc.cpp:52-54


class Filter(IntEnum):
    """to() filters of the apps (gg.h GG_FILTER_*)."""
    NONE = 0
    PARENT_UNSET = 1  # bfs.cpp:27-29
    UNVISITED = 2     # bc.cpp:38-40


class VUDF(IntEnum):
    """Vertex UDFs of the five apps (gg.h GG_VUDF_*)."""
    BFS_RESET = 0
    SSSP_RESET = 1
    PR_RESET = 2
    PR_CONTRIB = 3
    PR_UPDATE = 4
    CC_INIT = 5
    CC_PJUMP = 6
    BC_RESET = 7
    BC_MARK_VISITED = 8
    BC_MARK_UNVISITED = 9
    BC_BACKWARD_VERTEX = 10
    BC_FINAL = 11


class VertexData:
    """The VertexData<T> arrays the apps' UDFs touch (apps/*.cpp), as device
    tensors (or raw device addresses) by member name: parent, depth, dist,
    ids, updates, old_rank, new_rank, contrib, num_paths, dependences,
    visited; plus the scalars level, src and damping."""

    FIELDS = ("parent", "depth", "dist", "ids", "updates", "old_rank", "new_rank", "contrib",
              "num_paths", "dependences", "visited")

    def __init__(self, level: int = 0, src: int = -1, damping: float = 0.85, **arrays):
        unknown = set(arrays) - set(self.FIELDS)
        if unknown:
            raise TypeError(f"unknown vertex data {sorted(unknown)}")
        self.arrays = arrays
        self.level, self.src, self.damping = level, src, damping

    def to_c(self) -> L.gg_vertex_data:
        d = L.gg_vertex_data()
        for k, a in self.arrays.items():
            setattr(d, k, a if isinstance(a, int) else (a.data_ptr() if a is not None else None))
        d.level, d.src, d.damping = int(self.level), int(self.src), float(self.damping)
        return d


class edgeset_apply:
    """graphit::edgeset_apply (operators.h:38-178):

        edgeset_apply(s).from_(frontier).to(Filter.X).apply(g, udf, vd)
        edgeset_apply(s).from_(frontier).to(...).apply_modified(g, out, vd, udf, allow_dupes)
        edgeset_apply(s).from_(frontier).apply_priority(g, udf, pq, vd)

    A HybridGPUSchedule picks s1 when |from| <= threshold * V, else s2, at each
    call (operators.h:116-132).  `from_` is `from` in C++ (a Python keyword)."""

    def __init__(self, schedule=None):
        self.schedule = schedule if schedule is not None else SimpleGPUSchedule()
        self.from_set: Optional[VertexSubset] = None
        self.to_filter = Filter.NONE

    def from_(self, f: "VertexSubset") -> "edgeset_apply":
        self.from_set = f
        return self

    def to(self, filt) -> "edgeset_apply":
        self.to_filter = Filter(filt)
        return self

    def _simple(self, g: "GraphT") -> SimpleGPUSchedule:
        s = self.schedule
        if isinstance(s, HybridGPUSchedule):
            n = self.from_set.size() if self.from_set is not None else g.num_vertices
            return s.s1 if n <= s.threshold * g.num_vertices else s.s2
        if isinstance(s, LearnedGPUSchedule):
            return s.fallback
        return s

    def _run(self, g, udf, vd: VertexData, out, allow_dupes: bool):
        sc = self._simple(g).to_c()
        cvd = vd.to_c()
        call("gg_edgeset_apply", g.handle, C.byref(sc), int(udf), int(self.to_filter),
             self.from_set.handle if self.from_set is not None else None,
             out.handle if out is not None else None, int(bool(allow_dupes)), C.byref(cvd))

    def apply(self, g: "GraphT", udf, vd: VertexData) -> None:
        self._run(g, udf, vd, None, True)

    def apply_modified(self, g: "GraphT", to: "VertexSubset", vd: VertexData, udf,
                       allow_dupes: bool = True) -> None:
        self._run(g, udf, vd, to, allow_dupes)

    def apply_priority(self, g: "GraphT", udf, pq: "PriorityQueue", vd: VertexData | None = None) -> None:
        if udf != UDF.SSSP_RELAX:
            raise ValueError("apply_priority takes the SSSP relax UDF (updatePriorityMin)")
        sc = self._simple(g).to_c()
        cvd = (vd or VertexData()).to_c()
        call("gg_edgeset_apply_priority", g.handle, C.byref(sc), pq.handle, C.byref(cvd))


def vertexset_apply(target, vudf, vd: VertexData) -> None:
    """vertexset_apply(set | graph, udf) (operators.cpp:10-65)."""
    cvd = vd.to_c()
    if isinstance(target, VertexSubset):
        call("gg_vertexset_apply", target.g.handle, target.handle, int(vudf), C.byref(cvd))
    else:
        call("gg_vertexset_apply", target.handle, None, int(vudf), C.byref(cvd))


class PriorityQueue:
    """graphit_runtime::GPUPriorityQueue (gpu_priority_queue.h:21-247) with
    pq.init(edges, SP, 0, delta, src) of sssp.cpp:39; `priorities` is the
    device int32 array SP."""

    def __init__(self, g: "GraphT", priorities, init_priority: int, delta: int, src: int):
        self.g = g
        self._prio = priorities
        h = C.c_void_p()
        call("gg_pq_create", g.handle, _ptr(priorities), init_priority, delta, src, C.byref(h))
        self._h = h
        g._adopt(self)

    @property
    def handle(self):
        return self._h

    def finished(self) -> bool:
        f = C.c_int32()
        call("gg_pq_finished", self._h, C.byref(f))
        return bool(f.value)

    def dequeue(self) -> "VertexSubset":
        h = C.c_void_p()
        call("gg_pq_dequeue", self._h, C.byref(h))
        return VertexSubset._view(self.g, h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().gg_pq_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class VertexFrontierList:
    """graphit_runtime::VertexFrontierList (list.h:18-116), bc.cpp's level stack."""

    def __init__(self, g: "GraphT"):
        h = C.c_void_p()
        call("gg_frontier_list_create", g.handle, C.byref(h))
        self._h = h
        g._adopt(self)

    def insert(self, f: "VertexSubset") -> None:
        call("gg_frontier_list_insert", self._h, f.handle)

    def retrieve(self, f: "VertexSubset") -> None:
        call("gg_frontier_list_retrieve", self._h, f.handle)

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().gg_frontier_list_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- the apps
def _stats(st: L.gg_stats) -> dict:
    return st.as_dict()


def _resolve(app: str, schedule, fuse):
    if schedule is None:
        schedule, dflt_fuse = default_schedule(app)
        fuse = dflt_fuse if fuse is None else fuse
    return app_schedule(schedule, bool(fuse))


def bfs(g: GraphT, src: int, schedule=None, fuse=None, with_parent: bool = False):
    """apps/bfs.cpp: returns (depth, parent|None, stats)."""
    V = g.num_vertices
    depth = np.empty(V, dtype=np.int32)
    parent = np.empty(V, dtype=np.int32) if with_parent else None
    st = L.gg_stats()
    a = _resolve("bfs", schedule, fuse)
    call("gg_bfs", g.handle, C.byref(a), src, _ptr(depth), _ptr(parent), C.byref(st))
    return depth, parent, _stats(st)


def sssp(g: GraphT, src: int, delta: int, schedule=None, fuse=None):
    """apps/sssp.cpp: returns (dist, stats); INT_MAX marks unreached."""
    dist = np.empty(g.num_vertices, dtype=np.int32)
    st = L.gg_stats()
    a = _resolve("sssp", schedule, fuse)
    call("gg_sssp", g.handle, C.byref(a), src, delta, _ptr(dist), C.byref(st))
    return dist, _stats(st)


def pagerank(g: GraphT, iters: int = 20, damping: float = 0.85, schedule=None):
    """apps/pr.cpp: returns (rank, stats)."""
    rank = np.empty(g.num_vertices, dtype=np.float32)
    st = L.gg_stats()
    a = _resolve("pr", schedule, False)
    call("gg_pagerank", g.handle, C.byref(a), iters, damping, _ptr(rank), C.byref(st))
    return rank, _stats(st)


def cc(g: GraphT, schedule=None, fuse=None):
    """apps/cc.cpp: returns (labels, stats); label = min vertex id of the component.
    fuse=True runs the whole computation as one union-find pass (same labels)."""
    labels = np.empty(g.num_vertices, dtype=np.int32)
    st = L.gg_stats()
    a = _resolve("cc", schedule, fuse)
    call("gg_cc", g.handle, C.byref(a), _ptr(labels), C.byref(st))
    return labels, _stats(st)


def bfs_batch(g: GraphT, sources, out=None):
    """Batched BFS from many sources in one persistent launch per 64 sources.
    Returns (depth [nsrc, V] int32, stats); `out` may be a preallocated
    numpy array or CUDA tensor of that shape."""
    srcs = np.ascontiguousarray(sources, dtype=np.int32)
    if out is None:
        out = np.empty((len(srcs), g.num_vertices), dtype=np.int32)
    st = L.gg_stats()
    call("gg_bfs_batch", g.handle, _np_ptr(srcs), len(srcs), _ptr(out), C.byref(st))
    return out, _stats(st)


def bc_batch(g: GraphT, sources, out=None):
    """Batched BC (apps/bc.cpp per source, 64 sources per persistent launch).
    Returns (dependencies [nsrc, V] float32, stats)."""
    srcs = np.ascontiguousarray(sources, dtype=np.int32)
    if out is None:
        out = np.empty((len(srcs), g.num_vertices), dtype=np.float32)
    st = L.gg_stats()
    call("gg_bc_batch", g.handle, _np_ptr(srcs), len(srcs), _ptr(out), C.byref(st))
    return out, _stats(st)


def sssp_batch(g: GraphT, sources, delta: int, out=None):
    """Batched delta-stepping SSSP (32 sources per pass).  Returns
    (dist [nsrc, V] int32, stats)."""
    srcs = np.ascontiguousarray(sources, dtype=np.int32)
    if out is None:
        out = np.empty((len(srcs), g.num_vertices), dtype=np.int32)
    st = L.gg_stats()
    call("gg_sssp_batch", g.handle, _np_ptr(srcs), len(srcs), delta, _ptr(out), C.byref(st))
    return out, _stats(st)


class BatchPlan:
    """A batched BFS ("bfs"), SSSP ("sssp") or BC ("bc") captured into a CUDA
    graph once and replayed by run().  `out` is a CUDA tensor of shape
    [nsrc, V]: int32 for BFS and SSSP, float32 for BC.  "bfs_multi" /
    "sssp_multi" capture one multi-source traversal into `out` of shape [V]."""

    def __init__(self, g: GraphT, app: str, sources, out, delta: int = 32):
        self.g = g
        srcs = np.ascontiguousarray(sources, dtype=np.int32)
        h = C.c_void_p()
        call("gg_batch_plan_create", g.handle, BATCH_APPS[app], _np_ptr(srcs), len(srcs),
             delta, _ptr(out), C.byref(h))
        self._h = h
        g._adopt(self)

    def run(self) -> dict:
        st = L.gg_stats()
        call("gg_batch_plan_run", self._h, C.byref(st))
        return _stats(st)

    def close(self):
        if getattr(self, "_h", None):
            lib().gg_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


BATCH_APPS = {"bfs": 0, "sssp": 1, "bc": 2, "bfs_multi": 3, "sssp_multi": 4}


def set_batch_tuning(g: GraphT, app: str, blocks_per_sm: int = 0, chunk: int = 0,
                     edge_parallel_max: int = 0, bottom_up_div: int = 0, per_source_cta: int = 0) -> None:
    """Launch shape of the graph's batched `app` kernels (0 = built-in default)."""
    t = L.gg_batch_tuning(blocks_per_sm, chunk, edge_parallel_max, bottom_up_div, per_source_cta)
    call("gg_batch_set_tuning", g.handle, BATCH_APPS[app], C.byref(t))


def set_batch_selector(g: GraphT, app: str, selector: "Selector | None") -> None:
    """Attaches a selector network to the graph's batched `app` kernels (batched
    BFS: the direction of every level, decided on the device); None detaches
    it.  The graph keeps a reference to the selector while it is attached."""
    call("gg_batch_set_selector", g.handle, BATCH_APPS[app], selector._h if selector is not None else None)
    g._batch_selector = selector


def collect_batched_directions(g: GraphT, sources, max_rows: int = 1024):
    """Per-level features [levels, 12] and times [levels, 2] (ms; top-down,
    bottom-up) of a batched BFS over the first 64 sources."""
    srcs = np.ascontiguousarray(sources, dtype=np.int32)
    feats = np.empty((max_rows, N_FEATURES), dtype=np.float32)
    times = np.empty((max_rows, 2), dtype=np.float32)
    n = C.c_int32()
    call("gg_batch_collect", g.handle, BATCH_APPS["bfs"], _np_ptr(srcs), len(srcs), max_rows,
         _np_ptr(feats), _np_ptr(times), C.byref(n))
    return feats[:n.value].copy(), times[:n.value].copy()


def collect_fused_directions(g: GraphT, src: int, max_rows: int = 8192):
    """Per-level features [levels, 12] and times [levels, 2] (ms; push, pull)
    of the fused direction-optimising BFS from src (every level forced each
    way, best of two runs)."""
    feats = np.empty((max_rows, N_FEATURES), dtype=np.float32)
    times = np.empty((max_rows, 2), dtype=np.float32)
    n = C.c_int32()
    call("gg_bfs_collect_directions", g.handle, int(src), max_rows, _np_ptr(feats), _np_ptr(times),
         C.byref(n))
    return feats[:n.value].copy(), times[:n.value].copy()


def get_batch_tuning(g: GraphT, app: str) -> dict:
    t = L.gg_batch_tuning()
    call("gg_batch_get_tuning", g.handle, BATCH_APPS[app], C.byref(t))
    return t.as_dict()


def autotune_batch(g: GraphT, app: str, sources, delta: int = 32, max_rows: int = 64):
    """Runs the autotuner of the batched `app` on this graph; the winner becomes
    the graph's tuning.  Returns (best tuning dict, [(tuning dict, ms), ...])."""
    srcs = np.ascontiguousarray(sources, dtype=np.int32)
    best = L.gg_batch_tuning()
    rows = (L.gg_tune_row * max_rows)()
    n = C.c_int32()
    call("gg_batch_autotune", g.handle, BATCH_APPS[app], _np_ptr(srcs), len(srcs), delta,
         C.byref(best), rows, max_rows, C.byref(n))
    return best.as_dict(), [(rows[i].tuning.as_dict(), rows[i].ms) for i in range(min(n.value, max_rows))]


def bfs_multi(g: GraphT, sources, schedule=None, fuse=None):
    """Multi-source BFS (distance to the nearest source): (depth, stats)."""
    srcs = np.ascontiguousarray(sources, dtype=np.int32)
    depth = np.empty(g.num_vertices, dtype=np.int32)
    st = L.gg_stats()
    a = _resolve("bfs", schedule, fuse)
    call("gg_bfs_multi", g.handle, C.byref(a), _np_ptr(srcs), len(srcs), _ptr(depth), None,
         C.byref(st))
    return depth, _stats(st)


def sssp_multi(g: GraphT, sources, delta: int, schedule=None, fuse=None):
    """Multi-source delta-stepping SSSP: (dist, stats)."""
    srcs = np.ascontiguousarray(sources, dtype=np.int32)
    dist = np.empty(g.num_vertices, dtype=np.int32)
    st = L.gg_stats()
    a = _resolve("sssp", schedule, fuse)
    call("gg_sssp_multi", g.handle, C.byref(a), _np_ptr(srcs), len(srcs), delta, _ptr(dist),
         C.byref(st))
    return dist, _stats(st)


def sssp_parts(g: GraphT, part_begin, sources, delta: int):
    """SSSP on a disjoint union, one source per part, each part's loop in a CTA
    of its own (gg_sssp_parts).  part_begin: [nparts + 1] vertex offsets;
    sources: union ids.  Returns (dist over the union, stats)."""
    pb = np.ascontiguousarray(part_begin, dtype=np.int32)
    srcs = np.ascontiguousarray(sources, dtype=np.int32)
    dist = np.empty(g.num_vertices, dtype=np.int32)
    st = L.gg_stats()
    call("gg_sssp_parts", g.handle, _np_ptr(pb), len(srcs), _np_ptr(srcs), delta, _ptr(dist), C.byref(st))
    return dist, _stats(st)


MESH_MAX_DEGREE = 32  # a part whose largest out-degree is at most this counts as a mesh


def multigraph_batch(parts, app: str, local_sources, delta: int = 32, schedule=None, fuse=True,
                     by_class: bool = True):
    """Runs BFS or SSSP on many graphs of uneven size: the graphs become a
    disjoint union, each contributes its source, and the union is traversed
    once.  For SSSP with by_class, the parts are split by class first: meshes
    (largest out-degree <= MESH_MAX_DEGREE; high diameter, thousands of small
    buckets) run one CTA per part (sssp_parts), the others as one multi-source
    traversal of their union on the whole GPU.  Returns (list of per-graph
    results, stats); stats["loop_ms"] sums the classes' loops."""
    if schedule is None:
        schedule = SimpleGPUSchedule().configLoadBalancing(SimpleGPUSchedule.load_balancing_type.TWCE)
    if app not in ("bfs", "sssp"):
        raise ValueError(app)
    classes = [(list(range(len(parts))), "multi")]
    if app == "sssp" and by_class:
        mesh = {i for i, p in enumerate(parts)
                if p.num_edges == 0 or int(np.diff(np.asarray(p.offsets)).max()) <= MESH_MAX_DEGREE}
        rest = [i for i in range(len(parts)) if i not in mesh]
        classes = [(c, m) for c, m in ((rest, "multi"), (sorted(mesh), "parts")) if c]
    out = [None] * len(parts)
    total = None
    for idx, mode in classes:
        hg, offs = HostGraph.union([parts[i] for i in idx])
        g = GraphT(hg)
        srcs = np.array([offs[k] + int(local_sources[i]) for k, i in enumerate(idx)], dtype=np.int32)
        if app == "bfs":
            r, st = bfs_multi(g, srcs, schedule, fuse)
        elif mode == "parts":
            r, st = sssp_parts(g, offs, srcs, delta)
        else:
            r, st = sssp_multi(g, srcs, delta, schedule, fuse)
        g.close()
        for k, i in enumerate(idx):
            out[i] = r[offs[k]:offs[k + 1]]
        if total is None:
            total = dict(st)
            total["classes"] = []
        else:
            for key in ("loop_ms", "device_ms", "vertices_reached", "edges_traversed", "launches"):
                total[key] += st[key]
            total["iterations"] = max(total["iterations"], st["iterations"])
        total["classes"].append({"graphs": len(idx), "loop_ms": st["loop_ms"],
                                 "mode": "one CTA per part" if mode == "parts" else "one multi-source traversal"})
    return out, total


def bc(g: GraphT, src: int, schedule=None, fuse=None):
    """apps/bc.cpp: returns (dependences fp32, stats)."""
    dep = np.empty(g.num_vertices, dtype=np.float32)
    st = L.gg_stats()
    a = _resolve("bc", schedule, fuse)
    call("gg_bc", g.handle, C.byref(a), src, _ptr(dep), C.byref(st))
    return dep, _stats(st)


# --------------------------------------------------------- learned selector
N_FEATURES, N_OUTPUTS, N_CANDIDATES = 12, 11, 36
LB_HEAD = [SimpleGPUSchedule.load_balancing_type.TWCE, SimpleGPUSchedule.load_balancing_type.ETWC,
           SimpleGPUSchedule.load_balancing_type.CM, SimpleGPUSchedule.load_balancing_type.WM,
           SimpleGPUSchedule.load_balancing_type.VERTEX_BASED, SimpleGPUSchedule.load_balancing_type.EDGE_ONLY]
SEL_APPS = {"bfs": 0, "sssp": 1, "cc": 2}


def candidate_labels(c: int) -> tuple[int, int, int]:
    """Candidate index -> (direction, load-balancing head index, frontier type)."""
    return c // 18, (c // 3) % 6, c % 3


class Selector:
    """The bf16 MLP schedule selector (libgg.so kernels)."""

    def __init__(self, seed: int = 1, _handle=None):
        if _handle is None:
            _handle = C.c_void_p()
            call("gg_selector_create", seed, C.byref(_handle))
        self._h = _handle

    @classmethod
    def load(cls, path: str) -> "Selector":
        h = C.c_void_p()
        call("gg_selector_load", str(path).encode(), C.byref(h))
        return cls(_handle=h)

    @classmethod
    def pretrained(cls) -> "Selector":
        """The model shipped with the package (selector_model.bin, trained by
        easy_graphit_gb300.selector_train; its manifest is selector_model.json)."""
        return cls.load(str(Path(__file__).resolve().parent / "selector_model.bin"))

    @classmethod
    def pretrained_batched_bfs(cls) -> "Selector":
        """The per-level direction model of batched BFS shipped with the package
        (selector_batched_bfs.bin, trained by `easy_graphit_gb300.selector_train
        --batched-bfs`; manifest selector_batched_bfs.json)."""
        return cls.load(str(Path(__file__).resolve().parent / "selector_batched_bfs.bin"))

    @classmethod
    def pretrained_fused_bfs(cls) -> "Selector":
        """The per-level direction model of the fused single-source BFS loop
        shipped with the package (selector_fused_bfs.bin, trained by
        `easy_graphit_gb300.selector_train --fused-bfs`; manifest
        selector_fused_bfs.json)."""
        return cls.load(str(Path(__file__).resolve().parent / "selector_fused_bfs.bin"))

    def save(self, path: str) -> None:
        call("gg_selector_save", self._h, str(path).encode())

    @property
    def params(self) -> np.ndarray:
        n = lib().gg_selector_num_params()
        out = np.empty(n, dtype=np.float32)
        call("gg_selector_get_params", self._h, _np_ptr(out), n)
        return out

    @params.setter
    def params(self, p) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        call("gg_selector_set_params", self._h, _np_ptr(p), len(p))

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        out = np.empty((len(x), N_OUTPUTS), dtype=np.float32)
        call("gg_selector_forward", self._h, _np_ptr(x), len(x), _np_ptr(out))
        return out

    def grad(self, x, labels) -> tuple[np.ndarray, float]:
        x = np.ascontiguousarray(x, dtype=np.float32)
        labels = np.ascontiguousarray(labels, dtype=np.int32)
        g = np.empty(lib().gg_selector_num_params(), dtype=np.float32)
        loss = C.c_float()
        call("gg_selector_grad", self._h, _np_ptr(x), _np_ptr(labels), len(x), _np_ptr(g), C.byref(loss))
        return g, loss.value

    def train(self, x, labels, epochs: int = 500, lr: float = 3e-3) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        labels = np.ascontiguousarray(labels, dtype=np.int32)
        loss = C.c_float()
        call("gg_selector_train", self._h, _np_ptr(x), _np_ptr(labels), len(x), epochs, lr, C.byref(loss))
        return loss.value

    def predict(self, x) -> np.ndarray:
        z = self.forward(x)
        return np.stack([z[:, 0:2].argmax(1), z[:, 2:8].argmax(1), z[:, 8:11].argmax(1)], axis=1)

    def close(self):
        if getattr(self, "_h", None):
            lib().gg_selector_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def collect_timings(g: GraphT, app: str, src: int = 0, delta: int = 32, max_rows: int = 4096):
    """Per-iteration features [rows, 12] and candidate times [rows, 36] (ms)."""
    feats = np.empty((max_rows, N_FEATURES), dtype=np.float32)
    times = np.empty((max_rows, N_CANDIDATES), dtype=np.float32)
    n = C.c_int32()
    call("gg_selector_collect", g.handle, SEL_APPS[app], src, delta, max_rows, _np_ptr(feats),
         _np_ptr(times), C.byref(n))
    return feats[:n.value].copy(), times[:n.value].copy()


def labels_from_times(times: np.ndarray) -> np.ndarray:
    best = np.argmin(times, axis=1)
    return np.array([candidate_labels(int(c)) for c in best], dtype=np.int32).reshape(-1, 3)
