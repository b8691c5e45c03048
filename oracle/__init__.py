"""ORACLE -- test infrastructure only.

ctypes wrapper of oracle/liboracle.so (the CPU restatement in oracle.cpp) and
of the reference-built checker oracle/_ref/ref_gapbs (ref_gapbs.cpp compiled
against the reference's GAPBS headers).  The reference's own apps, compiled
against oracle/app_shim into oracle/_ref/app_*, are run by
tests/golden/make_app_golden.py.  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline legs use this package; the engine never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_BIN = HERE / "_ref" / "ref_gapbs"

_lib = None
_P = C.c_void_p


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    return LIB


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        i32, i64, f64, f32 = C.c_int32, C.c_int64, C.c_double, C.c_float
        sig = {
            "orc_bfs": (None, [i32, _P, _P, i32, _P]),
            "orc_bfs_check_parent": (i64, [i32, _P, _P, i32, _P, _P]),
            "orc_bfs_omp": (None, [i32, _P, _P, i32, _P, i32]),
            "orc_sssp_dijkstra": (None, [i32, _P, _P, _P, i32, _P]),
            "orc_sssp_delta_gpu": (i64, [i32, _P, _P, _P, i32, i32, _P]),
            "orc_sssp_ordered": (None, [i32, _P, _P, _P, i32, i32, _P, i32]),
            "orc_pagerank": (None, [i32, _P, _P, i32, f64, _P]),
            "orc_pagerank_omp": (None, [i32, _P, _P, _P, i32, f32, _P, i32]),
            "orc_cc": (None, [i32, _P, _P, _P]),
            "orc_cc_labelprop": (i32, [i32, _P, _P, _P]),
            "orc_cc_omp": (None, [i32, _P, _P, _P, i32]),
            "orc_bc": (None, [i32, _P, _P, i32, _P]),
            "orc_reached_edges": (i64, [i32, _P, _P]),
            "orc_rmat": (_P, [i32, i32, f32, f32, f32, i64, i32, i32, i32]),
            "orc_graph_vertices": (i32, [_P]),
            "orc_graph_edges": (i64, [_P]),
            "orc_graph_copy": (None, [_P, _P, _P, _P]),
            "orc_graph_free": (None, [_P]),
            "orc_pick_sources": (None, [i32, _P, i32, i64, _P]),
        }
        for k, (r, a) in sig.items():
            fn = getattr(L, k)
            fn.restype = r
            fn.argtypes = a
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def _csr(off, dst, w=None):
    off = np.ascontiguousarray(off, dtype=np.int32)
    dst = np.ascontiguousarray(dst, dtype=np.int32)
    w = None if w is None else np.ascontiguousarray(w, dtype=np.int32)
    return off, dst, w


def bfs(off, dst, src):
    off, dst, _ = _csr(off, dst)
    out = np.empty(len(off) - 1, dtype=np.int32)
    lib().orc_bfs(len(off) - 1, _p(off), _p(dst), src, _p(out))
    return out


def bfs_check_parent(off, dst, src, depth, parent) -> int:
    off, dst, _ = _csr(off, dst)
    depth = np.ascontiguousarray(depth, dtype=np.int32)
    parent = np.ascontiguousarray(parent, dtype=np.int32)
    return lib().orc_bfs_check_parent(len(off) - 1, _p(off), _p(dst), src, _p(depth), _p(parent))


def bfs_omp(off, dst, src, threads=0):
    off, dst, _ = _csr(off, dst)
    out = np.empty(len(off) - 1, dtype=np.int32)
    lib().orc_bfs_omp(len(off) - 1, _p(off), _p(dst), src, _p(out), threads)
    return out


def sssp_dijkstra(off, dst, w, src):
    off, dst, w = _csr(off, dst, w)
    out = np.empty(len(off) - 1, dtype=np.int32)
    lib().orc_sssp_dijkstra(len(off) - 1, _p(off), _p(dst), _p(w), src, _p(out))
    return out


def sssp_delta_gpu(off, dst, w, src, delta):
    """Sequential restatement of the GPU delta-stepping loop; (dist, advances)."""
    off, dst, w = _csr(off, dst, w)
    out = np.empty(len(off) - 1, dtype=np.int32)
    adv = lib().orc_sssp_delta_gpu(len(off) - 1, _p(off), _p(dst), _p(w), src, delta, _p(out))
    return out, adv


def sssp_ordered(off, dst, w, src, delta, threads=0):
    """OpenMP port of GAPBS OrderedProcessingOperatorNoMerge."""
    off, dst, w = _csr(off, dst, w)
    out = np.empty(len(off) - 1, dtype=np.int32)
    lib().orc_sssp_ordered(len(off) - 1, _p(off), _p(dst), _p(w), src, delta, _p(out), threads)
    return out


def pagerank(off, dst, iters=20, damp=0.85):
    off, dst, _ = _csr(off, dst)
    out = np.empty(len(off) - 1, dtype=np.float64)
    lib().orc_pagerank(len(off) - 1, _p(off), _p(dst), iters, damp, _p(out))
    return out


def pagerank_omp(toff, tsrc, outdeg, iters=20, damp=0.85, threads=0):
    toff, tsrc, _ = _csr(toff, tsrc)
    outdeg = np.ascontiguousarray(outdeg, dtype=np.int32)
    out = np.empty(len(toff) - 1, dtype=np.float32)
    lib().orc_pagerank_omp(len(toff) - 1, _p(toff), _p(tsrc), _p(outdeg), iters, damp, _p(out), threads)
    return out


def cc(off, dst):
    off, dst, _ = _csr(off, dst)
    out = np.empty(len(off) - 1, dtype=np.int32)
    lib().orc_cc(len(off) - 1, _p(off), _p(dst), _p(out))
    return out


def cc_labelprop(off, dst):
    off, dst, _ = _csr(off, dst)
    out = np.empty(len(off) - 1, dtype=np.int32)
    rounds = lib().orc_cc_labelprop(len(off) - 1, _p(off), _p(dst), _p(out))
    return out, rounds


def cc_omp(off, dst, threads=0):
    off, dst, _ = _csr(off, dst)
    out = np.empty(len(off) - 1, dtype=np.int32)
    lib().orc_cc_omp(len(off) - 1, _p(off), _p(dst), _p(out), threads)
    return out


def bc(off, dst, src):
    off, dst, _ = _csr(off, dst)
    out = np.empty(len(off) - 1, dtype=np.float64)
    lib().orc_bc(len(off) - 1, _p(off), _p(dst), src, _p(out))
    return out


def reached_edges(off, val) -> int:
    off = np.ascontiguousarray(off, dtype=np.int32)
    val = np.ascontiguousarray(val, dtype=np.int32)
    return lib().orc_reached_edges(len(off) - 1, _p(off), _p(val))


def transpose(off, dst):
    """In-neighbour CSR (numpy), for the pull-direction CPU baselines."""
    off = np.asarray(off, dtype=np.int64)
    dst = np.asarray(dst, dtype=np.int64)
    V = len(off) - 1
    src = np.repeat(np.arange(V, dtype=np.int64), np.diff(off))
    order = np.lexsort((src, dst))
    toff = np.zeros(V + 1, dtype=np.int64)
    np.add.at(toff, dst + 1, 1)
    return np.cumsum(toff).astype(np.int32), src[order].astype(np.int32)


# ------------------------------------------------------------ input graphs
K_RAND_SEED = 27491095  # GAPBS kRandSeed (runtime/infra_gapbs/util.h)


def rmat(scale: int, degree: int = 16, symmetrize: bool = False, a: float = 0.57, b: float = 0.19,
         c: float = 0.19, seed: int = K_RAND_SEED, wmin: int = 1, wmax: int = 255):
    """(offsets, dst, weights) of the R-MAT CSR, built on the host cores by the
    oracle's own restatement of GAPBS's generator and builder."""
    L = lib()
    h = L.orc_rmat(scale, degree, a, b, c, seed, int(symmetrize), wmin, wmax)
    try:
        V, E = L.orc_graph_vertices(h), L.orc_graph_edges(h)
        off = np.empty(V + 1, dtype=np.int32)
        dst = np.empty(E, dtype=np.int32)
        w = np.empty(E, dtype=np.int32)
        L.orc_graph_copy(h, _p(off), _p(dst), _p(w))
    finally:
        L.orc_graph_free(h)
    return off, dst, w


def pick_sources(off, n: int, seed: int = K_RAND_SEED):
    """n sources as GAPBS's SourcePicker draws them."""
    off = np.ascontiguousarray(off, dtype=np.int32)
    out = np.empty(n, dtype=np.int32)
    lib().orc_pick_sources(len(off) - 1, _p(off), n, seed, _p(out))
    return out


# ------------------------------------------------------ reference-built data
def ref_available() -> bool:
    return REF_BIN.exists()


def ref_graph(scale: int, degree: int, symmetrize: bool):
    """CSR built by the reference's GAPBS generator + builder."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "g.bin")
        subprocess.run([str(REF_BIN), "graph", str(scale), str(degree), str(int(symmetrize)), out],
                       check=True, capture_output=True)
        raw = open(out, "rb").read()
    V = np.frombuffer(raw, dtype=np.int32, count=1)[0]
    E = np.frombuffer(raw, dtype=np.int64, count=1, offset=4)[0]
    o = 12
    off = np.frombuffer(raw, dtype=np.int32, count=V + 1, offset=o).copy()
    o += 4 * (V + 1)
    dst = np.frombuffer(raw, dtype=np.int32, count=E, offset=o).copy()
    o += 4 * E
    w = np.frombuffer(raw, dtype=np.int32, count=E, offset=o).copy()
    return off, dst, w


def ref_sssp(scale: int, degree: int, symmetrize: bool, unit: bool, delta: int, sources):
    """Distances from the reference's OrderedProcessingOperatorNoMerge."""
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "d.bin")
        subprocess.run([str(REF_BIN), "sssp", str(scale), str(degree), str(int(symmetrize)),
                        str(int(unit)), str(delta), out, *map(str, sources)],
                       check=True, capture_output=True)
        raw = open(out, "rb").read()
    n, V = np.frombuffer(raw, dtype=np.int32, count=2)
    return np.frombuffer(raw, dtype=np.int32, offset=8).reshape(n, V).copy()
