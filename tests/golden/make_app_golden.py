"""Regenerates tests/golden/ref_apps.npz by running the reference's own apps.

easy_graphit's apps/{bfs,sssp,pr,cc,bc}.cpp are compiled with g++, where they
lie in the reference tree, against oracle/app_shim/ -- a host-execution
stand-in for the BuildIt staging library, which is an empty submodule in the
reference tree -- by `make -C oracle apps REF_DIR=<reference tree>`.  Each
binary runs the app's own testcase() (its UDFs, loops and constants) on a
.graphit_bin file and writes its VertexData arrays; float vertex data is held
in double there, so PageRank and BC come out in FP64.  Stored per graph g:
  * pr/<g>: old_rank after the app's 20 iterations;
  * cc/<g>: ID;
  * bc/<g>/s<k>: dependences from sources/<g>[k];
  * bfs/<g>: hop depths along the app's parent tree from sources/<g>[0] (-1 unreached);
  * sssp/<g>/d<delta>: SP from sources/<g>[0] (INT_MAX unreached), and
    sssp/<g>/adv<delta>: how many times the app's priority queue moved its
    window (the count the engine's single-source queues are held to);
  * config1/depth: bfs.cpp's hop depths on the symmetrized R-MAT 16 (edge
    factor 16) from its highest-degree vertex (config1/source, config1/sha256);
  * config2/...: sssp.cpp on the directed R-MAT 22 (edge factor 16, weights
    U[1,255]) from the first two SourcePicker sources at delta 8, 32 and 128
    -- distances too large to store, so their SHA-256 (config2/s<k>_sha256,
    equal at every delta) and the window moves (config2/s<k>_adv<delta>);
  * how to rebuild g: graph/<g>/{scale,degree,symmetrize,sha256} for the R-MAT
    graphs (oracle.rmat, itself pinned to the reference's builder), the full
    CSR graph/<g>/{offsets,dst,w} for the grid.

Usage: GG_REF_DIR=<reference tree> python tests/golden/make_app_golden.py
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

RMAT = {"rmat10_k16_sym": (10, 16, True), "rmat11_k8_dir": (11, 8, False)}
GRID = "grid32"
DELTAS = [1, 8, 32]
INT_MAX = 2**31 - 1


def digest(off, dst, w) -> str:
    h = hashlib.sha256()
    for a in (off, dst, w):
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()


def grid(n: int = 32, seed: int = 20261204):
    """n x n 4-neighbour grid, both directions, weights U[1, 1000] (CSR, targets ascending)."""
    rows = [[] for _ in range(n * n)]
    for r in range(n):
        for c in range(n):
            v = r * n + c
            for rr, cc in ((r - 1, c), (r, c - 1), (r, c + 1), (r + 1, c)):
                if 0 <= rr < n and 0 <= cc < n:
                    rows[v].append(rr * n + cc)
    off = np.zeros(n * n + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(x) for x in rows])
    dst = np.array([u for x in rows for u in x], dtype=np.int32)
    w = np.random.default_rng(seed).integers(1, 1001, len(dst)).astype(np.int32)
    return off, dst, w


def sources_for(off, k=2, seed=27491095):
    """Highest-degree vertex plus k-1 seeded non-zero-degree vertices."""
    deg = np.diff(off)
    rng = np.random.default_rng(seed)
    srcs = [int(np.argmax(deg))]
    while len(srcs) < k:
        s = int(rng.integers(0, len(deg)))
        if deg[s] > 0 and s not in srcs:
            srcs.append(s)
    return srcs


def write_graphit_bin(path, off, dst, w) -> None:
    """runtime/infra_gpu/graph.h:255-270: V, E, src[E], dst[E], weight[E], offsets[V+1] (int32)."""
    V, E = len(off) - 1, len(dst)
    src = np.repeat(np.arange(V, dtype=np.int32), np.diff(off))
    with open(path, "wb") as f:
        for a in (np.array([V, E]), src, dst, w, off):
            np.ascontiguousarray(a, dtype=np.int32).tofile(f)


def run_app(app: str, graph_file: str, *args) -> dict[str, np.ndarray]:
    """Runs oracle/_ref/app_<app> (max_cta, cta_size as its main() reads them)
    and returns the VertexData arrays it wrote."""
    exe = ROOT / "oracle" / "_ref" / f"app_{app}"
    with tempfile.TemporaryDirectory() as out:
        env = dict(os.environ, GG_SHIM_OUT=out, GG_SHIM_ARG0=graph_file)
        for i, a in enumerate(args):
            env[f"GG_SHIM_ARG{i + 1}"] = str(a)
        subprocess.run([str(exe), "60", "512"], env=env, check=True, capture_output=True)
        kinds = {"i32": np.int32, "u8": np.uint8, "f64": np.float64}
        res = {}
        for fn in os.listdir(out):
            name, ext = fn.rsplit(".", 1)
            res[name] = np.fromfile(os.path.join(out, fn), dtype=kinds[ext])
        return res


def depths_from_parents(parent: np.ndarray, src: int) -> np.ndarray:
    """Hop depth of every vertex along a BFS parent tree (parent[src] = src, -1 unreached)."""
    depth = np.full(len(parent), -1, dtype=np.int32)
    depth[src] = 0
    for v in range(len(parent)):
        if parent[v] < 0 or depth[v] >= 0:
            continue
        chain = []
        u = v
        while depth[u] < 0:
            chain.append(u)
            u = int(parent[u])
        for x in reversed(chain):
            depth[x] = depth[int(parent[x])] + 1
    return depth


def main() -> None:
    ref_dir = os.environ.get("GG_REF_DIR")
    if not ref_dir:
        sys.exit("set GG_REF_DIR to the reference tree")
    oracle.build()
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "apps", f"REF_DIR={ref_dir}"], check=True)
    graphs = {}
    out: dict[str, np.ndarray] = {}
    for name, (scale, deg, sym) in RMAT.items():
        off, dst, w = (np.asarray(a) for a in oracle.rmat(scale, deg, symmetrize=sym))
        graphs[name] = (off, dst, w)
        out[f"graph/{name}/scale"], out[f"graph/{name}/degree"] = np.array(scale), np.array(deg)
        out[f"graph/{name}/symmetrize"] = np.array(sym)
        out[f"graph/{name}/sha256"] = np.array(digest(off, dst, w))
    off, dst, w = grid()
    graphs[GRID] = (off, dst, w)
    out[f"graph/{GRID}/offsets"], out[f"graph/{GRID}/dst"], out[f"graph/{GRID}/w"] = off, dst, w
    with tempfile.TemporaryDirectory() as tmp:
        for name, (off, dst, w) in graphs.items():
            gf = os.path.join(tmp, f"{name}.graphit_bin")
            write_graphit_bin(gf, off, dst, w)
            srcs = sources_for(off)
            out[f"sources/{name}"] = np.array(srcs, dtype=np.int32)
            out[f"pr/{name}"] = run_app("pr", gf)["old_rank"]
            out[f"cc/{name}"] = run_app("cc", gf)["ID"]
            for k, s in enumerate(srcs):
                out[f"bc/{name}/s{k}"] = run_app("bc", gf, s, 0.0)["dependences"]
            out[f"bfs/{name}"] = depths_from_parents(run_app("bfs", gf, srcs[0], 0.0)["parent"], srcs[0])
            for d in DELTAS:
                r = run_app("sssp", gf, srcs[0], d)
                out[f"sssp/{name}/d{d}"] = r["SP"]
                out[f"sssp/{name}/adv{d}"] = r["pq_advances"]
        # the BFS workload as stated: symmetrized R-MAT 16, highest-degree source
        off, dst, w = (np.asarray(a) for a in oracle.rmat(16, 16, symmetrize=True))
        gf = os.path.join(tmp, "config1.graphit_bin")
        write_graphit_bin(gf, off, dst, w)
        src = int(np.argmax(np.diff(off)))
        out["config1/source"] = np.array(src, dtype=np.int32)
        out["config1/sha256"] = np.array(digest(off, dst, w))
        out["config1/depth"] = depths_from_parents(run_app("bfs", gf, src, 0.0)["parent"], src)
        # the SSSP workload's R-MAT 22 (a few minutes: the app runs five trials
        # and its queue scans every vertex per window move)
        off, dst, w = (np.asarray(a) for a in oracle.rmat(22, 16))
        gf = os.path.join(tmp, "config2.graphit_bin")
        write_graphit_bin(gf, off, dst, w)
        srcs = [int(x) for x in oracle.pick_sources(off, 2)]
        out["config2/sha256"] = np.array(digest(off, dst, w))
        out["config2/sources"] = np.array(srcs, dtype=np.int32)
        for k, src in enumerate(srcs):
            digests = set()
            for d in (8, 32, 128):
                r = run_app("sssp", gf, src, d)
                digests.add(hashlib.sha256(np.ascontiguousarray(r["SP"], dtype=np.int32).tobytes()).hexdigest())
                out[f"config2/s{k}_adv{d}"] = r["pq_advances"]
            assert len(digests) == 1, "distances depend on delta"
            out[f"config2/s{k}_sha256"] = np.array(digests.pop())
    path = Path(__file__).with_name("ref_apps.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({path.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
