"""Regenerates tests/golden/gapbs_ref.npz from the reference's own code.

Runs oracle/_ref/ref_gapbs -- easy_graphit's vendored GAPBS generator, builder
and OrderedProcessingOperatorNoMerge SSSP (runtime/infra_gapbs/), compiled by
`make -C oracle ref REF_DIR=<reference tree>` -- and stores:
  * graph/<name>/{sha256, V, E}: digests of the CSR the reference builds;
  * graph_small/{offsets,dst,w}: one full small CSR;
  * sssp/<name>/d<delta>: reference distances for a few sources;
  * bfs/<name>: reference delta-stepping with unit weights (= hop depths, -1 unreached).

Usage: python tests/golden/make_golden.py   (needs the reference tree)
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

GRAPHS = {  # name: (scale, degree, symmetrize)
    "rmat10_k16_sym": (10, 16, True),
    "rmat11_k8_dir": (11, 8, False),
    "rmat12_k16_dir": (12, 16, False),
    "rmat12_k16_sym": (12, 16, True),
    "rmat14_k16_dir": (14, 16, False),
}
SSSP_GRAPHS = ["rmat10_k16_sym", "rmat12_k16_dir"]
DELTAS = [1, 8, 32, 128]
INT_MAX = 2**31 - 1


def digest(off, dst, w) -> str:
    h = hashlib.sha256()
    for a in (off, dst, w):
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    return h.hexdigest()


def sources_for(off, k=4, seed=27491095):
    """Highest-degree vertex plus k-1 seeded non-zero-degree vertices."""
    deg = np.diff(off)
    rng = np.random.default_rng(seed)
    srcs = [int(np.argmax(deg))]
    while len(srcs) < k:
        s = int(rng.integers(0, len(deg)))
        if deg[s] > 0 and s not in srcs:
            srcs.append(s)
    return srcs


def main() -> None:
    oracle.build()
    subprocess_ref = ROOT / "oracle" / "_ref" / "ref_gapbs"
    if not subprocess_ref.exists():
        import subprocess
        subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    out: dict[str, np.ndarray] = {}
    csr = {}
    for name, (scale, deg, sym) in GRAPHS.items():
        off, dst, w = oracle.ref_graph(scale, deg, sym)
        csr[name] = (off, dst, w)
        out[f"graph/{name}/sha256"] = np.array(digest(off, dst, w))
        out[f"graph/{name}/V"] = np.array(len(off) - 1)
        out[f"graph/{name}/E"] = np.array(len(dst))
    off, dst, w = csr["rmat10_k16_sym"]
    out["graph_small/offsets"], out["graph_small/dst"], out["graph_small/w"] = off, dst, w
    for name in SSSP_GRAPHS:
        scale, deg, sym = GRAPHS[name]
        off = csr[name][0]
        srcs = sources_for(off)
        out[f"sources/{name}"] = np.array(srcs, dtype=np.int32)
        for d in DELTAS:
            out[f"sssp/{name}/d{d}"] = oracle.ref_sssp(scale, deg, sym, False, d, srcs)
        unit = oracle.ref_sssp(scale, deg, sym, True, 1, srcs)
        unit[unit == INT_MAX] = -1
        out[f"bfs/{name}"] = unit
    path = Path(__file__).with_name("gapbs_ref.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({path.stat().st_size} bytes, {len(out)} arrays)")


if __name__ == "__main__":
    main()
