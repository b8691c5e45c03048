"""Autotuned launch shapes of the batched kernels, per graph size.

    python -m easy_graphit_gb300.tune_report [--out report.md]

For R-MAT graphs of scale 12 to 22 (edge factor 16; BC on the symmetrized
graph) and 2-D grids of side 256 to 2048, runs gg_batch_autotune for batched
BFS (64 sources), SSSP (32 sources, delta 32) and BC (64 sources) and tabulates
the chosen CTAs per SM, work-item chunk and SSSP edge-parallel threshold with
the persistent kernel's time next to the built-in launch shape's.
"""
from __future__ import annotations

import argparse
import time

from .graphit import GraphT, HostGraph, autotune_batch, set_batch_tuning

SIZES = [("rmat", 12), ("rmat", 14), ("rmat", 16), ("rmat", 18), ("rmat", 20), ("rmat", 22),
         ("grid", 256), ("grid", 1024), ("grid", 2048)]
APPS = [("bfs", 64), ("sssp", 32), ("bc", 64)]


def builtin_row(rows, fit):
    """The trial that ran the built-in shape (all CTAs that fit, chunk 256, threshold 6)."""
    for t, ms in rows:
        if (t["blocks_per_sm"] == fit and t["chunk"] in (0, 256) and t["edge_parallel_max"] in (0, 6)
                and t["bottom_up_div"] in (0, 16)):
            return ms
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None)
    ap.add_argument("--delta", type=int, default=32)
    a = ap.parse_args()
    lines = ["| graph | V | E | app | sources | CTAs/SM | chunk | edge-parallel max | bottom-up div | tuned ms | built-in ms | trials |",
             "|---|---|---|---|---|---|---|---|---|---|---|---|"]
    t0 = time.time()
    for kind, size in SIZES:
        for app, nsrc in APPS:
            sym = app == "bc" or kind == "grid"
            hg = HostGraph.rmat(size, 16, symmetrize=sym) if kind == "rmat" else HostGraph.grid(size, size)
            g = GraphT(hg, symmetric=sym)
            srcs = hg.pick_sources(nsrc)
            best, rows = autotune_batch(g, app, srcs, a.delta)
            fit = max(t["blocks_per_sm"] for t, _ in rows)
            ms = min(m for t, m in rows if t == best)
            base = builtin_row(rows, fit)
            name = f"R-MAT {size}{' sym' if sym and kind == 'rmat' else ''}" if kind == "rmat" else f"grid {size}x{size}"
            base_s = f"{base:.3f}" if base is not None else "-"
            lines.append(f"| {name} | {hg.num_vertices} | {hg.num_edges} | {app} | {nsrc} | {best['blocks_per_sm']} | "
                         f"{best['chunk'] if app != 'bfs' else '-'} | "
                         f"{best['edge_parallel_max'] if app == 'sssp' else '-'} | "
                         f"{best['bottom_up_div'] if app == 'bfs' else '-'} | {ms:.3f} | {base_s} | {len(rows)} |")
            print(lines[-1], flush=True)
            set_batch_tuning(g, app)
            g.close()
    text = "\n".join(lines) + f"\n\n({time.time() - t0:.0f} s; delta {a.delta} for SSSP)\n"
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(text)


if __name__ == "__main__":
    main()
