"""Trains the learned schedule selector on timings generated by the engine.

    python -m easy_graphit_gb300.selector_train [--out easy_graphit_gb300/selector_model.bin]
    python -m easy_graphit_gb300.selector_train --batched-bfs [--out .../selector_batched_bfs.bin]
    python -m easy_graphit_gb300.selector_train --fused-bfs [--out .../selector_fused_bfs.bin]

--batched-bfs trains the per-level direction of the batched BFS instead: on
each training graph, 64 sources are traversed with every level top-down and
then bottom-up (gg_batch_collect); a level's label is its faster direction, and
levels where the two differ more weigh more (the row is repeated).  The model
runs on the device inside the batched kernel (gg_batch_set_selector); held-out
seeds compare it with both fixed directions, the built-in rule and the
per-level optimum.

--fused-bfs does the same for the fused single-source BFS loop (gg_bfs with
fuse = 1 and a learned schedule): every training source is traversed with every
level pushed and then pulled (gg_bfs_collect_directions); held-out graphs
compare the network with bfs.cpp's two schedules and with its hybrid rule fused.

Training graphs: R-MAT at scales 18 to 24 with skew a in [0.45, 0.75] (b = c =
(0.95 - a) / 2) and 2-D grids, GAPBS-seeded; for each, BFS and SSSP runs
(delta 32) and CC.  At every iteration the engine times all 36 candidate
schedules on the same state (gg_selector_collect); the fastest candidate's
(direction, load balancing, frontier type) is the label.  Training is
full-batch Adam on the GPU kernels.  Evaluation uses held-out seeds: the
learned schedule against the apps' hand-written GraphIt schedules, results
checked bit-exact against the oracle.  Writes the parameter file and a JSON
manifest beside it.
"""
from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np

from .graphit import (GraphT, HostGraph, LearnedGPUSchedule, Selector, bfs, bfs_batch, cc,
                      collect_batched_directions, collect_fused_directions, collect_timings, default_schedule,
                      labels_from_times,
                      set_batch_selector, set_batch_tuning, sssp)

PKG = Path(__file__).resolve().parent
DEFAULT_OUT = PKG / "selector_model.bin"
BATCHED_BFS_OUT = PKG / "selector_batched_bfs.bin"
FUSED_BFS_OUT = PKG / "selector_fused_bfs.bin"

TRAIN_SEEDS = [101, 102, 103]
HELDOUT_SEEDS = [901, 902]


def rmat(scale, a, seed, sym):
    b = (0.95 - a) / 2
    return HostGraph.rmat(scale, 16, a=a, b=b, c=b, seed=seed, symmetrize=sym)


def training_graphs(scales, skews):
    out = []
    for i, scale in enumerate(scales):
        for j, a in enumerate(skews):
            out.append((f"rmat{scale}_a{a:.2f}", scale, a, TRAIN_SEEDS[(i + j) % len(TRAIN_SEEDS)]))
    return out


def collect(scales, skews, grids, max_rows, log):
    X, T = [], []
    for name, scale, a, seed in training_graphs(scales, skews):
        for app in ("bfs", "cc", "sssp"):
            sym = app != "sssp"
            hg = rmat(scale, a, seed, sym)
            g = GraphT(hg, symmetric=sym)
            srcs = hg.pick_sources(2 if app == "bfs" else 1, seed=seed)
            for s in srcs:
                t0 = time.time()
                f, t = collect_timings(g, app, int(s), 32, max_rows)
                X.append(f)
                T.append(t)
                log(f"{name} {app} src={int(s)} rows={len(f)} ({time.time() - t0:.1f}s)")
                if app == "cc":
                    break
            g.close()
    for n in grids:
        hg = HostGraph.grid(n, n, seed=TRAIN_SEEDS[0])
        g = GraphT(hg, symmetric=True)
        for app in ("bfs", "sssp"):
            s = int(hg.pick_sources(1, seed=7)[0])
            f, t = collect_timings(g, app, s, 32, max_rows)
            X.append(f)
            T.append(t)
            log(f"grid{n} {app} rows={len(f)}")
        g.close()
    return np.concatenate(X), np.concatenate(T)


def evaluate(model, scale, log):
    """Held-out graphs: learned schedule vs the apps' hand-written schedules;
    both must produce identical results."""
    rows = []
    for seed in HELDOUT_SEEDS:
        for app in ("bfs", "sssp", "cc"):
            sym = app != "sssp"
            hg = rmat(scale, 0.57, seed, sym)
            g = GraphT(hg, symmetric=sym)
            src = int(hg.pick_sources(1, seed=seed)[0])
            plain, fuse = default_schedule(app)
            learned = LearnedGPUSchedule(model)
            times, outs = {}, {}
            for label, sch, fz in (("plain", plain, fuse), ("learned", learned, False)):
                best = None
                for _ in range(3):
                    if app == "bfs":
                        out, _, st = bfs(g, src, sch, fz)
                    elif app == "sssp":
                        out, st = sssp(g, src, 32, sch, fz)
                    else:
                        out, st = cc(g, sch)
                    outs[label] = out
                    best = st["device_ms"] if best is None else min(best, st["device_ms"])
                times[label] = best
            if not np.array_equal(outs["plain"], outs["learned"]):
                raise AssertionError(f"{app}: learned and plain schedules disagree")
            rows.append({"app": app, "seed": seed, "scale": scale, "plain_ms": times["plain"],
                         "learned_ms": times["learned"], "speedup": times["plain"] / times["learned"]})
            log(f"heldout {app} seed={seed}: plain {times['plain']:.2f} ms, learned {times['learned']:.2f} ms")
            g.close()
    return rows


# ------------------------------------------------------------ batched BFS
def collect_batched_bfs(scales, skews, grids, log):
    X, T = [], []
    for name, scale, a, seed in training_graphs(scales, skews):
        for sym in (True, False):
            hg = rmat(scale, a, seed, sym)
            g = GraphT(hg, symmetric=sym)
            for grp in range(2):
                f, t = collect_batched_directions(g, hg.pick_sources(64, seed=seed + 17 * grp))
                X.append(f)
                T.append(t)
                log(f"{name}{' sym' if sym else ''} group {grp}: {len(f)} levels, "
                    f"top-down {t[:, 0].sum():.2f} ms, bottom-up {t[:, 1].sum():.2f} ms, best {t.min(1).sum():.2f} ms")
            g.close()
    for n in grids:
        hg = HostGraph.grid(n, n, seed=TRAIN_SEEDS[0])
        g = GraphT(hg, symmetric=True)
        f, t = collect_batched_directions(g, hg.pick_sources(64, seed=7))
        X.append(f)
        T.append(t)
        log(f"grid{n}: {len(f)} levels")
        g.close()
    return np.concatenate(X), np.concatenate(T)


def batched_rows(X, T):
    """Labels (direction = the faster one; the other heads fixed) and rows
    repeated by how much the choice matters (1 + 4 x the relative gap, at most 9)."""
    lab = np.zeros((len(X), 3), dtype=np.int32)
    lab[:, 0] = (T[:, 1] < T[:, 0]).astype(np.int32)
    gap = np.abs(T[:, 0] - T[:, 1]) / np.maximum(T.min(1), 1e-6)
    rep = 1 + np.minimum(8, np.floor(4 * gap)).astype(np.int64)
    return np.repeat(X, rep, axis=0), np.repeat(lab, rep, axis=0)


def evaluate_batched(model, log):
    """Held-out seeds: per-level cost of each policy on the measured level times
    (every level top-down, every level bottom-up, the network's choice, the
    per-level optimum), and whole batched runs with the network attached against
    top-down only and the built-in rule, depths compared."""
    rows = []
    for name, hg, sym in (("rmat20_sym", rmat(20, 0.57, HELDOUT_SEEDS[0], True), True),
                          ("rmat22", rmat(22, 0.57, HELDOUT_SEEDS[1], False), False),
                          ("rmat21_a0.65_sym", rmat(21, 0.65, HELDOUT_SEEDS[1], True), True),
                          ("grid1024", HostGraph.grid(1024, 1024, seed=HELDOUT_SEEDS[0]), True)):
        g = GraphT(hg, symmetric=sym)
        srcs = hg.pick_sources(64, seed=HELDOUT_SEEDS[0])
        f, t = collect_batched_directions(g, srcs)
        pull = model.predict(f)[:, 0]
        per_level = {"top_down_ms": float(t[:, 0].sum()), "bottom_up_ms": float(t[:, 1].sum()),
                     "learned_ms": float(t[np.arange(len(t)), pull].sum()), "optimum_ms": float(t.min(1).sum())}

        def run(label):
            best, out = None, None
            for _ in range(5):
                out, st = bfs_batch(g, srcs)
                best = st["loop_ms"] if best is None else min(best, st["loop_ms"])
            return best, out
        set_batch_tuning(g, "bfs", bottom_up_div=-1)
        td_ms, d_td = run("top-down")
        set_batch_tuning(g, "bfs")
        rule_ms, d_rule = run("rule")
        set_batch_selector(g, "bfs", model)
        learned_ms, d_learned = run("learned")
        set_batch_selector(g, "bfs", None)
        if not (np.array_equal(d_td, d_rule) and np.array_equal(d_rule, d_learned)):
            raise AssertionError(f"{name}: depths differ between policies")
        row = {"graph": name, "V": hg.num_vertices, "E": hg.num_edges, "levels": int(len(t)),
               "per_level_cost": per_level,
               "runs_ms": {"top_down_only": td_ms, "builtin_rule": rule_ms, "learned": learned_ms}}
        rows.append(row)
        log(json.dumps(row))
        g.close()
    return rows


def main_batched_bfs(a, log):
    scales = [int(s) for s in a.scales.split(",")]
    skews = [float(s) for s in a.skews.split(",")]
    grids = [int(s) for s in a.grids.split(",") if s]
    t0 = time.time()
    X, T = collect_batched_bfs(scales, skews, grids, log)
    Xr, lab = batched_rows(X, T)
    log(f"collected {len(X)} levels ({len(Xr)} weighted rows) in {time.time() - t0:.1f}s")
    model = Selector(seed=27491095)
    loss = model.train(Xr, lab, epochs=a.epochs, lr=a.lr)
    pull = model.predict(X)[:, 0]
    acc = float((pull == (T[:, 1] < T[:, 0])).mean())
    regret = float(T[np.arange(len(T)), pull].sum() / T.min(1).sum())
    log(f"loss {loss:.4f} direction accuracy {acc:.3f} time / per-level optimum {regret:.3f}")
    out = a.out if a.out != str(DEFAULT_OUT) else str(BATCHED_BFS_OUT)
    model.save(out)
    evals = evaluate_batched(model, log)
    manifest = {
        "file": Path(out).name, "params": int(len(model.params)),
        "architecture": "12 -> 64 -> 64 -> 11 (bf16 MLP); the direction head picks each level's direction "
                        "of the batched BFS, on the device; the other heads are unused",
        "training": {"levels": int(len(X)), "weighted_rows": int(len(Xr)), "scales": scales, "skews": skews,
                     "grids": grids, "seeds": TRAIN_SEEDS, "sources_per_graph": "2 groups of 64 (R-MAT), 64 (grids)",
                     "epochs": a.epochs, "lr": a.lr, "final_loss": loss, "direction_accuracy": acc,
                     "time_over_per_level_optimum": regret},
        "heldout": evals,
    }
    Path(out).with_suffix(".json").write_text(json.dumps(manifest, indent=1))
    log(json.dumps(manifest))


# ------------------------------------------------- fused single-source BFS
def collect_fused_bfs(scales, skews, grids, log):
    X, T = [], []
    for name, scale, a, seed in training_graphs(scales, skews):
        for sym in (True, False):
            hg = rmat(scale, a, seed, sym)
            g = GraphT(hg, symmetric=sym)
            deg = np.diff(np.array(hg.offsets))
            srcs = [int(np.argmax(deg))] + [int(v) for v in hg.pick_sources(3, seed=seed + 5)]
            for src in srcs:
                f, t = collect_fused_directions(g, src)
                X.append(f)
                T.append(t)
            log(f"{name}{' sym' if sym else ''}: {sum(len(x) for x in X[-4:])} levels from 4 sources")
            g.close()
    for n in grids:
        hg = HostGraph.grid(n, n, seed=TRAIN_SEEDS[0])
        g = GraphT(hg, symmetric=True)
        for src in hg.pick_sources(2, seed=7):
            f, t = collect_fused_directions(g, int(src))
            X.append(f)
            T.append(t)
        log(f"grid{n}: {sum(len(x) for x in X[-2:])} levels from 2 sources")
        g.close()
    return np.concatenate(X), np.concatenate(T)


def fused_heldout_graphs():
    return (("rmat16_sym", HostGraph.rmat(16, 16, symmetrize=True), True),
            ("rmat20_sym", rmat(20, 0.57, HELDOUT_SEEDS[0], True), True),
            ("rmat22", rmat(22, 0.57, HELDOUT_SEEDS[1], False), False),
            ("rmat21_a0.65_sym", rmat(21, 0.65, HELDOUT_SEEDS[1], True), True),
            ("grid1024", HostGraph.grid(1024, 1024, seed=HELDOUT_SEEDS[0]), True))


def evaluate_fused(model, log, reps=5):
    """Held-out graphs, two sources each (the highest-degree vertex and a
    SourcePicker source): per-level cost of each policy on the measured level
    times, and whole runs (best of `reps` trial times) of bfs.cpp's two
    schedules -- PUSH TWCE fused, and the hybrid "power" schedule unfused as
    the reference runs it -- against the same hybrid rule fused and the
    network fused; depths compared."""
    rows = []
    plain, plain_fuse = default_schedule("bfs")
    power, _ = default_schedule("bfs", power=True)
    learned = LearnedGPUSchedule(model)
    for name, hg, sym in fused_heldout_graphs():
        g = GraphT(hg, symmetric=sym)
        deg = np.diff(np.array(hg.offsets))
        for src in (int(np.argmax(deg)), int(hg.pick_sources(1, seed=HELDOUT_SEEDS[0])[0])):
            f, t = collect_fused_directions(g, src)
            pull = model.predict(f)[:, 0]
            per_level = {"push_ms": float(t[:, 0].sum()), "pull_ms": float(t[:, 1].sum()),
                         "learned_ms": float(t[np.arange(len(t)), pull].sum()),
                         "optimum_ms": float(t.min(1).sum())}

            def run(sched, fuse):
                best, out = None, None
                for _ in range(reps):
                    out, _, st = bfs(g, src, sched, fuse)
                    best = st["device_ms"] if best is None else min(best, st["device_ms"])
                return best, out
            runs = {}
            outs = []
            for label, sched, fuse in (("plain_push_twce_fused", plain, plain_fuse),
                                       ("power_hybrid_unfused", power, False),
                                       ("power_hybrid_fused", power, True),
                                       ("learned_fused", learned, True)):
                runs[label], d = run(sched, fuse)
                outs.append(d)
            if not all(np.array_equal(outs[0], d) for d in outs[1:]):
                raise AssertionError(f"{name}: depths differ between schedules")
            row = {"graph": name, "V": hg.num_vertices, "E": hg.num_edges, "source": src, "levels": int(len(t)),
                   "per_level_cost": per_level, "runs_ms": runs}
            rows.append(row)
            log(json.dumps(row))
        g.close()
    return rows


def main_fused_bfs(a, log):
    scales = [int(s) for s in a.scales.split(",")]
    skews = [float(s) for s in a.skews.split(",")]
    grids = [int(s) for s in a.grids.split(",") if s]
    t0 = time.time()
    X, T = collect_fused_bfs(scales, skews, grids, log)
    Xr, lab = batched_rows(X, T)
    log(f"collected {len(X)} levels ({len(Xr)} weighted rows) in {time.time() - t0:.1f}s")
    model = Selector(seed=27491095)
    loss = model.train(Xr, lab, epochs=a.epochs, lr=a.lr)
    pull = model.predict(X)[:, 0]
    acc = float((pull == (T[:, 1] < T[:, 0])).mean())
    regret = float(T[np.arange(len(T)), pull].sum() / T.min(1).sum())
    log(f"loss {loss:.4f} direction accuracy {acc:.3f} time / per-level optimum {regret:.3f}")
    out = a.out if a.out != str(DEFAULT_OUT) else str(FUSED_BFS_OUT)
    model.save(out)
    evals = evaluate_fused(model, log)
    manifest = {
        "file": Path(out).name, "params": int(len(model.params)),
        "architecture": "12 -> 64 -> 64 -> 11 (bf16 MLP); the direction head picks each level's direction "
                        "(push or pull) inside the fused single-source BFS loop, on the device; the other "
                        "heads are unused",
        "training": {"levels": int(len(X)), "weighted_rows": int(len(Xr)), "scales": scales, "skews": skews,
                     "grids": grids, "seeds": TRAIN_SEEDS,
                     "sources_per_graph": "4 (R-MAT: the highest-degree vertex and 3 SourcePicker sources), "
                                          "2 (grids)",
                     "epochs": a.epochs, "lr": a.lr, "final_loss": loss, "direction_accuracy": acc,
                     "time_over_per_level_optimum": regret},
        "heldout": evals,
    }
    Path(out).with_suffix(".json").write_text(json.dumps(manifest, indent=1))
    log(json.dumps(manifest))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--fused-bfs", action="store_true",
                   help="train the per-level direction of the fused single-source BFS (selector_fused_bfs.bin)")
    p.add_argument("--batched-bfs", action="store_true",
                   help="train the per-level direction of the batched BFS (selector_batched_bfs.bin)")
    p.add_argument("--out", default=str(DEFAULT_OUT))
    p.add_argument("--scales", default="18,20,22,24")
    p.add_argument("--skews", default="0.45,0.57,0.75")
    p.add_argument("--grids", default="256,512")
    p.add_argument("--max-rows", type=int, default=120)
    p.add_argument("--epochs", type=int, default=3000)
    p.add_argument("--lr", type=float, default=3e-3)
    p.add_argument("--eval-scale", type=int, default=20)
    a = p.parse_args()
    log = lambda m: print(m, flush=True)
    if a.batched_bfs:
        main_batched_bfs(a, log)
        return
    if a.fused_bfs:
        main_fused_bfs(a, log)
        return
    scales = [int(s) for s in a.scales.split(",")]
    skews = [float(s) for s in a.skews.split(",")]
    grids = [int(s) for s in a.grids.split(",") if s]
    t0 = time.time()
    X, T = collect(scales, skews, grids, a.max_rows, log)
    lab = labels_from_times(T)
    log(f"collected {len(X)} rows in {time.time() - t0:.1f}s")
    model = Selector(seed=27491095)
    loss = model.train(X, lab, epochs=a.epochs, lr=a.lr)
    acc = (model.predict(X) == lab).mean(0)
    # time of the predicted candidate relative to the fastest, per row
    pred = model.predict(X)
    cand = pred[:, 0] * 18 + pred[:, 1] * 3 + pred[:, 2]
    regret = float(np.mean(T[np.arange(len(T)), cand] / T.min(1)))
    log(f"loss {loss:.4f} accuracy {acc} mean time / best {regret:.3f}")
    model.save(a.out)
    evals = evaluate(model, a.eval_scale, log)
    manifest = {
        "file": Path(a.out).name, "params": int(len(model.params)),
        "architecture": "12 -> 64 -> 64 -> 11 (bf16 MLP; heads: direction 2, load balancing 6, frontier 3)",
        "training": {"rows": int(len(X)), "scales": scales, "skews": skews, "grids": grids,
                     "seeds": TRAIN_SEEDS, "apps": ["bfs", "sssp (delta 32)", "cc"],
                     "epochs": a.epochs, "lr": a.lr, "final_loss": loss,
                     "accuracy": [float(v) for v in acc], "mean_time_over_best": regret},
        "heldout": evals,
    }
    Path(a.out).with_suffix(".json").write_text(json.dumps(manifest, indent=1))
    log(json.dumps(manifest))


if __name__ == "__main__":
    main()
