"""gg_app, the apps' trial-loop driver: argument handling on the CPU, results
through the binary on the GPU."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from tests.conftest import rel_l1

EXE = Path(__file__).resolve().parents[1] / "easy_graphit_gb300" / "gg_app"


def run(*args, **kw):
    return subprocess.run([str(EXE), *map(str, args)], capture_output=True, text=True, timeout=300, **kw)


def test_usage_and_bad_arguments_exit_2():
    assert run().returncode == 2
    assert run("bfs").returncode == 2
    assert run("apsp", "rmat:10").returncode == 2
    r = run("bfs", "rmat:x")
    assert r.returncode == 2 and "bad generator" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("app", ["bfs", "sssp", "pr", "cc", "bc"])
def test_trials_and_results_match_the_oracle(app, tmp_path):
    from easy_graphit_gb300 import HostGraph
    sym = app in ("bfs", "cc", "bc")
    spec = "rmat:13:16" + (":sym" if sym else "")
    hg = HostGraph.rmat(13, 16, symmetrize=sym)
    off, dst, w = np.array(hg.offsets), np.array(hg.dst), np.array(hg.weights)
    src = int(hg.pick_sources(1)[0])
    out = tmp_path / "out.bin"
    args = [app, spec] + ([src] if app in ("bfs", "sssp", "bc") else []) + (["8"] if app == "sssp" else [])
    r = run(*args, "--out", out, "--max-cta", 80, "--cta-size", 256)
    assert r.returncode == 0, r.stderr
    times = [float(x) for x in r.stdout.split()]
    assert len(times) == {"bfs": 4, "sssp": 5, "pr": 10, "cc": 10, "bc": 3}[app] and min(times) > 0
    if app == "bfs":
        np.testing.assert_array_equal(np.fromfile(out, dtype=np.int32), oracle.bfs(off, dst, src))
    elif app == "sssp":
        np.testing.assert_array_equal(np.fromfile(out, dtype=np.int32), oracle.sssp_dijkstra(off, dst, w, src))
    elif app == "cc":
        np.testing.assert_array_equal(np.fromfile(out, dtype=np.int32), oracle.cc(off, dst))
    elif app == "pr":
        assert rel_l1(np.fromfile(out, dtype=np.float32), oracle.pagerank(off, dst, 20, float(np.float32(0.85)))) <= 1e-6
    else:
        assert rel_l1(np.fromfile(out, dtype=np.float32), oracle.bc(off, dst, src)) <= 1e-6


@pytest.mark.gpu
def test_power_schedules_run():
    r = run("bfs", "rmat:12:16:sym", "--power", "--trials", 2)
    assert r.returncode == 0, r.stderr
    assert len(r.stdout.split()) == 2
