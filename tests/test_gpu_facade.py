"""The C++ facade (include/graphit/schedule.h, operators.h): the reference's
operator chain and schedule API in C++ over the C ABI.  tests/cpp/facade_apps.cpp
writes the testcase() loops of apps/bfs.cpp, sssp.cpp and bc.cpp against it;
here it is compiled (no GPU needed) and run on the GPU, and its outputs are held
to the oracle: valid BFS trees, bit-exact SSSP distances, BC within 1e-6
relative L1 of FP64."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from tests.conftest import ROOT, rel_l1

PKG = ROOT / "easy_graphit_gb300"
EXE = PKG / "_build" / "facade_apps"
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def build_driver() -> Path:
    EXE.parent.mkdir(exist_ok=True)
    src = ROOT / "tests" / "cpp" / "facade_apps.cpp"
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", f"-I{ROOT / 'include'}", f"-I{CUDA / 'include'}",
           str(src), f"-L{PKG}", "-lgg", f"-L{CUDA / 'lib64'}", "-lcudart", f"-Wl,-rpath,{PKG}", "-o", str(EXE)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return EXE


def test_facade_compiles_against_the_headers():
    """The C++ headers and a driver written against them compile (-Wall -Werror)."""
    assert build_driver().exists()


@pytest.mark.gpu
def test_facade_apps_match_the_oracle(tmp_path):
    from easy_graphit_gb300 import HostGraph
    exe = build_driver()
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    rd = lambda n, t=np.int32: np.fromfile(tmp_path / f"{n}.bin", dtype=t)
    s_sym, s_dir, V_sym, V_dir = rd("meta")
    hs, hd = HostGraph.rmat(12, 16, symmetrize=True), HostGraph.rmat(12, 16)
    off, dst = np.array(hs.offsets), np.array(hs.dst)
    doff, ddst, dw = np.array(hd.offsets), np.array(hd.dst), np.array(hd.weights)
    assert (V_sym, V_dir) == (hs.num_vertices, hd.num_vertices)
    depth = oracle.bfs(off, dst, int(s_sym))
    for name in ("bfs_push_twce", "bfs_power", "bfs_power_t0"):
        assert oracle.bfs_check_parent(off, dst, int(s_sym), depth, rd(name)) == 0, name
    np.testing.assert_array_equal(rd("bfs_app_depth"), depth)
    ref = oracle.sssp_dijkstra(doff, ddst, dw, int(s_dir))
    for name in ("sssp_vertex_d8", "sssp_twce_boolmap_d32"):
        np.testing.assert_array_equal(rd(name), ref, err_msg=name)
    bc_ref = oracle.bc(off, dst, int(s_sym))
    for name in ("bc_push_twce", "bc_push_twce_unfused_dedup"):
        assert rel_l1(rd(name, np.float32), bc_ref) <= 1e-6, name
