import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "gapbs_ref.npz"
INT_MAX = 2**31 - 1


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a engine")


@pytest.fixture(scope="session", autouse=True)
def built_libs():
    """libgg.so and the oracle library, built in-tree if missing."""
    from easy_graphit_gb300 import build

    if not build.LIB.exists():
        build.build_lib()
    import oracle

    if not oracle.LIB.exists():
        oracle.build()
    yield


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


APP_GOLDEN = ROOT / "tests" / "golden" / "ref_apps.npz"
APP_GRAPHS = ["rmat10_k16_sym", "rmat11_k8_dir", "grid32"]


@pytest.fixture(scope="session")
def app_golden():
    """Outputs of the reference's own apps/*.cpp (tests/golden/make_app_golden.py)."""
    return np.load(APP_GOLDEN)


def app_graph(app_golden, name):
    """(offsets, dst, w) of a graph of ref_apps.npz: the R-MAT ones rebuilt by
    the oracle's generator (checked against the stored digest), the grid stored whole."""
    import hashlib

    import oracle

    if f"graph/{name}/offsets" in app_golden.files:
        return (app_golden[f"graph/{name}/offsets"], app_golden[f"graph/{name}/dst"],
                app_golden[f"graph/{name}/w"])
    off, dst, w = (np.asarray(a, dtype=np.int32) for a in oracle.rmat(
        int(app_golden[f"graph/{name}/scale"]), int(app_golden[f"graph/{name}/degree"]),
        symmetrize=bool(app_golden[f"graph/{name}/symmetrize"])))
    h = hashlib.sha256()
    for a in (off, dst, w):
        h.update(np.ascontiguousarray(a, dtype=np.int32).tobytes())
    assert h.hexdigest() == str(app_golden[f"graph/{name}/sha256"]), name
    return off, dst, w


def rel_l1(x, ref):
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(x - ref).sum() / max(np.abs(ref).sum(), 1e-300))


def shortest_paths_certified(off, dst, w, dist, src) -> bool:
    """dist is the exact shortest-path distance array from src iff dist[src] = 0,
    no edge can improve it (dist[v] <= dist[u] + w), and every other reached
    vertex has a tight in-edge (dist[v] = dist[u] + w): with positive weights the
    tight edges then lead back to src."""
    V = len(off) - 1
    u = np.repeat(np.arange(V, dtype=np.int64), np.diff(off))
    du = dist[u].astype(np.int64)
    dv = dist[dst].astype(np.int64)
    reached_u = du != INT_MAX
    if not np.all(~reached_u | (dv <= du + w)):
        return False
    tight = reached_u & (dv == du + w)
    has_tight = np.bincount(dst[tight], minlength=V) > 0
    reached = dist != INT_MAX
    reached[src] = False
    return bool(dist[src] == 0 and np.all(has_tight[reached]))
