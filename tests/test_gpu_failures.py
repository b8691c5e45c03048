"""Failure detection, exercised without faulting the GPU.

The reference reports a CUDA error by exit(-1) (runtime/infra_gpu/support.h:
4-10) and has no guard on its frontier queues (vertex_frontier.h:176-194
writes past 6*V).  Here every failure comes back as a status and leaves the
CUDA context usable:
  * a grid barrier that can never complete gives up at its time limit
    (GG_ERR_TIMEOUT);
  * a persistent loop past its wall-clock limit (GG_LOOP_TIMEOUT_MS) stops
    with GG_ERR_TIMEOUT;
  * a relax whose enqueues exceed the queue capacity drops them, flags the
    overflow and returns GG_ERR_OVERFLOW, never writing past the queue;
  * an allocation beyond the device pool's limit (GG_DEVICE_POOL_LIMIT_BYTES)
    returns GG_ERR_OOM.
After each, a BFS on the same process must still match the oracle.  Limits
read from the environment are set in a child process.
"""
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import oracle
from easy_graphit_gb300 import UDF, Filter, GraphT, HostGraph, VertexData, VertexSubset, bfs, edgeset_apply
from easy_graphit_gb300 import SimpleGPUSchedule as T
from easy_graphit_gb300 import _lib as L
from tests.conftest import ROOT

pytestmark = pytest.mark.gpu


def bfs_still_exact():
    hg = HostGraph.rmat(12, 16, symmetrize=True)
    g = GraphT(hg, symmetric=True)
    off, dst = np.array(hg.offsets), np.array(hg.dst)
    src = int(np.argmax(np.diff(off)))
    depth, _, _ = bfs(g, src)
    np.testing.assert_array_equal(depth, oracle.bfs(off, dst, src))
    g.close()


def child(code: str, env: dict) -> subprocess.CompletedProcess:
    e = dict(os.environ, **env)
    prog = "import sys\nsys.path.insert(0, %r)\n" % str(ROOT) + textwrap.dedent(code)
    return subprocess.run([sys.executable, "-c", prog], env=e, capture_output=True, text=True, timeout=600)


def test_grid_barrier_gives_up_at_its_limit():
    st = L.lib().gg_debug_barrier_timeout(50000)  # 50 ms; the barrier waits for one block too many
    assert st == L.GG_ERR_TIMEOUT, L.last_error()
    assert "timed out" in L.last_error()
    bfs_still_exact()


def test_queue_overflow_is_reported_not_written_past():
    """K_{64,64} behind one source: a BC-forward apply with duplicates allowed
    enqueues every A->B edge (64*64 = 4096 entries) into a queue of 6*V = 774;
    the surplus is dropped and the call returns GG_ERR_OVERFLOW."""
    import torch
    k = 64
    V = 1 + 2 * k
    u = [0] * k + [1 + i for i in range(k) for _ in range(k)]
    v = [1 + i for i in range(k)] + [1 + k + j for _ in range(k) for j in range(k)]
    hg = HostGraph.from_edges(V, np.array(u, np.int32), np.array(v, np.int32))
    g = GraphT(hg)
    sigma = torch.zeros(V, dtype=torch.float64, device="cuda")
    visited = torch.zeros(V, dtype=torch.uint8, device="cuda")
    sigma[:1 + k] = 1.0
    visited[:1 + k] = 1
    vd = VertexData(num_paths=sigma, visited=visited)
    f = VertexSubset(g)
    for a in range(1, 1 + k):
        f.addVertex(a)
    with pytest.raises(L.GGError) as e:
        edgeset_apply(T().configLoadBalancing(T.load_balancing_type.TWCE)).from_(f).to(
            Filter.UNVISITED).apply_modified(g, f, vd, UDF.BC_FORWARD, allow_dupes=True)
    assert e.value.status == L.GG_ERR_OVERFLOW
    with pytest.raises(L.GGError) as e2:  # the overflowed frontier is refused, not read
        f.size()
    assert e2.value.status == L.GG_ERR_OVERFLOW
    assert float(sigma[1 + k:].sum()) == k * k  # every edge still applied its UDF
    g.close()
    bfs_still_exact()


def test_persistent_loop_stops_at_its_time_limit():
    r = child("""
        import numpy as np
        import oracle
        from easy_graphit_gb300 import GraphT, HostGraph, SimpleGPUSchedule as T, bfs, sssp
        from easy_graphit_gb300 import _lib as L
        hg = HostGraph.grid(1024, 1024)
        g = GraphT(hg, symmetric=True)
        twce = T().configLoadBalancing(T.load_balancing_type.TWCE)
        try:
            sssp(g, 0, 1, twce, True)   # ~10^5 buckets: far longer than 1 ms
            print("NO_TIMEOUT")
        except L.GGError as e:
            print("STATUS", e.status)
        small = HostGraph.rmat(10, 8, symmetrize=True)
        g2 = GraphT(small, symmetric=True)
        off, dst = np.array(small.offsets), np.array(small.dst)
        d, _, _ = bfs(g2, 0, twce, False)   # host-driven loop: no persistent-loop limit
        print("BFS_OK", bool(np.array_equal(d, oracle.bfs(off, dst, 0))))
    """, {"GG_LOOP_TIMEOUT_MS": "1"})
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"STATUS {L.GG_ERR_TIMEOUT}" in r.stdout, r.stdout
    assert "BFS_OK True" in r.stdout, r.stdout


def test_device_pool_limit_gives_oom():
    r = child("""
        import numpy as np
        from easy_graphit_gb300 import GraphT, HostGraph
        from easy_graphit_gb300 import _lib as L
        hg = HostGraph.rmat(16, 16)   # ~4 MB of CSR on the device
        try:
            GraphT(hg)
            print("NO_OOM")
        except L.GGError as e:
            print("STATUS", e.status, L.last_error())
        tiny = HostGraph.rmat(6, 4)   # fits under the limit: the context is still usable
        g = GraphT(tiny)
        print("TINY_OK", g.num_vertices)
    """, {"GG_DEVICE_POOL_LIMIT_BYTES": str(1 << 20)})
    assert r.returncode == 0, r.stdout + r.stderr
    assert f"STATUS {L.GG_ERR_OOM}" in r.stdout, r.stdout
    assert "TINY_OK" in r.stdout, r.stdout
