"""Replica execution across ranks (world size 2, gloo, CPU): per-rank source
draws are deterministic and differ between ranks, shards partition a unit list,
and the whole-job throughput is (sum of edges) / (max of times) -- the N>1 path
of bench.py without a GPU."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, outdir):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from easy_graphit_gb300 import HostGraph
    from easy_graphit_gb300.replicas import aggregate_teps, rank_sources, shard

    hg = HostGraph.rmat(10, 8)
    srcs = rank_sources(hg, 16, rank)
    again = rank_sources(hg, 16, rank)
    assert np.array_equal(srcs, again)
    # per-rank fake work: rank r "traverses" 1e6*(r+1) edges in 10*(r+1) ms
    gteps, ms = aggregate_teps(1e6 * (rank + 1), 10.0 * (rank + 1))
    np.save(os.path.join(outdir, f"r{rank}.npy"),
            np.concatenate([srcs.astype(np.float64), [gteps, ms], shard(list(range(10)), rank, world)]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r0 = np.load(tmp_path / "r0.npy")
    r1 = np.load(tmp_path / "r1.npy")
    s0, s1 = r0[:16], r1[:16]
    assert not np.array_equal(s0, s1)  # different sources per rank (weak scaling)
    # whole job: 3e6 edges / 20 ms (the slower rank) = 0.15 GTEPS on both ranks
    assert r0[16] == pytest.approx(0.15) and r1[16] == pytest.approx(0.15)
    assert r0[17] == 20.0 and r1[17] == 20.0
    assert list(r0[18:]) + list(r1[18:]) == list(range(10))
