"""easy_graphit_gb300: GraphIt's GPU edge-traversal path (edgeset.apply /
vertexset.apply frontier operators and the BFS, SSSP, PageRank, CC and BC apps)
as hand-written sm_103a CUDA behind a C ABI (libgg.so, include/gg.h)."""
from .graphit import (  # noqa: F401
    GraphT,
    HostGraph,
    HybridGPUSchedule,
    SimpleGPUSchedule,
    VertexSubset,
    app_schedule,
    bc,
    bfs,
    bfs_batch,
    cc,
    default_schedule,
    pagerank,
    sssp,
    sssp_batch,
)
