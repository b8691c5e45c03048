"""easy_graphit_gb300: GraphIt's GPU edge-traversal path (edgeset.apply /
vertexset.apply frontier operators and the BFS, SSSP, PageRank, CC and BC apps)
as hand-written sm_103a CUDA behind a C ABI (libgg.so, include/gg.h)."""
from .graphit import (  # noqa: F401
    BatchPlan,
    GraphT,
    HostGraph,
    HybridGPUSchedule,
    SimpleGPUSchedule,
    VertexSubset,
    app_schedule,
    bc,
    bfs,
    bfs_batch,
    bfs_multi,
    cc,
    default_schedule,
    multigraph_batch,
    pagerank,
    sssp,
    sssp_batch,
    sssp_multi,
)
